"""k-local operators and the Liouvillian (test infrastructure, see
``oracle/__init__``).

Restates:

* row tables of a local operator: src/Operators/Operators/KLocalOperator.jl:54-112
  (diagonal entry always stored, even when zero, :76-80; off-diagonal entries
  kept when |v| >= 1e-5, :86),
* ``accumulate_connections!`` :183-199 and sums KLocalOperatorSum.jl:65-106
  (operators on an identical site list are merged, ``add!`` of
  OpConnection.jl:120-124 adds matrix elements of identical changes),
* products of single-site operators KLocalOperator.jl:271-314
  (``kron(opr.mat, opl.mat)`` on the sorted site pair),
* Pauli / ladder matrices SimpleOperators.jl:11-96,
* the Liouvillian KLocalLiouvillian.jl:9-52 with tensors
  KLocalOperatorTensor.jl:129-157.

Sites are 0-based here (the reference is 1-based).
"""
import numpy as np

from .hilbert import Hilbert

THRESH = 1e-5   # `abs(val) < 10e-6 && continue`, KLocalOperator.jl:86


def _digits(idx, d, k):
    out = []
    for _ in range(k):
        idx, r = divmod(idx, d)
        out.append(r)
    return out


class LocalOp:
    """One k-local operator with its per-row connection table."""

    def __init__(self, hilb: Hilbert, sites, mat):
        self.hilb = hilb
        self.sites = list(sites)
        self.mat = np.array(mat, dtype=np.complex128)
        d = hilb.d
        k = len(self.sites)
        assert self.mat.shape == (d ** k, d ** k)
        # conns[r] = list of [mel, [(site, new_value), ...]]
        self.conns = []
        for r in range(d ** k):
            row = [[self.mat[r, r], []]]
            dr = _digits(r, d, k)
            for c in range(d ** k):
                if c == r or abs(self.mat[r, c]) < THRESH:
                    continue
                dc = _digits(c, d, k)
                ch = [(self.sites[i], float(hilb.value(dc[i])))
                      for i in range(k) if dr[i] != dc[i]]
                row.append([self.mat[r, c], ch])
            self.conns.append(row)

    def copy(self):
        o = LocalOp.__new__(LocalOp)
        o.hilb, o.sites, o.mat = self.hilb, list(self.sites), self.mat.copy()
        o.conns = [[[m, list(ch)] for m, ch in row] for row in self.conns]
        return o

    def with_matrix(self, mat):
        return LocalOp(self.hilb, self.sites, mat)

    def conj(self):
        o = self.copy()
        o.mat = np.conj(o.mat)
        for row in o.conns:
            for e in row:
                e[0] = np.conj(e[0])
        return o

    def transpose(self):
        return self.with_matrix(self.mat.T.copy())

    def adjoint(self):
        return self.transpose().conj()

    def scale(self, a):
        return self.with_matrix(a * self.mat)

    def add_samesite_(self, other):
        """``_add_samesite!`` (KLocalOperator.jl:213-249): matrices add and
        the connection rows are merged with ``add!``."""
        assert self.sites == other.sites
        self.mat = self.mat + other.mat
        for row_l, row_r in zip(self.conns, other.conns):
            for mel, ch in row_r:
                key = sorted(ch)
                for e in row_l:
                    if sorted(e[1]) == key:
                        e[0] = e[0] + mel
                        break
                else:
                    row_l.append([mel, list(ch)])
        return self


def _local(hilb, i, mat):
    return LocalOp(hilb, [i], mat)


def sigmax(hilb, i):
    d = hilb.d; S = (d - 1) / 2
    D = [np.sqrt((S + 1) * 2 * a - a * (a + 1)) for a in range(1, d)]
    return _local(hilb, i, np.diag(D, 1) + np.diag(D, -1))


def sigmay(hilb, i):
    d = hilb.d; S = (d - 1) / 2
    D = np.array([1j * np.sqrt((S + 1) * 2 * a - a * (a + 1)) for a in range(1, d)])
    return _local(hilb, i, np.diag(D, -1) + np.diag(-D, 1))


def sigmaz(hilb, i):
    d = hilb.d; S = (d - 1) / 2
    D = [2 * (S - k) for k in range(d)]          # m = S:-1:-S
    return _local(hilb, i, np.diag(D).astype(np.complex128))


def sigmam(hilb, i):
    d = hilb.d; S = (d - 1) / 2
    S2 = (S + 1) * S
    D = [np.sqrt(S2 - m * (m - 1)) for m in [S - k for k in range(d - 1)]]
    return _local(hilb, i, np.diag(D, -1).astype(np.complex128))


def sigmap(hilb, i):
    d = hilb.d; S = (d - 1) / 2
    S2 = (S + 1) * S
    D = [np.sqrt(S2 - m * (m + 1)) for m in [S - 1 - k for k in range(d - 1)]]
    return _local(hilb, i, np.diag(D, 1).astype(np.complex128))


def prod(opl: LocalOp, opr: LocalOp) -> LocalOp:
    """``opl * opr`` for the cases used on the hot path
    (KLocalOperator.jl:271-314)."""
    if opl.sites == opr.sites:
        return opl.with_matrix(opl.mat @ opr.mat)
    assert len(opl.sites) == 1 and len(opr.sites) == 1
    if opl.sites[0] > opr.sites[0]:
        opl, opr = opr, opl
    return LocalOp(opl.hilb, [opl.sites[0], opr.sites[0]], np.kron(opr.mat, opl.mat))


class OpSum:
    """KLocalOperatorSum: list of LocalOp on distinct site lists."""

    def __init__(self, hilb, ops=()):
        self.hilb = hilb
        self.ops = []
        for o in ops:
            self.add_(o)

    def copy(self):
        s = OpSum(self.hilb)
        s.ops = [o.copy() for o in self.ops]
        return s

    def add_(self, op: LocalOp):
        for o in self.ops:
            if o.sites == op.sites:
                o.add_samesite_(op)
                return self
        self.ops.append(op.copy())
        return self

    def __add__(self, op):
        s = self.copy()
        if isinstance(op, OpSum):
            for o in op.ops:
                s.add_(o)
        else:
            s.add_(op)
        return s

    def __sub__(self, op):
        if isinstance(op, OpSum):
            return self + OpSum(self.hilb, [o.scale(-1) for o in op.ops])
        return self + op.scale(-1)

    def adjoint(self):
        s = OpSum(self.hilb)
        s.ops = [o.adjoint() for o in self.ops]
        return s

    def scale(self, a):
        return OpSum(self.hilb, [o.scale(a) for o in self.ops])


def connections_ket(H: OpSum, sigma):
    """Ordered (mel, changes) list visited by ``accumulate_connections!`` on a
    ket configuration ``sigma`` (1-D array)."""
    out = []
    for o in H.ops:
        r = int(o.hilb.local_index(sigma, o.sites))
        for mel, ch in o.conns[r]:
            out.append((mel, ch))
    return out


class Liouvillian:
    """KLocalLiouvillian: three lists of (left, right) tensor operators.
    ``None`` stands for KLocalIdentity."""

    def __init__(self, hilb, HnH_l, HnH_r, LLdag):
        self.hilb = hilb
        self.HnH_l = HnH_l
        self.HnH_r = HnH_r
        self.LLdag = LLdag


def liouvillian(H: OpSum, Lops):
    """``liouvillian(H, Lops)``, KLocalLiouvillian.jl:26-33 and :9-20."""
    HnH = H.copy()
    for L in Lops:
        HnH = HnH + prod(L.adjoint(), L).scale(-0.5j)
    HnH_l = [(o.scale(-1.0j), None) for o in HnH.ops]
    HnH_r = [(None, o.scale(1.0j)) for o in HnH.adjoint().ops]
    LLdag = [(L, L.conj()) for L in Lops]
    return Liouvillian(H.hilb, HnH_l, HnH_r, LLdag)


def connections_doubled(lv: Liouvillian, sigma, eta):
    """Ordered (mel, row_changes, col_changes) visited by
    ``accumulate_connections!(acc, ::KLocalLiouvillian, (σ, η))``."""
    out = []
    h = lv.hilb
    for opl, _ in lv.HnH_l:
        r = int(h.local_index(sigma, opl.sites))
        for mel, ch in opl.conns[r]:
            out.append((mel, ch, []))
    for _, opr in lv.HnH_r:
        r = int(h.local_index(eta, opr.sites))
        for mel, ch in opr.conns[r]:
            out.append((mel, [], ch))
    for opl, opr in lv.LLdag:
        rr = int(h.local_index(sigma, opl.sites))
        rc = int(h.local_index(eta, opr.sites))
        for ml, chl in opl.conns[rr]:
            for mr, chr_ in opr.conns[rc]:
                out.append((ml * mr, chl, chr_))
    return out


def apply_changes(sigma, changes):
    s = np.array(sigma, dtype=np.float64, copy=True)
    for site, val in changes:
        s[site] = val
    return s


# ---------------------------------------------------------------------------
# dense matrices
# ---------------------------------------------------------------------------

def to_matrix(H: OpSum):
    """``to_matrix`` (OpConversion.jl:6-24) from the connection tables."""
    h = H.hilb
    mat = np.zeros((h.dim, h.dim), dtype=np.complex128)
    for i, s in enumerate(h.all_states()):
        for mel, ch in connections_ket(H, s):
            j = h.index_of_state(apply_changes(s, ch))
            mat[i, j] += mel
    return mat


def liouvillian_to_matrix(lv: Liouvillian):
    """Dense super-operator on vec(ρ) (column-major, index = col*dim + row)."""
    h = lv.hilb
    D = h.dim
    mat = np.zeros((D * D, D * D), dtype=np.complex128)
    states = h.all_states()
    for ic, eta in enumerate(states):
        for ir, sig in enumerate(states):
            i = ic * D + ir
            for mel, chl, chr_ in connections_doubled(lv, sig, eta):
                jr = h.index_of_state(apply_changes(sig, chl))
                jc = h.index_of_state(apply_changes(eta, chr_))
                mat[i, jc * D + jr] += mel
    return mat


def embed(hilb: Hilbert, i, local):
    """Independent dense embedding of a single-site matrix on site i
    (first site least significant, like QuantumOptics' ``embed``)."""
    out = np.array([[1.0 + 0j]])
    for s in range(hilb.n_sites):
        m = local if s == i else np.eye(hilb.d)
        out = np.kron(m, out)
    return out


def dense_liouvillian(Hd, Ld_list):
    """Independent dense Liouvillian on column-major vec(ρ):
    L = -i(H⊗... ) per QuantumOptics conventions: spre(A)=I⊗A, spost(B)=Bᵀ⊗I."""
    D = Hd.shape[0]
    I = np.eye(D)
    HnH = Hd.astype(np.complex128).copy()
    for L in Ld_list:
        HnH = HnH - 0.5j * L.conj().T @ L
    out = -1j * np.kron(I, HnH) + 1j * np.kron(HnH.conj(), I)
    for L in Ld_list:
        out = out + np.kron(L.conj(), L)
    return out
