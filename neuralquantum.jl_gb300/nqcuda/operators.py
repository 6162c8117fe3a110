"""k-local operators of the reference API and their flattening into the
``nq_op_table`` of include/nqcuda.h.

Mirrors src/Operators/: ``sigmax/sigmay/sigmaz/sigmam/sigmap(hilb, i)``
(SimpleOperators.jl:11-96, sites are 1-based like the reference),
``LocalOperator(hilb)``, operator sums with same-site merging
(KLocalOperatorSum.jl:89-101, KLocalOperator.jl:213-249), products
(KLocalOperator.jl:271-314), adjoints, scalar multiples and
``liouvillian(H, Lops)`` (KLocalLiouvillian.jl:9-37).

Row tables follow KLocalOperator.jl:54-112: every row stores its diagonal
entry first (even when zero), then the off-diagonal entries with
|v| >= 1e-5 in column order; each entry records the changed sites and their
new values.  Merging two operators on the same sites adds matrix elements of
identical changes and appends the rest (OpConnection.jl:114-124).
"""
import ctypes

import numpy as np

from . import _lib
from .hilbert import SuperOpSpace, physical

_THRESH = 1e-5


def _digits(idx, k):
    return [(idx >> d) & 1 for d in range(k)]


class KLocalOperator:
    def __init__(self, hilb, sites0, mat):
        self.hilb = hilb
        self.sites = list(sites0)
        self.mat = np.asarray(mat, dtype=np.complex128).copy()
        k = len(self.sites)
        if self.mat.shape != (1 << k, 1 << k):
            raise ValueError("matrix size does not match the number of sites")
        self.rows = []
        for r in range(1 << k):
            row = [[complex(self.mat[r, r]), ()]]
            dr = _digits(r, k)
            for c in range(1 << k):
                if c == r or abs(self.mat[r, c]) < _THRESH:
                    continue
                dc = _digits(c, k)
                ch = tuple((self.sites[d], hilb.value(dc[d])) for d in range(k) if dr[d] != dc[d])
                row.append([complex(self.mat[r, c]), ch])
            self.rows.append(row)

    # --- algebra -----------------------------------------------------------
    def _rebuilt(self, mat):
        return KLocalOperator(self.hilb, self.sites, mat)

    def copy(self):
        o = KLocalOperator.__new__(KLocalOperator)
        o.hilb, o.sites, o.mat = self.hilb, list(self.sites), self.mat.copy()
        o.rows = [[[m, ch] for m, ch in row] for row in self.rows]
        return o

    def __neg__(self):
        return self._rebuilt(-self.mat)

    def __rmul__(self, a):
        if np.isscalar(a):
            return self._rebuilt(a * self.mat)
        return NotImplemented

    def __mul__(self, other):
        if np.isscalar(other):
            return self._rebuilt(other * self.mat)
        if isinstance(other, KLocalOperator):
            return _prod(self, other)
        if isinstance(other, KLocalOperatorSum):
            return KLocalOperatorSum(self.hilb, [_prod(self, o) for o in other.ops])
        return NotImplemented

    def __truediv__(self, a):
        return self._rebuilt(self.mat / a)

    def conj(self):
        o = self.copy()
        o.mat = np.conj(o.mat)
        for row in o.rows:
            for e in row:
                e[0] = complex(np.conj(e[0]))
        return o

    def transpose(self):
        return self._rebuilt(self.mat.T.copy())

    def adjoint(self):
        return self.transpose().conj()

    @property
    def H(self):
        return self.adjoint()

    def _merge_(self, other):
        if self.sites != other.sites:
            raise ValueError("can only merge operators on identical sites")
        self.mat = self.mat + other.mat
        for row_l, row_r in zip(self.rows, other.rows):
            for mel, ch in row_r:
                key = sorted(ch)
                for e in row_l:
                    if sorted(e[1]) == key:
                        e[0] = e[0] + mel
                        break
                else:
                    row_l.append([mel, ch])
        return self

    def __add__(self, other):
        return KLocalOperatorSum(self.hilb, [self]) + other

    def __radd__(self, other):
        if isinstance(other, (int, float)) and other == 0:
            return KLocalOperatorSum(self.hilb, [self])
        return NotImplemented

    def __sub__(self, other):
        return KLocalOperatorSum(self.hilb, [self]) - other


def _prod(opl, opr):
    if opl.sites == opr.sites:
        return opl._rebuilt(opl.mat @ opr.mat)
    if len(opl.sites) == 1 and len(opr.sites) == 1:
        if opl.sites[0] > opr.sites[0]:
            opl, opr = opr, opl
        return KLocalOperator(opl.hilb, [opl.sites[0], opr.sites[0]], np.kron(opr.mat, opl.mat))
    raise NotImplementedError("products beyond single-site factors are not supported")


class KLocalOperatorSum:
    def __init__(self, hilb, ops=()):
        self.hilb = hilb
        self.ops = []
        for o in ops:
            self._add_(o)

    def copy(self):
        s = KLocalOperatorSum(self.hilb)
        s.ops = [o.copy() for o in self.ops]
        return s

    def _add_(self, op):
        for o in self.ops:
            if o.sites == op.sites:
                o._merge_(op)
                return self
        self.ops.append(op.copy())
        return self

    def __add__(self, other):
        s = self.copy()
        if isinstance(other, KLocalOperatorSum):
            for o in other.ops:
                s._add_(o)
        elif isinstance(other, KLocalOperator):
            s._add_(other)
        else:
            return NotImplemented
        return s

    def __sub__(self, other):
        if isinstance(other, KLocalOperatorSum):
            return self + KLocalOperatorSum(self.hilb, [-o for o in other.ops])
        return self + (-other)

    def __rmul__(self, a):
        if np.isscalar(a):
            return KLocalOperatorSum(self.hilb, [a * o for o in self.ops])
        return NotImplemented

    def __mul__(self, other):
        if np.isscalar(other):
            return other * self
        if isinstance(other, KLocalOperator):
            return KLocalOperatorSum(self.hilb, [_prod(o, other) for o in self.ops])
        return NotImplemented

    def __truediv__(self, a):
        return (1.0 / a) * self

    def adjoint(self):
        s = KLocalOperatorSum(self.hilb)
        s.ops = [o.adjoint() for o in self.ops]
        return s

    @property
    def H(self):
        return self.adjoint()


def LocalOperator(hilb):
    """Empty operator sum (``LocalOperator(hilb)``)."""
    return KLocalOperatorSum(hilb)


def _site0(hilb, i):
    n = physical(hilb).n_sites
    if not 1 <= i <= n:
        raise ValueError(f"site {i} outside 1..{n}")
    return i - 1


def sigmax(hilb, i):
    return KLocalOperator(hilb, [_site0(hilb, i)], [[0, 1], [1, 0]])


def sigmay(hilb, i):
    return KLocalOperator(hilb, [_site0(hilb, i)], [[0, -1j], [1j, 0]])


def sigmaz(hilb, i):
    # diag(2m for m = S:-1:-S): local index 0 carries +1 (SimpleOperators.jl:55-65)
    return KLocalOperator(hilb, [_site0(hilb, i)], [[1, 0], [0, -1]])


def sigmam(hilb, i):
    return KLocalOperator(hilb, [_site0(hilb, i)], [[0, 0], [1, 0]])


def sigmap(hilb, i):
    return KLocalOperator(hilb, [_site0(hilb, i)], [[0, 1], [0, 0]])


class KLocalLiouvillian:
    """``KLocalLiouvillian``: -i HnH ⊗ 1 (row), +i 1 ⊗ HnH† (column) and
    Σ L ⊗ conj(L); HnH = H - i/2 Σ L†L."""

    def __init__(self, hilb, HnH_l, HnH_r, LLdag):
        self.hilb = SuperOpSpace(hilb)
        self.HnH_l, self.HnH_r, self.LLdag = HnH_l, HnH_r, LLdag


def liouvillian(H, Lops):
    HnH = H.copy()
    for L in Lops:
        HnH = HnH + (-0.5j) * (L.adjoint() * L)
    HnH_l = [(-1.0j) * o for o in HnH.ops]
    HnH_r = [(1.0j) * o for o in HnH.adjoint().ops]
    LLdag = [(L, L.conj()) for L in Lops]
    return KLocalLiouvillian(H.hilb, HnH_l, HnH_r, LLdag)


# ---------------------------------------------------------------------------
# flattening
# ---------------------------------------------------------------------------

class OpTable:
    """Flattened operator; keeps the numpy arrays alive for the ctypes struct."""

    def __init__(self, ops):
        # ops: list of (digit_sites, rows) with rows[r] = [(mel, ((site, val), ...)), ...]
        n_ops = len(ops)
        self.op_n_sites = np.zeros(n_ops, np.int32)
        self.op_sites = np.zeros(8 * n_ops, np.int32)
        self.op_row_offset = np.zeros(n_ops, np.int32)
        row_off, mels, nch, csite, cval = [0], [], [], [], []
        r0 = 0
        for o, (sites, rows) in enumerate(ops):
            if len(sites) > 8:
                raise ValueError("at most 8 digit sites per operator")
            self.op_n_sites[o] = len(sites)
            self.op_sites[8 * o:8 * o + len(sites)] = sites
            self.op_row_offset[o] = r0
            r0 += len(rows)
            for row in rows:
                for mel, ch in row:
                    mels += [mel.real, mel.imag]
                    nch.append(len(ch))
                    s8 = [0] * 8
                    v8 = [0] * 8
                    for q, (s, v) in enumerate(ch):
                        s8[q], v8[q] = s, v
                    csite += s8
                    cval += v8
                row_off.append(len(nch))
        self.n_ops, self.n_rows, self.n_conns = n_ops, r0, len(nch)
        self.row_conn_offset = np.array(row_off, np.int32)
        self.conn_mel = np.array(mels if mels else [0.0, 0.0], np.float64)
        self.conn_n_changes = np.array(nch if nch else [0], np.int32)
        self.conn_change_site = np.array(csite if csite else [0] * 8, np.int32)
        self.conn_change_value = np.array(cval if cval else [0] * 8, np.int8)

    def struct(self):
        p = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
        return _lib.NqOpTable(self.n_ops, self.n_rows, self.n_conns,
                              p(self.op_n_sites, ctypes.c_int32), p(self.op_sites, ctypes.c_int32),
                              p(self.op_row_offset, ctypes.c_int32),
                              p(self.row_conn_offset, ctypes.c_int32),
                              p(self.conn_mel, ctypes.c_double),
                              p(self.conn_n_changes, ctypes.c_int32),
                              p(self.conn_change_site, ctypes.c_int32),
                              p(self.conn_change_value, ctypes.c_int8))

    def connections(self, config):
        """(mel, changes) visited for one configuration (a host-side mirror of
        the device walk, used by tests)."""
        out = []
        for o in range(self.n_ops):
            k = self.op_n_sites[o]
            r = 0
            for d in range(k):
                s = self.op_sites[8 * o + d]
                r |= (1 if config[s] > 0 else 0) << d
            row = self.op_row_offset[o] + r
            for c in range(self.row_conn_offset[row], self.row_conn_offset[row + 1]):
                mel = complex(self.conn_mel[2 * c], self.conn_mel[2 * c + 1])
                ch = [(int(self.conn_change_site[8 * c + q]), int(self.conn_change_value[8 * c + q]))
                      for q in range(self.conn_n_changes[c])]
                out.append((mel, ch))
        return out


def op_table(op):
    """Flatten a KLocalOperatorSum / KLocalOperator / KLocalLiouvillian in the
    order ``accumulate_connections!`` visits it."""
    if isinstance(op, KLocalOperator):
        op = KLocalOperatorSum(op.hilb, [op])
    if isinstance(op, KLocalOperatorSum):
        return OpTable([(o.sites, [[(m, ch) for m, ch in row] for row in o.rows]) for o in op.ops])
    if isinstance(op, KLocalLiouvillian):
        N = physical(op.hilb).n_sites
        ops = []
        for o in op.HnH_l:
            ops.append((o.sites, [[(m, ch) for m, ch in row] for row in o.rows]))
        for o in op.HnH_r:
            shift = lambda ch: tuple((s + N, v) for s, v in ch)
            ops.append(([s + N for s in o.sites], [[(m, shift(ch)) for m, ch in row] for row in o.rows]))
        for L, R in op.LLdag:
            k = len(L.sites)
            rows = [None] * (1 << (2 * k))    # row index = r_row + 2^k r_col
            for rc in range(1 << k):
                for rr in range(1 << k):
                    row = []
                    for ml, chl in L.rows[rr]:
                        for mr, chr_ in R.rows[rc]:
                            row.append((ml * mr, tuple(chl) + tuple((s + N, v) for s, v in chr_)))
                    rows[rr + (rc << k)] = row
            ops.append((list(L.sites) + [s + N for s in R.sites], rows))
        return OpTable(ops)
    raise TypeError(f"cannot flatten {type(op)}")
