"""Exact-enumeration helpers for small systems (test infrastructure, see
``oracle/__init__``).

* dense TFIM Hamiltonians built from independent Kronecker products (the
  conventions pinned by test/Operators/ising.jl:5-42),
* a matrix-free Lanczos ground state for the 1D TFIM of examples/ising1d.jl
  (known answer -1.274549484318 * 20, examples/ising1d.jl:46-47),
* exact |ψ|^2 / |ρ|^2 / ρ(σ,σ) distributions for chi-square sampler tests
  (test/Samplers/test_samplers.jl:7-31).
"""
import numpy as np
import scipy.sparse.linalg as spla

from . import operators as ops
from .hilbert import Hilbert, SPIN


def tfim_1d(hilb, h, J, periodic=True, sign_x=-1.0):
    """``H = sign_x * h Σσx + J Σσzσz`` built with the reference operator API
    (examples/ising1d.jl:15-18)."""
    N = hilb.n_sites
    H = ops.OpSum(hilb)
    for i in range(N):
        H = H + ops.sigmax(hilb, i).scale(sign_x * h)
        if periodic or i + 1 < N:
            H = H + ops.prod(ops.sigmaz(hilb, i), ops.sigmaz(hilb, (i + 1) % N)).scale(J)
    return H


def tfim_2d(hilb, Lx, Ly, h, J):
    """examples/ising2d.jl:16-26 (coord(i,j) = i + (j-1)*dims[2])."""
    H = ops.OpSum(hilb)
    coord = lambda i, j: i + j * Ly
    for i in range(Lx):
        for j in range(Ly):
            p = coord(i, j)
            H = H - ops.sigmax(hilb, p).scale(h)
            H = H + ops.prod(ops.sigmaz(hilb, p), ops.sigmaz(hilb, coord((i + 1) % Lx, j))).scale(J)
            H = H + ops.prod(ops.sigmaz(hilb, p), ops.sigmaz(hilb, coord(i, (j + 1) % Ly))).scale(J)
    return H


def dissipative_ising(hilb, g, V, gamma=1.0, periodic=False):
    """Configs of the dissipative TFIM: H = g/2 Σσx + V/4 Σσzσz, L_i = √γ σ⁻_i
    (examples/dissipative_ising1d.jl:17-31, open chain unless periodic)."""
    N = hilb.n_sites
    H = ops.OpSum(hilb)
    for i in range(N):
        H = H + ops.sigmax(hilb, i).scale(g / 2.0)
    for i in range(N):
        if periodic or i + 1 < N:
            H = H + ops.prod(ops.sigmaz(hilb, i), ops.sigmaz(hilb, (i + 1) % N)).scale(V / 4.0)
    Ls = [ops.sigmam(hilb, i).scale(np.sqrt(gamma)) for i in range(N)]
    return H, Ls


def tfim_ground_energy_1d(N, h, J):
    """Matrix-free Lanczos for H = -hΣσx + JΣσzσz, periodic, spin basis bit
    s=1 <-> value +1."""
    dim = 1 << N
    idx = np.arange(dim, dtype=np.int64)
    bits = ((idx[:, None] >> np.arange(N)) & 1).astype(np.float64) * 2 - 1
    diag = J * np.sum(bits * np.roll(bits, -1, axis=1), axis=1)

    def mv(v):
        v = np.asarray(v).ravel()
        out = diag * v
        for i in range(N):
            out -= h * v[idx ^ (1 << i)]
        return out

    A = spla.LinearOperator((dim, dim), matvec=mv, dtype=np.float64)
    w = spla.eigsh(A, k=1, which="SA", tol=1e-12)[0]
    return float(w[0])


def psi_vector(net, hilb):
    return net.logpsi(hilb.all_states())


def ket_distribution(net, hilb):
    lp = np.real(net.logpsi(hilb.all_states())) * 2
    p = np.exp(lp - lp.max())
    return p / p.sum()


def doubled_distribution(net, hilb):
    st = hilb.all_states()
    D = hilb.dim
    sr = np.repeat(st[None], D, axis=0).reshape(-1, hilb.n_sites)   # row fast
    sc = np.repeat(st, D, axis=0)
    lp = np.real(net.logpsi(sr, sc)) * 2
    p = np.exp(lp - lp.max())
    return p / p.sum()      # index = col*D + row


def diagonal_distribution(net, hilb):
    """p(σ) ∝ ρ(σ, σ) = exp(Re logρ(σ, σ)) (base_networks.jl:157), index = σ."""
    st = hilb.all_states()
    lp = np.real(net.logpsi(st, st))
    p = np.exp(lp - lp.max())
    return p / p.sum()


def density_matrix(net, hilb):
    """ρ[σ, η] = exp(logρ(σ, η)) over all states (row index σ)."""
    st = hilb.all_states()
    D = hilb.dim
    sr = np.repeat(st, D, axis=0)                                    # row slow
    sc = np.repeat(st[None], D, axis=0).reshape(-1, hilb.n_sites)    # column fast
    return np.exp(net.logpsi(sr, sc)).reshape(D, D)


def dm_expectation(net, O):
    """Tr(ρ O) / Tr(ρ) by dense enumeration."""
    rho = density_matrix(net, O.hilb)
    return np.trace(rho @ ops.to_matrix(O)) / np.trace(rho)


def exact_local_energy_expectation(net, H):
    """<ψ|H|ψ>/<ψ|ψ> by dense enumeration."""
    hilb = H.hilb
    psi = np.exp(psi_vector(net, hilb))
    Hd = ops.to_matrix(H)
    return np.vdot(psi, Hd @ psi) / np.vdot(psi, psi)


def tfim_ground_energy_2d(Lx, Ly, h, J, z2=True, iters=300, tol=1e-11):
    """Ground energy of ``tfim_2d(Lx, Ly, h, J)`` by the matrix-free Lanczos
    recurrence of oracle/lanczos.c (even sector of the global spin flip when
    ``z2``): the lowest eigenvalue of the tridiagonal Lanczos matrix, taken
    once it changes by less than ``tol`` between 20-step checkpoints."""
    import scipy.linalg as sla
    from . import cbuild
    lib = cbuild.lib()
    alpha = np.zeros(iters)
    beta = np.zeros(iters)
    k = lib.tfim2d_lanczos(int(Lx), int(Ly), float(h), float(J), 1 if z2 else 0, int(iters),
                           alpha.ctypes.data, beta.ctypes.data)
    if k <= 0:
        raise MemoryError("tfim2d_lanczos failed")
    prev = None
    e = None
    for m in list(range(20, k, 20)) + [k]:
        e = float(sla.eigh_tridiagonal(alpha[:m], beta[:m - 1], eigvals_only=True,
                                       select="i", select_range=(0, 0))[0])
        if prev is not None and abs(e - prev) < tol:
            return e
        prev = e
    return e
