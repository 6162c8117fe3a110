"""Hilbert spaces of the reference API (src/Hilbert/).

``HomogeneousSpin(N, 1//2)`` (HomogeneousSpin.jl:23-52) and
``HomogeneousFock(N, 2)`` (HomogeneousFock.jl) with two local states, plus
``SuperOpSpace`` (SuperHilbert.jl:17-20) for density matrices.  Local index k
of a spin site has value 2k - 1 (-1 / +1); of a Fock site the value k.
"""


class HomogeneousSpin:
    kind = "spin"

    def __init__(self, n_sites, S=0.5):
        if abs(S - 0.5) > 1e-12:
            raise ValueError("only spin-1/2 (two local states) is supported")
        self.n_sites = int(n_sites)
        self.local_dim = 2

    def value(self, k):
        return 2 * k - 1

    def index(self, v):
        return (int(v) + 1) // 2

    def __repr__(self):
        return f"HomogeneousSpin({self.n_sites}, 2)"


class HomogeneousFock:
    kind = "fock"

    def __init__(self, n_sites, n_max=2):
        if n_max != 2:
            raise ValueError("only two local states are supported")
        self.n_sites = int(n_sites)
        self.local_dim = 2

    def value(self, k):
        return k

    def index(self, v):
        return int(v)

    def __repr__(self):
        return f"HomogeneousFock({self.n_sites}, 2)"


class SuperOpSpace:
    """Doubled space of density matrices: configurations (σ, η)."""

    def __init__(self, basis):
        self.basis = basis
        self.n_sites = 2 * basis.n_sites
        self.local_dim = basis.local_dim
        self.kind = basis.kind


def physical(h):
    return h.basis if isinstance(h, SuperOpSpace) else h


def nsites(h):
    return h.n_sites
