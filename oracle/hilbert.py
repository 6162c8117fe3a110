"""Hilbert-space encodings (test infrastructure, see ``oracle/__init__``).

Restates src/Hilbert/HomogeneousSpin.jl and HomogeneousFock.jl for local
dimension d:

* spin:  value of local index k (0-based) is ``2k - (d-1)``
  (``set!`` HomogeneousSpin.jl:116-125, ``local_index`` :164-179), so for
  spin-1/2 index 0 <-> -1 and index 1 <-> +1.
* Fock:  value of local index k is ``k`` (HomogeneousFock.jl:106-114, 148-163).

Configurations are float64 arrays of site values; multi-site local indices put
the first listed site in the least significant digit.  Doubled states (row,
col) follow src/Hilbert/SuperHilbert.jl: the flat index is
``col_index * dim + row_index`` (``toint`` SuperHilbert.jl:50-56).
"""
import numpy as np

SPIN = "spin"
FOCK = "fock"


class Hilbert:
    def __init__(self, n_sites, kind=SPIN, local_dim=2):
        self.n_sites = int(n_sites)
        self.kind = kind
        self.d = int(local_dim)

    # ---- encodings ----
    def value(self, k):
        k = np.asarray(k)
        if self.kind == SPIN:
            return (2 * k - (self.d - 1)).astype(np.float64)
        return k.astype(np.float64)

    def index_of_value(self, v):
        v = np.asarray(v)
        if self.kind == SPIN:
            return np.rint((v + (self.d - 1)) / 2).astype(np.int64)
        return np.rint(v).astype(np.int64)

    def fill_value(self):
        """Value used by ``state(...)`` to fill new state buffers
        (HomogeneousSpin.jl:69-70 -> -(d-1); HomogeneousFock.jl:48-49 -> 0)."""
        return float(-(self.d - 1)) if self.kind == SPIN else 0.0

    @property
    def dim(self):
        return self.d ** self.n_sites

    def local_index(self, sigma, sites):
        """0-based local row index of ``sigma`` (..., N) on ``sites``."""
        idx = 0
        for k, s in enumerate(sites):
            idx = idx + self.index_of_value(sigma[..., s]) * self.d ** k
        return idx

    def state_from_index(self, i):
        """``set!(σ, h, i+1)``: configuration of the 0-based basis index i."""
        i = np.asarray(i, dtype=np.int64)
        out = np.empty(i.shape + (self.n_sites,), dtype=np.float64)
        v = i.copy()
        for s in range(self.n_sites):
            v, r = np.divmod(v, self.d)
            out[..., s] = self.value(r)
        return out

    def index_of_state(self, sigma):
        """``toint(σ, h) - 1``."""
        sigma = np.asarray(sigma)
        idx = np.zeros(sigma.shape[:-1], dtype=np.int64)
        for s in range(self.n_sites):
            idx += self.index_of_value(sigma[..., s]) * self.d ** s
        return idx

    def all_states(self):
        return self.state_from_index(np.arange(self.dim))

    def flip(self, value):
        """Local flip of a 2-level site (HomogeneousSpin.jl:95-104,
        HomogeneousFock.jl:72-81)."""
        assert self.d == 2
        if self.kind == SPIN:
            return -value
        return 1.0 - value
