"""Lattices and lattice operators of the reference API (host side).

``HyperCube(dims; periodic, neighbours_distances)``
(src/External/ColoredGraphs/WrappedSimpleGraphs/HyperCube.jl:26-95): vertex v
(1-based) has the column-major coordinates of v in ``dims``; every vertex is
joined to its ±Δ neighbours along each dimension (wrapping where periodic).
The graph is simple, so ``edges`` lists every pair once as (u, v) with u < v
in increasing order, the iteration order of the reference's SimpleGraph, which
fixes the term order of the operators built from it.

``quantum_ising_hamiltonian(lattice, hilb; g, V)`` and
``lattice_average_operator(lattice, hilb, op)``
(src/Operators/SimpleOperators.jl:160-185) build the reference's operators
from a lattice; ``translational_symm_table`` (HyperCube.jl:103-136) lists the
lattice translations used by NDMSymm.
"""
import numpy as np

from .operators import LocalOperator, sigmax, sigmaz


def _coords(v, dims):
    """Column-major coordinates (1-based) of vertex v (1-based)."""
    c, r = [], v - 1
    for d in dims:
        c.append(r % d + 1)
        r //= d
    return c


class HyperCube:
    def __init__(self, dims, periodic=True, neighbours_distances=(1,)):
        self.dims = [int(d) for d in dims]
        nv = int(np.prod(self.dims))
        if isinstance(periodic, (list, tuple)):
            if len(periodic) != len(self.dims):
                raise ValueError("periodic should match sizes")
            per = [bool(p) for p in periodic]
        else:
            per = [bool(periodic)] * len(self.dims)
        if isinstance(neighbours_distances, int):
            neighbours_distances = [neighbours_distances]
        for dist in neighbours_distances:
            if not all(dist < d for d in self.dims):
                raise ValueError("neighbours_distances must be smaller than every dimension")
        self.periodic = per
        self.vert_coords = [_coords(v, self.dims) for v in range(1, nv + 1)]
        index = {tuple(c): v for v, c in enumerate(self.vert_coords, start=1)}
        adj = set()
        for v, co in enumerate(self.vert_coords, start=1):
            for j, (dim, loop) in enumerate(zip(self.dims, per)):
                for delta in neighbours_distances:
                    for dj in (delta, -delta):
                        nj = co[j] + dj
                        if nj < 1 or nj > dim:
                            if not loop:
                                continue
                            nj = (nj - 1) % dim + 1
                        c2 = list(co)
                        c2[j] = nj
                        u = index[tuple(c2)]
                        if u != v:
                            adj.add((min(u, v), max(u, v)))
        self._edges = sorted(adj)
        self._nv = nv

    def nv(self):
        return self._nv

    def ne(self):
        return len(self._edges)

    def vertices(self):
        return list(range(1, self._nv + 1))

    def edges(self):
        """(src, dst) pairs, 1-based, src < dst, in increasing order."""
        return list(self._edges)

    def __repr__(self):
        return f"HyperCube with {self._nv} vertices, {len(self._edges)} edges"


def translational_symm_table(lattice):
    """``translational_symm_table(g::HyperCube)``: for every translation the
    vector vec(circshift(reshape(1:nv, dims), shift)) (1-based sites), shifts
    in the reference's loop order (first dimension outermost)."""
    dims = lattice.dims
    if len(dims) > 3:
        raise ValueError("translations of hypercubes of up to 3 dimensions")
    lat = np.arange(1, lattice.nv() + 1).reshape(dims, order="F")
    table = []
    for shift in np.ndindex(*dims):
        table.append(np.roll(lat, shift, axis=tuple(range(len(dims)))).reshape(-1, order="F").tolist())
    return table


def quantum_ising_hamiltonian(lattice, hilb, g, V):
    """H = Σ_i g/2 σx_i + Σ_(i,j) V/4 σz_i σz_j over the lattice's vertices
    and edges (SimpleOperators.jl:160-173)."""
    H = LocalOperator(hilb)
    for i in lattice.vertices():
        H = H + (g / 2.0) * sigmax(hilb, i)
    for i, j in lattice.edges():
        H = H + (V / 4.0) * sigmaz(hilb, i) * sigmaz(hilb, j)
    return H


def lattice_average_operator(lattice, hilb, op):
    """(1/nv) Σ_i op(hilb, i) (SimpleOperators.jl:175-185)."""
    O = LocalOperator(hilb)
    for i in lattice.vertices():
        O = O + op(hilb, i)
    return O / lattice.nv()
