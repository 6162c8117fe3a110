"""Network parameter containers of the reference API (host side).

``RBM(T, N, α, f)`` (src/Networks/ClosedSystems/RBM.jl:40-48),
``NDM(T, N, αh, αa, f)`` (src/Networks/MixedDensityMatrix/NDM.jl:50-63) and
``RBMSplit(T, N, α)`` (src/Networks/MixedDensityMatrix/RBMSplit.jl:33-42)
hold their arrays on the host in the reference layout; the engine keeps the
authoritative FP64 copy on the device while a ``BatchedSampler`` is bound and
writes it back after every ``update_``.  The flat parameter vector is the
functor field order with column-major arrays (src/tuple_logic.jl:31-72).
"""
import numpy as np

af_logcosh = "logcosh"
af_softplus = "softplus"
identity = "identity"


class RBM:
    def __init__(self, T, N, alpha, f=af_softplus):
        self.dtype = np.dtype(T)
        if self.dtype.kind != "c":
            raise ValueError("the RBM takes complex weights (ComplexF32 / ComplexF64)")
        self.N = int(N)
        self.M = int(round(alpha * N))
        self.f = f
        self.a = np.zeros(self.N, self.dtype)
        self.b = np.zeros(self.M, self.dtype)
        self.W = np.zeros((self.M, self.N), self.dtype)

    @property
    def n_params(self):
        return self.N + self.M + self.M * self.N

    def flat(self):
        return np.concatenate([self.a, self.b, self.W.reshape(-1, order="F")]).astype(np.complex128)

    def set_flat(self, v):
        v = np.asarray(v)
        N, M = self.N, self.M
        self.a = v[:N].astype(self.dtype)
        self.b = v[N:N + M].astype(self.dtype)
        self.W = v[N + M:].reshape((M, N), order="F").astype(self.dtype)

    def __repr__(self):
        return f"RBM({self.dtype}, n={self.N}, α={self.M / self.N}, f={self.f})"


class NDM:
    FIELDS = ("b_mu", "h_mu", "w_mu", "u_mu", "b_la", "h_la", "d_la", "w_la", "u_la")

    def __init__(self, T, N, alpha_h, alpha_a, f=af_softplus):
        self.dtype = np.dtype(T)
        if self.dtype.kind == "c":          # NDM.jl:46-47: complex T becomes real
            self.dtype = np.dtype(self.dtype.type(0).real.dtype)
        self.N = int(N)
        self.Mh = int(round(alpha_h * N))
        self.Ma = int(round(alpha_a * N))
        self.f = f
        N, Mh, Ma = self.N, self.Mh, self.Ma
        self.shapes = {"b_mu": (N,), "h_mu": (Mh,), "w_mu": (Mh, N), "u_mu": (Ma, N),
                       "b_la": (N,), "h_la": (Mh,), "d_la": (Ma,), "w_la": (Mh, N),
                       "u_la": (Ma, N)}
        for k in self.FIELDS:
            setattr(self, k, np.zeros(self.shapes[k], self.dtype))

    @property
    def n_params(self):
        return sum(int(np.prod(s)) for s in self.shapes.values())

    def flat(self):
        return np.concatenate([getattr(self, k).reshape(-1, order="F") for k in self.FIELDS])

    def set_flat(self, v):
        v = np.real(np.asarray(v))
        o = 0
        for k in self.FIELDS:
            n = int(np.prod(self.shapes[k]))
            setattr(self, k, v[o:o + n].reshape(self.shapes[k], order="F").astype(self.dtype))
            o += n


class RBMSplit:
    """Density-matrix RBM over (σ, η) with complex weights: fields ar, ac (N),
    b (αN), Wr, Wc (αN x N); the activation is logcosh (logℒ), as in the
    reference, unless given."""

    FIELDS = ("ar", "ac", "b", "Wr", "Wc")

    def __init__(self, T, N, alpha, f=af_logcosh):
        self.dtype = np.dtype(T)
        if self.dtype.kind != "c":
            raise ValueError("RBMSplit takes complex weights (ComplexF32 / ComplexF64)")
        self.N = int(N)
        self.M = int(round(alpha * N))
        self.f = f
        N, M = self.N, self.M
        self.shapes = {"ar": (N,), "ac": (N,), "b": (M,), "Wr": (M, N), "Wc": (M, N)}
        for k in self.FIELDS:
            setattr(self, k, np.zeros(self.shapes[k], self.dtype))

    @property
    def n_params(self):
        return 2 * self.N + self.M + 2 * self.M * self.N

    def flat(self):
        return np.concatenate([getattr(self, k).reshape(-1, order="F") for k in self.FIELDS]).astype(np.complex128)

    def set_flat(self, v):
        v = np.asarray(v)
        o = 0
        for k in self.FIELDS:
            n = int(np.prod(self.shapes[k]))
            setattr(self, k, v[o:o + n].reshape(self.shapes[k], order="F").astype(self.dtype))
            o += n

    def __repr__(self):
        return f"RBMSplit({self.dtype}, n={self.N}, α={self.M / self.N})"


class NDMSymm(NDM):
    """``NDMSymm(T, N, αh, αa, permutations, f=logℒ)`` (NDMSymm.jl:17-30): the
    trainable parameters are those of a symmetric NDM with αh hidden and αa
    ancilla features (fields as NDM); the network evaluated is the bare NDM
    whose units are those features under every permutation (site lists,
    0-based or, as translational_symm_table gives them, 1-based).  The
    symmetric visible biases are kept at their means."""

    def __init__(self, T, N, alpha_h, alpha_a, permutations, f=af_logcosh):
        super().__init__(T, N, alpha_h / N, alpha_a / N, f)
        perms = np.asarray(permutations, dtype=np.int64)
        if perms.ndim != 2 or perms.shape[1] != self.N:
            raise ValueError("permutations must be a list of site lists of length N")
        if all(sorted(p.tolist()) == list(range(1, self.N + 1)) for p in perms):
            perms = perms - 1            # 1-based site lists (translational_symm_table)
        for p in perms:
            if sorted(p.tolist()) != list(range(self.N)):
                raise ValueError("every permutation must be a permutation of the sites 0..N-1")
        self.permutations = perms

    @property
    def n_symm(self):
        return len(self.permutations)

    def __repr__(self):
        return f"NDMSymm({self.dtype}, n={self.N}, αh={self.Mh}, αa={self.Ma}, n_symm={self.n_symm})"


def glorot_uniform(T, *dims, rng=None):
    """``glorot_uniform`` (src/Networks/utils.jl:7): (rand(T, dims) .- 0.5) *
    sqrt(24 / Σ dims); for a complex T Julia's rand draws both parts in [0, 1)
    and the shift applies to the real part only."""
    rng = np.random.default_rng() if rng is None else rng
    T = np.dtype(T)
    scale = np.sqrt(24.0 / sum(dims))
    if T.kind == "c":
        v = (rng.random(dims) - 0.5) + 1j * rng.random(dims)
    else:
        v = rng.random(dims) - 0.5
    return (v * scale).astype(T)


class Dense:
    """``Dense(T, in, out, σ=identity)`` (Chains/Layers/Dense.jl:24-36):
    y = σ.(W x .+ b), W out x in, glorot-uniform initialisation."""

    def __init__(self, T, n_in, n_out, f=identity, rng=None):
        self.dtype = np.dtype(T)
        self.n_in, self.n_out, self.f = int(n_in), int(n_out), f
        self.W = glorot_uniform(self.dtype, self.n_out, self.n_in, rng=rng)
        self.b = glorot_uniform(self.dtype, self.n_out, rng=rng)

    def arrays(self):
        return [self.W, self.b]


class DenseSplit:
    """``DenseSplit(T, in, out, σ=identity)`` (Chains/Layers/DenseSplit.jl:3-19):
    the first layer of a density-matrix chain, y = σ.(Wr σr .+ Wc σc .+ b) on
    the row and column configurations, Wr and Wc out x in, glorot-uniform
    initialisation; functor order Wr, Wc, b."""

    def __init__(self, T, n_in, n_out, f=identity, rng=None):
        self.dtype = np.dtype(T)
        self.n_in, self.n_out, self.f = int(n_in), int(n_out), f
        self.Wr = glorot_uniform(self.dtype, self.n_out, self.n_in, rng=rng)
        self.Wc = glorot_uniform(self.dtype, self.n_out, self.n_in, rng=rng)
        self.b = glorot_uniform(self.dtype, self.n_out, rng=rng)

    def arrays(self):
        return [self.Wr, self.Wc, self.b]


class PositiveDefR:
    """``PositiveDefR(T, in, out, σ=identity)`` (Chains/Layers/PositiveDefR.jl):
    the first layer of a density-matrix chain,
    y = σ.(Wr (σr .+ σc) .+ im Wi (σr .- σc) .+ b), with real Wr, Wi (out x in)
    and b, glorot-uniform initialisation; functor order Wr, Wi, b.  T is the
    real element type (STD_REAL_PREC = Float32 by default)."""

    def __init__(self, T=np.float32, n_in=None, n_out=None, f=identity, rng=None):
        self.dtype = np.dtype(T)
        if self.dtype.kind == "c":
            raise ValueError("PositiveDefR takes real weights (Float32 / Float64)")
        self.n_in, self.n_out, self.f = int(n_in), int(n_out), f
        self.Wr = glorot_uniform(self.dtype, self.n_out, self.n_in, rng=rng)
        self.Wi = glorot_uniform(self.dtype, self.n_out, self.n_in, rng=rng)
        self.b = glorot_uniform(self.dtype, self.n_out, rng=rng)

    def arrays(self):
        return [self.Wr, self.Wi, self.b]


class WSum:
    """``WSum(T, in)`` (Chains/Layers/WeightedSum.jl): logψ = Σ_i c_i x_i."""

    def __init__(self, T, n_in, rng=None):
        self.dtype = np.dtype(T)
        self.n_in = int(n_in)
        self.c = glorot_uniform(self.dtype, self.n_in, rng=rng)

    def arrays(self):
        return [self.c]


class _SumAutobatch:
    """``sum_autobatch`` (Chains/Layers/sum.jl): logψ = Σ_i x_i."""

    def arrays(self):
        return []

    def __repr__(self):
        return "sum_autobatch"


sum_autobatch = _SumAutobatch()


class Chain:
    """``Chain(layers...)`` (Chains/Chain.jl:24-27)."""

    def __init__(self, *layers):
        self.layers = list(layers)


class PureStateAnsatz:
    """``PureStateAnsatz(chain, N)`` (ClosedSystems/PureChainWrapper.jl:23-41):
    a ket whose logψ is the chain's output; the flat parameter vector is the
    functor order of the layers (Dense: W column-major, then b; WSum: c)."""

    def __init__(self, chain, n_sites):
        if isinstance(n_sites, int):
            self.N = n_sites
        else:
            self.N = n_sites.n_sites
        self.chain = chain if isinstance(chain, Chain) else Chain(*chain)
        layers = self.chain.layers
        if not layers or not all(isinstance(l, Dense) for l in layers[:-1]) or \
                not isinstance(layers[-1], (WSum, _SumAutobatch)) or len(layers) < 2:
            raise ValueError("the chain is Dense layers closed by WSum or sum_autobatch")
        width = self.N
        for l in layers[:-1]:
            if l.n_in != width:
                raise ValueError("layer widths do not match")
            width = l.n_out
        if isinstance(layers[-1], WSum) and layers[-1].n_in != width:
            raise ValueError("WSum width does not match the last Dense layer")
        self.out_width = width
        self.dtype = np.result_type(*[a.dtype for l in layers for a in l.arrays()])

    @property
    def n_params(self):
        return sum(a.size for l in self.chain.layers for a in l.arrays())

    def flat(self):
        return np.concatenate([a.reshape(-1, order="F") for l in self.chain.layers for a in l.arrays()]).astype(
            np.complex128)

    def set_flat(self, v):
        v = np.asarray(v)
        o = 0
        for l in self.chain.layers:
            if isinstance(l, Dense):
                n = l.W.size
                l.W = v[o:o + n].reshape(l.W.shape, order="F").astype(l.dtype)
                o += n
                l.b = v[o:o + l.n_out].astype(l.dtype)
                o += l.n_out
            elif isinstance(l, WSum):
                l.c = v[o:o + l.n_in].astype(l.dtype)
                o += l.n_in

    def __repr__(self):
        return f"PureStateAnsatz(Chain of {len(self.chain.layers)} layers, N={self.N})"


class MixedStateAnsatz:
    """``MixedStateAnsatz(chain, N)`` (MixedDensityMatrix/MixedChainWrapper.jl:
    3-37): a density matrix whose logρ(σ, η) is the chain's output for the
    pair of configurations; the chain is DenseSplit(N, out) or
    PositiveDefR(N, out) followed by Dense layers and closed by WSum or
    sum_autobatch.  Parameters in the functor order (DenseSplit: Wr, Wc, b;
    PositiveDefR: Wr, Wi, b; Dense: W, b; WSum: c), as a complex vector.
    Since DenseSplit's θ = Wr σ + Wc η + b is a Dense layer on the 2N doubled
    sites with W = [Wr Wc], whose column-major storage is Wr then Wc, the flat
    vector is that of a chain over the doubled sites.  PositiveDefR's
    parameters are real: the vector holds them with zero imaginary part, and
    ``real_sr`` is set, since the reference's SR takes its element type from
    the first trainable array (SRDirect.jl:11-38)."""

    def __init__(self, chain, n_sites):
        self.N = n_sites if isinstance(n_sites, int) else n_sites.n_sites
        self.chain = chain if isinstance(chain, Chain) else Chain(*chain)
        layers = self.chain.layers
        if len(layers) < 2 or not isinstance(layers[0], (DenseSplit, PositiveDefR)) or \
                not all(isinstance(l, Dense) for l in layers[1:-1]) or not isinstance(layers[-1], (WSum, _SumAutobatch)):
            raise ValueError("the chain is DenseSplit or PositiveDefR, then Dense layers, closed by WSum or "
                             "sum_autobatch")
        if layers[0].n_in != self.N:
            raise ValueError("the first layer's input width must be the number of sites")
        self.real_sr = isinstance(layers[0], PositiveDefR)
        width = layers[0].n_out
        for l in layers[1:-1]:
            if l.n_in != width:
                raise ValueError("layer widths do not match")
            width = l.n_out
        if isinstance(layers[-1], WSum) and layers[-1].n_in != width:
            raise ValueError("WSum width does not match the last Dense layer")
        self.dtype = np.result_type(*[a.dtype for l in layers for a in l.arrays()])

    @property
    def n_params(self):
        return sum(a.size for l in self.chain.layers for a in l.arrays())

    def flat(self):
        return np.concatenate([a.reshape(-1, order="F") for l in self.chain.layers for a in l.arrays()]).astype(
            np.complex128)

    def set_flat(self, v):
        v = np.asarray(v)
        o = 0
        for l in self.chain.layers:
            names = {DenseSplit: ("Wr", "Wc", "b"), PositiveDefR: ("Wr", "Wi", "b"), Dense: ("W", "b"),
                     WSum: ("c",)}.get(type(l), ())
            for name in names:
                a = getattr(l, name)
                x = v[o:o + a.size].reshape(a.shape, order="F")
                setattr(l, name, (np.real(x) if l.dtype.kind != "c" else x).astype(l.dtype))
                o += a.size

    def __repr__(self):
        return f"MixedStateAnsatz(Chain of {len(self.chain.layers)} layers, N={self.N})"


def PureChain(N, *layers):
    """``PureChain(N, layers...)`` (PureChainWrapper.jl:57-60)."""
    return PureStateAnsatz(Chain(*layers), N)


def init_random_pars_(net, sigma=0.01, rng=None):
    """``init_random_pars!`` (src/utils/rng.jl:27-38): every weight is drawn
    from randn * sqrt(sigma); complex draws have variance 1/2 per part."""
    rng = np.random.default_rng() if rng is None else rng
    p = net.flat()
    chain = getattr(net, "chain", None)
    if chain is not None and any(a.dtype.kind != "c" for l in chain.layers for a in l.arrays()):
        # a chain holding real arrays (PositiveDefR): each array drawn in its own type
        parts = []
        for a in (a for l in chain.layers for a in l.arrays()):
            if a.dtype.kind == "c":
                parts.append((rng.standard_normal(a.size) + 1j * rng.standard_normal(a.size)) / np.sqrt(2.0))
            else:
                parts.append(rng.standard_normal(a.size) + 0j)
        net.set_flat(np.concatenate(parts) * np.sqrt(sigma))
        return net
    if np.iscomplexobj(p):
        v = (rng.standard_normal(p.size) + 1j * rng.standard_normal(p.size)) / np.sqrt(2.0)
    else:
        v = rng.standard_normal(p.size)
    net.set_flat(v * np.sqrt(sigma))
    return net
