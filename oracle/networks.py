"""RBM and NDM networks in FP64 (test infrastructure, see ``oracle/__init__``).

Flat parameter order = functor field order, each array column-major
(src/tuple_logic.jl:31-72):

* RBM  (src/Networks/ClosedSystems/RBM.jl:3-12):  a (N), b (M), W (M x N)
* NDM  (src/Networks/MixedDensityMatrix/NDM.jl:3-19): b_mu (N), h_mu (aN),
  w_mu (aN x N), u_mu (bN x N), b_la (N), h_la (aN), d_la (bN), w_la (aN x N),
  u_la (bN x N)
* RBMSplit (src/Networks/MixedDensityMatrix/RBMSplit.jl:3-10): ar (N),
  ac (N), b (aN), Wr (aN x N), Wc (aN x N)
* NDMSymm (src/Networks/MixedDensityMatrix/NDMSymm.jl:3-40): the trainable
  vector is the symmetric NDM's (NDM order with ah hidden, aa ancilla)
* Chain of Dense layers + WSum / sum_autobatch (src/Networks/Chains/): per
  Dense layer W (out x in) then b, then the WSum weights c

Activations follow src/Networks/activation.jl:5-45; the derivative used by the
networks is ``fwd_der(f, x)`` (tanh for logcosh, sigmoid for softplus).
"""
import numpy as np

LOGCOSH = "logcosh"
SOFTPLUS = "softplus"
IDENTITY = "identity"


def logcosh(x):
    """``logℒ2`` (activation.jl:9-13)."""
    x = np.asarray(x)
    if np.iscomplexobj(x):
        re, im = x.real, x.imag
        return _logcosh_real(re) + np.log(np.cos(im) + 1j * np.tanh(re) * np.sin(im))
    return _logcosh_real(x)


def _logcosh_real(x):
    ax = np.abs(x)
    with np.errstate(over="ignore"):
        small = np.log(np.cosh(np.where(ax <= 12.0, x, 0.0)))
    return np.where(ax <= 12.0, small, ax - np.log(2.0))


def softplus(x):
    """``logℒ(x) = log1p(exp(x))`` (activation.jl:20)."""
    return np.log1p(np.exp(x))


def act(name, x):
    if name == IDENTITY:
        return np.asarray(x)
    return logcosh(x) if name == LOGCOSH else softplus(x)


def dact(name, x):
    """``fwd_der(f, x)`` (activation.jl:22-29)."""
    if name == IDENTITY:
        return np.ones_like(np.asarray(x))
    if name == LOGCOSH:
        return np.tanh(x)
    return 1.0 / (1.0 + np.exp(-x))


# ---------------------------------------------------------------------------
# RBM
# ---------------------------------------------------------------------------

class RBM:
    def __init__(self, n, m, activation=LOGCOSH, dtype=np.complex128):
        self.N, self.M = int(n), int(m)
        self.activation = activation
        self.a = np.zeros(self.N, dtype)
        self.b = np.zeros(self.M, dtype)
        self.W = np.zeros((self.M, self.N), dtype)

    @property
    def n_params(self):
        return self.N + self.M + self.M * self.N

    def flat(self):
        return np.concatenate([self.a, self.b, self.W.reshape(-1, order="F")])

    def set_flat(self, v):
        v = np.asarray(v)
        N, M = self.N, self.M
        self.a = v[:N].astype(self.a.dtype).copy()
        self.b = v[N:N + M].astype(self.b.dtype).copy()
        self.W = v[N + M:].reshape((M, N), order="F").astype(self.W.dtype).copy()

    def theta(self, sigma):
        """θ = Wσ + b for a batch sigma (B, N) -> (B, M)."""
        return sigma @ self.W.T + self.b[None, :]

    def logpsi(self, sigma):
        """RBMBatched.jl:37-56."""
        sigma = np.atleast_2d(sigma)
        th = self.theta(sigma)
        return sigma @ self.a + act(self.activation, th).sum(axis=1)

    def logpsi_and_grad(self, sigma):
        """RBMBatched.jl:58-91; grad has shape (B, P)."""
        sigma = np.atleast_2d(sigma)
        th = self.theta(sigma)
        out = sigma @ self.a + act(self.activation, th).sum(axis=1)
        g = dact(self.activation, th)
        B = sigma.shape[0]
        dW = g[:, :, None] * np.conj(sigma)[:, None, :]            # (B, M, N)
        grad = np.concatenate([sigma.astype(g.dtype), g,
                               dW.transpose(0, 2, 1).reshape(B, -1)], axis=1)
        return out, grad

    def log_prob(self, sigma):
        """``log_prob_ψ!`` for kets: 2 Re logψ (base_batched_networks.jl:255-258)."""
        return 2.0 * np.real(self.logpsi(sigma))


# ---------------------------------------------------------------------------
# NDM
# ---------------------------------------------------------------------------

class NDM:
    FIELDS = ("b_mu", "h_mu", "w_mu", "u_mu", "b_la", "h_la", "d_la", "w_la", "u_la")

    def __init__(self, n, alpha_h, alpha_a, activation=SOFTPLUS):
        self.N = int(n)
        self.Mh = int(round(alpha_h * n))
        self.Ma = int(round(alpha_a * n))
        self.activation = activation
        N, Mh, Ma = self.N, self.Mh, self.Ma
        self.shapes = {"b_mu": (N,), "h_mu": (Mh,), "w_mu": (Mh, N), "u_mu": (Ma, N),
                       "b_la": (N,), "h_la": (Mh,), "d_la": (Ma,), "w_la": (Mh, N),
                       "u_la": (Ma, N)}
        for f in self.FIELDS:
            setattr(self, f, np.zeros(self.shapes[f]))

    @property
    def n_params(self):
        return sum(int(np.prod(s)) for s in self.shapes.values())

    def flat(self):
        return np.concatenate([getattr(self, f).reshape(-1, order="F") for f in self.FIELDS])

    def set_flat(self, v):
        v = np.real(np.asarray(v)).astype(np.float64)
        o = 0
        for f in self.FIELDS:
            n = int(np.prod(self.shapes[f]))
            setattr(self, f, v[o:o + n].reshape(self.shapes[f], order="F").copy())
            o += n

    def _parts(self, sr, sc):
        f = self.activation
        tl_s = sr @ self.w_la.T + self.h_la
        tm_s = sr @ self.w_mu.T + self.h_mu
        tl_c = sc @ self.w_la.T + self.h_la
        tm_c = sc @ self.w_mu.T + self.h_mu
        ssum = sr + sc
        sdif = sr - sc
        pi = 0.5 * ssum @ self.u_la.T + 0.5j * sdif @ self.u_mu.T + self.d_la
        gl = 0.5 * (act(f, tl_s).sum(1) + act(f, tl_c).sum(1) + ssum @ self.b_la)
        gm = 0.5 * (act(f, tm_s).sum(1) - act(f, tm_c).sum(1) + sdif @ self.b_mu)
        out = gl + 1j * gm + act(f, pi).sum(1)
        return out, tl_s, tm_s, tl_c, tm_c, ssum, sdif, pi

    def logpsi(self, sr, sc):
        """NDM.jl:76-96 / NDMBatched.jl:94-175 for batches (B, N)."""
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        return self._parts(sr, sc)[0]

    def logpsi_and_grad(self, sr, sc):
        """NDMBatched.jl:177-280; grad (B, P) complex in the flat order."""
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        out, tl_s, tm_s, tl_c, tm_c, ssum, sdif, pi = self._parts(sr, sc)
        f = self.activation
        dl_s, dm_s = dact(f, tl_s), dact(f, tm_s)
        dl_c, dm_c = dact(f, tl_c), dact(f, tm_c)
        dpi = dact(f, pi)
        B = sr.shape[0]

        def outer(v, w):   # (B, M, N) -> column-major flattening
            return (v[:, :, None] * np.conj(w)[:, None, :]).transpose(0, 2, 1).reshape(B, -1)

        parts = {
            "b_mu": 0.5j * sdif,
            "h_mu": 0.5j * (dm_s - dm_c),
            "w_mu": 0.5j * (outer(dm_s, sr) - outer(dm_c, sc)),
            "u_mu": 0.5j * outer(dpi, sdif),
            "b_la": 0.5 * ssum + 0j,
            "h_la": 0.5 * (dl_s + dl_c) + 0j,
            "d_la": dpi,
            "w_la": 0.5 * (outer(dl_s, sr) + outer(dl_c, sc)) + 0j,
            "u_la": 0.5 * outer(dpi, ssum),
        }
        grad = np.concatenate([parts[k] for k in self.FIELDS], axis=1)
        return out, grad

    def log_prob(self, sr, sc):
        """2 Re log ρ(σ, η) on doubled states (base_batched_networks.jl:255-258)."""
        return 2.0 * np.real(self.logpsi(sr, sc))


class RBMSplit:
    """logρ(σ, η) = ar·σ + ac·η + Σ_h f(b_h + Wr_h·σ + Wc_h·η), complex
    parameters (RBMSplit.jl:48-50 for the value, :111-129 for ∇: ar → σ,
    ac → η, b → f'(θ), Wr → f'(θ) σᵀ, Wc → f'(θ) ηᵀ)."""

    FIELDS = ("ar", "ac", "b", "Wr", "Wc")

    def __init__(self, n, m, activation=LOGCOSH):
        self.N, self.M = int(n), int(m)
        self.activation = activation
        N, M = self.N, self.M
        self.shapes = {"ar": (N,), "ac": (N,), "b": (M,), "Wr": (M, N), "Wc": (M, N)}
        for f in self.FIELDS:
            setattr(self, f, np.zeros(self.shapes[f], np.complex128))

    @property
    def n_params(self):
        return 2 * self.N + self.M + 2 * self.M * self.N

    def flat(self):
        return np.concatenate([getattr(self, f).reshape(-1, order="F") for f in self.FIELDS])

    def set_flat(self, v):
        v = np.asarray(v).astype(np.complex128)
        o = 0
        for f in self.FIELDS:
            n = int(np.prod(self.shapes[f]))
            setattr(self, f, v[o:o + n].reshape(self.shapes[f], order="F").copy())
            o += n

    def _theta(self, sr, sc):
        return sr @ self.Wr.T + sc @ self.Wc.T + self.b[None, :]

    def logpsi(self, sr, sc):
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        return sr @ self.ar + sc @ self.ac + act(self.activation, self._theta(sr, sc)).sum(axis=1)

    def logpsi_and_grad(self, sr, sc):
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        th = self._theta(sr, sc)
        out = sr @ self.ar + sc @ self.ac + act(self.activation, th).sum(axis=1)
        g = dact(self.activation, th)
        B = sr.shape[0]
        dWr = (g[:, :, None] * sr[:, None, :]).transpose(0, 2, 1).reshape(B, -1)
        dWc = (g[:, :, None] * sc[:, None, :]).transpose(0, 2, 1).reshape(B, -1)
        grad = np.concatenate([sr.astype(np.complex128), sc.astype(np.complex128), g, dWr, dWc], axis=1)
        return out, grad

    def log_prob(self, sr, sc):
        """2 Re logρ on doubled states (base_batched_networks.jl:255-258)."""
        return 2.0 * np.real(self.logpsi(sr, sc))


class NDMSymm:
    """NDMSymm.jl: a symmetric NDM ``sym`` (ah hidden, aa ancilla features)
    and the bare NDM with ah n_symm / aa n_symm units built from it by
    ``set_bare_params!`` (:89-133: visible biases replaced by their mean,
    hidden and ancilla biases repeated, bare unit j + f n_symm carrying the
    symmetric weights (f, i) on site perms[j][i]).  logρ is the bare NDM's;
    ∇logρ is the bare gradient mapped by ``construct_∇matrices`` (:135-180).
    ``perms`` are 0-based."""

    def __init__(self, n, ah, aa, perms, activation=LOGCOSH):
        self.N, self.ah, self.aa = int(n), int(ah), int(aa)
        self.perms = np.asarray(perms, dtype=np.int64)
        self.ns = len(self.perms)
        self.activation = activation
        self.sym = NDM(n, ah / n, aa / n, activation)
        self.bare = NDM(n, ah * self.ns / n, aa * self.ns / n, activation)
        self._set_bare()

    @property
    def n_params(self):
        return self.sym.n_params

    def flat(self):
        return self.sym.flat()

    def set_flat(self, v):
        self.sym.set_flat(v)
        self._set_bare()

    def _set_bare(self):
        s, b, ns = self.sym, self.bare, self.ns
        s.b_mu = np.full_like(s.b_mu, s.b_mu.mean())
        s.b_la = np.full_like(s.b_la, s.b_la.mean())
        b.b_mu = s.b_mu.copy()
        b.b_la = s.b_la.copy()
        b.h_mu = np.repeat(s.h_mu, ns)
        b.h_la = np.repeat(s.h_la, ns)
        b.d_la = np.repeat(s.d_la, ns)
        for f in range(self.ah):
            for j, perm in enumerate(self.perms):
                for i, ip in enumerate(perm):
                    b.w_mu[j + f * ns, ip] = s.w_mu[f, i]
                    b.w_la[j + f * ns, ip] = s.w_la[f, i]
        for f in range(self.aa):
            for j, perm in enumerate(self.perms):
                for i, ip in enumerate(perm):
                    b.u_mu[j + f * ns, ip] = s.u_mu[f, i]
                    b.u_la[j + f * ns, ip] = s.u_la[f, i]

    def grad_matrix(self):
        """(P_sym, P_bare) matrix of construct_∇matrices in the flat orders."""
        s, b, ns, N = self.sym, self.bare, self.ns, self.N
        def offs(net):
            o, out = 0, {}
            for f in NDM.FIELDS:
                out[f] = o
                o += int(np.prod(net.shapes[f]))
            return out
        so, bo = offs(s), offs(b)
        G = np.zeros((s.n_params, b.n_params))
        for f in ("b_mu", "b_la"):
            G[so[f]:so[f] + N, bo[f]:bo[f] + N] = 1.0 / N
        for f, m in (("h_mu", self.ah), ("h_la", self.ah), ("d_la", self.aa)):
            for k in range(m):
                G[so[f] + k, bo[f] + k * ns:bo[f] + (k + 1) * ns] = 1.0
        for f, m, mb in (("w_mu", self.ah, b.Mh), ("w_la", self.ah, b.Mh),
                         ("u_mu", self.aa, b.Ma), ("u_la", self.aa, b.Ma)):
            for fe in range(m):
                for j, perm in enumerate(self.perms):
                    for i, ip in enumerate(perm):
                        G[so[f] + fe + m * i, bo[f] + (j + fe * ns) + mb * ip] = 1.0
        return G

    def logpsi(self, sr, sc):
        return self.bare.logpsi(sr, sc)

    def logpsi_and_grad(self, sr, sc):
        out, g = self.bare.logpsi_and_grad(sr, sc)
        return out, g @ self.grad_matrix().T

    def log_prob(self, sr, sc):
        return self.bare.log_prob(sr, sc)


class Chain:
    """Feed-forward ket (Chain.jl:24-90): ``layers`` is a list of
    ("dense", n_in, n_out, activation), then one ("wsum", n_in) or
    ("sum", n_in).  Dense.jl:73-104: θ = W x + b, y = f(θ), ∇W = δθ xᵀ,
    ∇b = δθ, δ_in = Wᵀ δθ with δθ = δ f'(θ); WeightedSum.jl: logψ = Σ c x,
    ∇c = x, δ = c; sum.jl: logψ = Σ x, δ = 1.  Complex parameters."""

    def __init__(self, n, layers):
        self.N = int(n)
        self.layers = [tuple(l) for l in layers]
        self.params = []
        for l in self.layers:
            if l[0] == "dense":
                self.params.append([np.zeros((l[2], l[1]), np.complex128), np.zeros(l[2], np.complex128)])
            elif l[0] == "wsum":
                self.params.append([np.zeros(l[1], np.complex128)])
            else:
                self.params.append([])

    @property
    def n_params(self):
        return sum(a.size for ps in self.params for a in ps)

    def flat(self):
        return np.concatenate([a.reshape(-1, order="F") for ps in self.params for a in ps])

    def set_flat(self, v):
        v = np.asarray(v).astype(np.complex128)
        o = 0
        for ps in self.params:
            for k, a in enumerate(ps):
                ps[k] = v[o:o + a.size].reshape(a.shape, order="F").copy()
                o += a.size

    def _forward(self, sigma):
        x = np.atleast_2d(sigma).astype(np.complex128)
        xs, ths = [], []
        for l, ps in zip(self.layers, self.params):
            xs.append(x)
            if l[0] == "dense":
                th = x @ ps[0].T + ps[1][None, :]
                ths.append(th)
                x = act(l[3], th)
            elif l[0] == "wsum":
                ths.append(None)
                return x @ ps[0], xs, ths
            else:
                ths.append(None)
                return x.sum(axis=1), xs, ths
        raise ValueError("the chain must end with wsum or sum")

    def logpsi(self, sigma):
        return self._forward(sigma)[0]

    def logpsi_and_grad(self, sigma):
        out, xs, ths = self._forward(sigma)
        B = out.shape[0]
        grads = [None] * len(self.layers)
        last = len(self.layers) - 1
        if self.layers[last][0] == "wsum":
            grads[last] = [xs[last]]
            d = np.repeat(self.params[last][0][None, :], B, axis=0)
        else:
            grads[last] = []
            d = np.ones_like(xs[last])
        for li in range(last - 1, -1, -1):
            l, ps = self.layers[li], self.params[li]
            dth = d * dact(l[3], ths[li])
            gW = (dth[:, :, None] * xs[li][:, None, :]).transpose(0, 2, 1).reshape(B, -1)
            grads[li] = [gW, dth]
            d = dth @ ps[0]
        grad = np.concatenate([g for gs in grads for g in gs], axis=1)
        return out, grad

    def log_prob(self, sigma):
        return 2.0 * np.real(self.logpsi(sigma))


def init_random_pars(net, rng, sigma=1e-4):
    """``init_random_pars!`` (src/utils/rng.jl:27-38): randn * sqrt(sigma);
    complex randn has variance 1/2 per part (Julia convention)."""
    p = net.flat()
    if np.iscomplexobj(p):
        v = (rng.standard_normal(p.size) + 1j * rng.standard_normal(p.size)) / np.sqrt(2)
    else:
        v = rng.standard_normal(p.size)
    net.set_flat(v * np.sqrt(sigma))
    return net


class MixedChain:
    """``MixedStateAnsatz(Chain(DenseSplit(N, M, f), Dense..., sum | WSum), N)``
    (MixedDensityMatrix/MixedChainWrapper.jl:3-37, Layers/DenseSplit.jl:11):
    logρ(σ, η) is the chain's output with the first layer
    θ = Wr σ + Wc η + b.  That layer is a Dense layer on the concatenated
    (σ, η) with W = [Wr Wc], whose column-major storage is Wr then Wc, so the
    flat vector (Wr, Wc, b, later layers) is the ``Chain`` over 2N inputs
    with layers[0] = ("dense", 2N, M, f).  ``layers`` lists the DenseSplit as
    ("dense_split", N, M, f).

    ``("positive_def_r", N, M, f)`` opens the chain with PositiveDefR
    (Layers/PositiveDefR.jl:11-12): θ = Wr (σ + η) + i Wi (σ − η) + b, flat
    vector (Wr, Wi, b, later layers).  It is the Dense layer above with
    W = [Wr + i Wi, Wr − i Wi]; the gradient of PositiveDefRBatched.jl's
    backprop, ∇Wr = δθ (σ + η)ᵀ and ∇Wi = i δθ (σ − η)ᵀ, is
    ∇Wr = ∇W_σ + ∇W_η and ∇Wi = i (∇W_σ − ∇W_η) of that Dense layer.  Its
    parameters are real in the reference, so SR takes S and F real
    (``real_sr``; SRDirect.jl:11-38)."""

    def __init__(self, n, layers):
        self.N = int(n)
        first = layers[0]
        assert first[0] in ("dense_split", "positive_def_r") and first[1] == self.N
        self.pdr = first[0] == "positive_def_r"
        self.real_sr = self.pdr
        self.chain = Chain(2 * self.N, [("dense", 2 * self.N, first[2], first[3])] + list(layers[1:]))
        self._v = self.chain.flat()

    @property
    def n_params(self):
        return self.chain.n_params

    def flat(self):
        return self._v.copy() if self.pdr else self.chain.flat()

    def set_flat(self, v):
        v = np.asarray(v).astype(np.complex128)
        self._v = v.copy()
        if self.pdr:
            nw = self.chain.params[0][0].size // 2         # Wr (M x N) of W = [W_σ W_η]
            v = v.copy()
            wr, wi = self._v[:nw], self._v[nw:2 * nw]
            v[:nw], v[nw:2 * nw] = wr + 1j * wi, wr - 1j * wi
        self.chain.set_flat(v)

    def dense_split(self):
        """(Wr, Wc, b) of the first layer."""
        W, b = self.chain.params[0]
        return W[:, :self.N], W[:, self.N:], b

    def logpsi(self, sr, sc):
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        return self.chain.logpsi(np.concatenate([sr, sc], axis=1))

    def logpsi_and_grad(self, sr, sc):
        sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
        out, g = self.chain.logpsi_and_grad(np.concatenate([sr, sc], axis=1))
        if self.pdr:
            nw = self.chain.params[0][0].size // 2         # Wr (M x N) of W = [W_σ W_η]
            gs, ge = g[:, :nw].copy(), g[:, nw:2 * nw].copy()
            g[:, :nw], g[:, nw:2 * nw] = gs + ge, 1j * (gs - ge)
        return out, g

    def log_prob(self, sr, sc):
        return 2.0 * np.real(self.logpsi(sr, sc))
