"""Masked autoregressive proposal network (test infrastructure, see
``oracle/__init__``).  The reference has no learned proposal; this is the
FP64 definition the GPU kernels are checked against.

MADE (Germain et al., ICML 2015) with two ReLU hidden layers:
  input degrees i = 1..N, hidden degrees m(k) = 1 + (k mod (N-1)),
  W1[k,i] allowed iff m1(k) >= i, W2[k',k] iff m2(k') >= m1(k),
  W3[i,k'] iff i > m2(k');  logits l = W3 relu(W2 relu(W1 x + b1) + b2) + b3,
  q(x) = Π_i σ(l_i)^{x_i} σ(-l_i)^{1-x_i}, x_i ∈ {0,1} the local index of
  site i (spin: (1+s)/2; Fock: the value).
Ancestral sampling draws x_i = [u_i < σ(l_i)] with u_i from the Philox
stream TAG_AR at counter (k*N + i) // 4 of chain c (see ``sample_bits``).
"""
import numpy as np

from . import philox
from .hilbert import SPIN


def degrees(N, H):
    return 1 + (np.arange(H) % max(N - 1, 1))


def masks(N, H):
    din = np.arange(1, N + 1)
    m1 = degrees(N, H)
    m2 = degrees(N, H)
    M1 = (m1[:, None] >= din[None, :]).astype(np.float64)
    M2 = (m2[:, None] >= m1[None, :]).astype(np.float64)
    M3 = (din[:, None] > m2[None, :]).astype(np.float64)
    return M1, M2, M3


class MADE:
    def __init__(self, N, H=128, rng=None, scale=None):
        self.N, self.H = N, H
        self.M1, self.M2, self.M3 = masks(N, H)
        rng = np.random.default_rng(0) if rng is None else rng
        s1 = scale or 1.0 / np.sqrt(N)
        s2 = scale or 1.0 / np.sqrt(H)
        self.W1 = rng.standard_normal((H, N)) * s1 * self.M1
        self.b1 = np.zeros(H)
        self.W2 = rng.standard_normal((H, H)) * s2 * self.M2
        self.b2 = np.zeros(H)
        self.W3 = rng.standard_normal((N, H)) * s2 * self.M3
        self.b3 = np.zeros(N)

    FIELDS = ("W1", "b1", "W2", "b2", "W3", "b3")

    def flat(self):
        return np.concatenate([getattr(self, f).reshape(-1) for f in self.FIELDS])

    def set_flat(self, v):
        o = 0
        for f in self.FIELDS:
            a = getattr(self, f)
            setattr(self, f, np.asarray(v[o:o + a.size], dtype=np.float64).reshape(a.shape))
            o += a.size

    def forward(self, x):
        """x (B, N) in {0,1} -> logits (B, N) and the intermediates."""
        h1 = x @ (self.W1 * self.M1).T + self.b1
        a1 = np.maximum(h1, 0)
        h2 = a1 @ (self.W2 * self.M2).T + self.b2
        a2 = np.maximum(h2, 0)
        l = a2 @ (self.W3 * self.M3).T + self.b3
        return l, (h1, a1, h2, a2)

    def logq(self, x):
        l, _ = self.forward(x)
        z = (2 * x - 1) * l
        return -np.sum(np.logaddexp(0, -z), axis=1)

    def nll_grad(self, x):
        """mean NLL over the batch and its gradient (flat, FIELDS order)."""
        B = x.shape[0]
        l, (h1, a1, h2, a2) = self.forward(x)
        z = (2 * x - 1) * l
        nll = np.mean(np.sum(np.logaddexp(0, -z), axis=1))
        d3 = (1.0 / (1.0 + np.exp(-l)) - x) / B          # d nll / d l
        gW3 = (d3.T @ a2) * self.M3
        gb3 = d3.sum(0)
        d2 = (d3 @ (self.W3 * self.M3)) * (h2 > 0)
        gW2 = (d2.T @ a1) * self.M2
        gb2 = d2.sum(0)
        d1 = (d2 @ (self.W2 * self.M2)) * (h1 > 0)
        gW1 = (d1.T @ x) * self.M1
        gb1 = d1.sum(0)
        return nll, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])

    def sample_with_uniforms(self, u):
        """Ancestral sampling with given uniforms u (B, N)."""
        B = u.shape[0]
        x = np.zeros((B, self.N))
        for i in range(self.N):
            l, _ = self.forward(x)
            x[:, i] = (u[:, i] < 1.0 / (1.0 + np.exp(-l[:, i]))).astype(np.float64)
        return x


def ar_uniforms(seed, call, chains, slot, N):
    """Uniforms of AR proposal `slot` of every chain: word q = slot*N + i of the
    Philox stream TAG_AR, block q // 4, lane q % 4; u = (w >> 8) * 2^-24."""
    k0, k1 = philox.split_seed(seed)
    chains = np.asarray(chains, dtype=np.uint64)
    q = np.uint64(slot) * np.uint64(N) + np.arange(N, dtype=np.uint64)
    r = philox.philox4x32_10((q // np.uint64(4))[None, :], np.uint64(call), chains[:, None],
                             philox.TAG_AR, k0, k1)
    r = np.stack(r, axis=-1)
    sel = (q % np.uint64(4)).astype(np.int64)
    w = np.take_along_axis(r, sel[None, :, None].repeat(len(chains), 0), axis=2)[..., 0]
    return (w >> np.uint32(8)).astype(np.float64) * 2.0 ** -24


def mix_is_ar(seed, call, chains, step, p_ar):
    """Move-type choice of Metropolis step `step`: AR proposal iff the
    TAG_MIX word is below p_ar * 2^32."""
    k0, k1 = philox.split_seed(seed)
    r0, _, _, _ = philox.philox4x32_10(np.uint64(step), np.uint64(call),
                                       np.asarray(chains, dtype=np.uint64), philox.TAG_MIX, k0, k1)
    return r0.astype(np.float64) < p_ar * 4294967296.0


def to_bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as
    float64: the inference copy the GPU kernels read."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + np.uint64(0x7FFF) + ((u >> np.uint64(16)) & np.uint64(1))) & np.uint64(0xFFFF0000)
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def inference_copy(made):
    """MADE whose weights are the BF16-rounded float32 weights and whose
    biases are the float32 biases (the GPU's proposal / log q network)."""
    m = MADE(made.N, made.H)
    m.W1 = to_bf16(made.W1 * made.M1)
    m.W2 = to_bf16(made.W2 * made.M2)
    m.W3 = to_bf16(made.W3 * made.M3)
    m.b1 = np.asarray(made.b1, np.float32).astype(np.float64)
    m.b2 = np.asarray(made.b2, np.float32).astype(np.float64)
    m.b3 = np.asarray(made.b3, np.float32).astype(np.float64)
    return m


def bits_to_x(bits, N):
    bits = np.asarray(bits, dtype=np.uint64)
    return ((bits[..., None] >> np.arange(N, dtype=np.uint64)) & np.uint64(1)).astype(np.float64)


def x_to_bits(x):
    x = np.asarray(x).astype(np.uint64)
    return np.sum(x << np.arange(x.shape[-1], dtype=np.uint64), axis=-1, dtype=np.uint64)


def run_mixture(log_prob, hilb, made, p_ar, n_chains, chain_length, burn, passes, seed, call=0,
                gpu_accept_bits=None, tie_tol=1e-3):
    """Replays one call of the mixture Metropolis sampler.

    Step t of chain c is an AR move iff ``mix_is_ar``; otherwise it is the
    local flip of ``oracle.sampler.run``.  Both use the step's TAG_MH uniform
    u.  The chain's k-th AR move proposes x' from slot k (``ar_uniforms``) and
    accepts iff u < exp(lp(x') - lp(x) + log q(x) - log q(x')); lp = 2 Re
    log psi.  ``made`` must be the inference copy (BF16 weights).  Near-ties
    are resolved with ``gpu_accept_bits`` as in ``oracle.sampler.run``.
    Returns (samples (L, B, N) site values, info)."""
    from . import sampler as osm
    N = hilb.n_sites
    chains = np.arange(n_chains)
    passes = osm.fix_passes(passes)
    T = passes * (burn + chain_length)
    is_ar = np.stack([mix_is_ar(seed, call, chains, t, p_ar) for t in range(T)])     # (T, B)
    n_slots = int(is_ar.sum(0).max()) if T else 0
    if n_slots:
        u = np.stack([ar_uniforms(seed, call, chains, k, N) for k in range(n_slots)], 1)   # (B, S, N)
        xp = made.sample_with_uniforms(u.reshape(-1, N)).reshape(n_chains, n_slots, N)
        lqp = made.logq(xp.reshape(-1, N)).reshape(n_chains, n_slots)
    sigma = osm.init_configs(hilb, seed, call, chains, N)
    lp = log_prob(sigma)
    to_x = (lambda s: (s + 1) / 2) if hilb.kind == SPIN else (lambda s: s)
    from_x = (lambda x: 2 * x - 1) if hilb.kind == SPIN else (lambda x: x)
    samples = np.empty((chain_length, n_chains, N))
    slot = np.zeros(n_chains, dtype=np.int64)
    info = {"ambiguous": 0, "mismatch": 0, "accepted": 0, "steps": 0, "ar": 0, "ar_accepted": 0}
    rows = np.arange(n_chains)
    t = 0
    for sweep in range(burn + chain_length):
        for _ in range(passes):
            site, u = philox.mh_draws(seed, call, chains, t, N)
            ar = is_ar[t]
            new = sigma.copy()
            new[rows, site] = hilb.flip(sigma[rows, site])
            lq_new = np.zeros(n_chains)
            lq_cur = np.zeros(n_chains)
            if ar.any():
                k = np.minimum(slot, max(n_slots - 1, 0))
                new[ar] = from_x(xp[rows[ar], k[ar]])
                lq_new[ar] = lqp[rows[ar], k[ar]]
                lq_cur[ar] = made.logq(to_x(sigma[ar]))
            lpn = log_prob(new)
            delta = lpn - lp + lq_cur - lq_new
            with np.errstate(over="ignore", divide="ignore"):
                acc = u < np.exp(delta)
                logu = np.log(np.maximum(u, 1e-300))
            if gpu_accept_bits is not None:
                g = np.asarray(gpu_accept_bits[t], dtype=bool)
                amb = np.abs(logu - delta) < tie_tol
                info["ambiguous"] += int(np.sum(amb & (g != acc)))
                info["mismatch"] += int(np.sum(~amb & (g != acc)))
                acc = np.where(amb, g, acc)
            sigma = np.where(acc[:, None], new, sigma)
            lp = np.where(acc, lpn, lp)
            slot += ar
            info["accepted"] += int(acc.sum())
            info["ar"] += int(ar.sum())
            info["ar_accepted"] += int((acc & ar).sum())
            info["steps"] += n_chains
            t += 1
        k = sweep - burn
        if k >= 0:
            samples[k] = sigma
    return samples, info
