"""Philox4x32-10 counter-based RNG and the counter schema of the sampler.

Test infrastructure (see ``oracle/__init__``).  The reference draws from a
``MersenneTwister`` (src/utils/rng.jl:9-11); the GPU engine replaces it with
the counter-based Philox4x32-10 generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11), so that every draw is
addressable by (chain, call, step) and replayable here bit for bit.

Counter schema (identical in ``csrc/philox.cuh``):

* key   = (seed & 0xffffffff, seed >> 32)
* init  : word q of chain c in call n  -> philox((q // 4, n, c, TAG_INIT))[q % 4]
* MH    : step t of chain c in call n  -> r = philox((t, n, c, TAG_MH));
          site = (r0 * nsites) >> 32,  u = (r1 >> 8) * 2**-24
* exact : draw t of chain c in call n  -> r = philox((t, n, c, TAG_EXACT));
          u = ((r0 >> 5) * 2**26 + (r1 >> 6)) * 2**-53
"""
import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint64(0x9E3779B9)
W1 = np.uint64(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

TAG_INIT = 0
TAG_MH = 1
TAG_AR = 2      # learned autoregressive proposal draws
TAG_MIX = 3     # proposal-type selection of the mixture kernel
TAG_EXACT = 4   # exact-sampler draws


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10.  Inputs are integer arrays (broadcastable);
    returns four uint32 arrays."""
    c0 = np.asarray(c0, dtype=np.uint64) & MASK32
    c1 = np.asarray(c1, dtype=np.uint64) & MASK32
    c2 = np.asarray(c2, dtype=np.uint64) & MASK32
    c3 = np.asarray(c3, dtype=np.uint64) & MASK32
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    c0 = c0.copy(); c1 = c1.copy(); c2 = c2.copy(); c3 = c3.copy()
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        n0 = (hi1 ^ c1 ^ k0) & MASK32
        n1 = lo1
        n2 = (hi0 ^ c3 ^ k1) & MASK32
        n3 = lo0
        c0, c1, c2, c3 = n0, n1, n2, n3
        k0 = (k0 + W0) & MASK32
        k1 = (k1 + W1) & MASK32
    return (c0.astype(np.uint32), c1.astype(np.uint32),
            c2.astype(np.uint32), c3.astype(np.uint32))


def split_seed(seed):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return seed & 0xFFFFFFFF, seed >> 32


def init_words(seed, call, chains, nwords):
    """Random words used to initialise the configurations of ``chains``
    (array of chain ids) in sample call ``call``: shape (len(chains), nwords)."""
    k0, k1 = split_seed(seed)
    chains = np.asarray(chains, dtype=np.uint64)
    q = np.arange(nwords, dtype=np.uint64)
    blk = q // np.uint64(4)
    r = philox4x32_10(blk[None, :], np.uint64(call), chains[:, None], TAG_INIT, k0, k1)
    r = np.stack(r, axis=-1)  # (chains, nwords, 4)
    sel = (q % np.uint64(4)).astype(np.int64)
    return np.take_along_axis(r, sel[None, :, None].repeat(len(chains), 0), axis=2)[..., 0]


def mh_draws(seed, call, chains, step, nsites):
    """(site, u) of Metropolis step ``step`` for every chain in ``chains``.
    ``site`` is 0-based; ``u`` is exactly representable in float32."""
    k0, k1 = split_seed(seed)
    chains = np.asarray(chains, dtype=np.uint64)
    r0, r1, _, _ = philox4x32_10(np.uint64(step), np.uint64(call), chains, TAG_MH, k0, k1)
    site = ((r0.astype(np.uint64) * np.uint64(nsites)) >> np.uint64(32)).astype(np.int64)
    u = (r1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
    return site, u


def mh_raw(seed, call, chains, step):
    """(r0, u) of Metropolis step ``step``: the raw 32-bit word that picks the
    move (index floor(r0 n / 2^32) among n candidates) and the uniform."""
    k0, k1 = split_seed(seed)
    chains = np.asarray(chains, dtype=np.uint64)
    r0, r1, _, _ = philox4x32_10(np.uint64(step), np.uint64(call), chains, TAG_MH, k0, k1)
    u = (r1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
    return r0.astype(np.uint64), u


def exact_uniforms(seed, call, chains, t):
    """53-bit uniforms in [0, 1) of exact-sampler draw ``t`` for ``chains``."""
    k0, k1 = split_seed(seed)
    chains = np.asarray(chains, dtype=np.uint64)
    r0, r1, _, _ = philox4x32_10(np.uint64(t), np.uint64(call), chains, TAG_EXACT, k0, k1)
    a = (r0.astype(np.uint64) >> np.uint64(5)).astype(np.float64)
    b = (r1.astype(np.uint64) >> np.uint64(6)).astype(np.float64)
    return (a * 67108864.0 + b) / 9007199254740992.0
