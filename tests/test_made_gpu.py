"""GPU parity of the learned autoregressive proposal (MADE) and of the mixture
sampler against the FP64 oracle (oracle/made.py), through the C-ABI.

Tolerances:
* log q against the oracle evaluated with the same BF16-rounded weights:
  absolute 2e-4 (FP32 accumulation over N*H + H*H + N*H terms).
* proposals: identical bit strings except draws within FP32 rounding of the
  Bernoulli threshold (at most 1 in 10^4 proposals).
* NLL gradient (FP32 master, FP32 forward/backward): relative 1e-4 of max.
* mixture sampler: accept decisions identical to the replay except near-ties
  |log u - Δ| < 1e-3; chains that met no such tie end in the same state.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import made as omade, networks as onw, exact as oex, sampler as osm
from oracle.hilbert import Hilbert, SPIN

pytestmark = pytest.mark.gpu


def make(N=8, alpha=2, B=128, L=6, burn=4, sigma=0.3 ** 2, seed=5, p_ar=0.5, passes=None):
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, alpha, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    s = nq.MetropolisSampler(nq.LocalRule(), L, passes or N, burn=burn, seed=seed * 13 + 3)
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B)
    eng = is_.engine
    eng.proposal_init(hidden=128, p_ar=p_ar, seed=seed)
    onet = onw.RBM(N, net.M, onw.LOGCOSH)
    onet.set_flat(net.flat())
    return is_, eng, onet, Hilbert(N, SPIN)


def random_made(N, seed, bias=0.3):
    m = omade.MADE(N, 128, rng=np.random.default_rng(seed))
    rng = np.random.default_rng(seed + 1)
    m.b1 = rng.standard_normal(128) * bias
    m.b2 = rng.standard_normal(128) * bias
    m.b3 = rng.standard_normal(N) * bias
    m.set_flat(m.flat().astype(np.float32).astype(np.float64))
    return m


def test_made_logq_parity(nqlib):
    N = 10
    _, eng, _, _ = make(N=N)
    m = random_made(N, 21)
    eng.proposal_set_params(m.flat())
    back = eng.proposal_get_params().astype(np.float64)
    assert np.array_equal(back, m.flat())            # master is stored as given (already masked)
    rng = np.random.default_rng(4)
    bits = rng.integers(0, 2 ** N, size=3000, dtype=np.uint64)
    lq = eng.proposal_logq(bits).astype(np.float64)
    ref = omade.inference_copy(m).logq(omade.bits_to_x(bits, N))
    assert np.max(np.abs(lq - ref)) < 2e-4
    # and q is normalised over the whole space
    allb = np.arange(2 ** N, dtype=np.uint64)
    assert abs(np.sum(np.exp(eng.proposal_logq(allb).astype(np.float64))) - 1.0) < 1e-3


def test_made_masked_entries_are_dropped(nqlib):
    N = 6
    _, eng, _, _ = make(N=N)
    m = random_made(N, 3)
    dense = m.flat() + 0.5                           # every masked entry now non-zero
    eng.proposal_set_params(dense)
    M1, M2, M3 = omade.masks(N, 128)
    mask = np.concatenate([M1.ravel(), np.ones(128), M2.ravel(), np.ones(128), M3.ravel(), np.ones(N)])
    np.testing.assert_array_equal(eng.proposal_get_params(), (dense * mask).astype(np.float32))


def test_made_proposals_replay(nqlib):
    N, B, S = 12, 64, 24
    _, eng, _, _ = make(N=N, B=B)
    m = random_made(N, 8)
    eng.proposal_set_params(m.flat())
    mi = omade.inference_copy(m)
    for call in (0, 7):
        x, lq = eng.proposal_sample(call, S)
        u = np.stack([omade.ar_uniforms(eng.cfg.seed, call, np.arange(B), k, N) for k in range(S)], 1)
        ref_x = mi.sample_with_uniforms(u.reshape(-1, N))
        ref_bits = omade.x_to_bits(ref_x).reshape(B, S)
        same = x == ref_bits
        assert np.mean(~same) <= 1e-4 + 1.0 / same.size
        ref_lq = mi.logq(omade.bits_to_x(x.reshape(-1), N)).reshape(B, S)
        assert np.max(np.abs(lq - ref_lq)) < 2e-4


def test_made_nll_gradient(nqlib):
    N = 9
    _, eng, _, _ = make(N=N)
    m = random_made(N, 12)
    eng.proposal_set_params(m.flat())
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2 ** N, size=777, dtype=np.uint64)
    g, nll = eng.proposal_grad(bits)
    ref_nll, ref_g = m.nll_grad(omade.bits_to_x(bits, N))
    assert np.max(np.abs(g - ref_g)) / np.max(np.abs(ref_g)) < 1e-4
    assert abs(nll - ref_nll) < 1e-3 * max(1.0, abs(ref_nll))


def test_made_training_lowers_nll(nqlib):
    N, B, L = 8, 512, 8
    is_, eng, _, _ = make(N=N, B=B, L=L, p_ar=0.0)
    eng.sample(0, want_samples=False)
    samples, _ = eng.sample(1)
    x = ((samples.reshape(-1, N) + 1) // 2).astype(np.int64)
    bits = omade.x_to_bits(x)
    _, nll0 = eng.proposal_grad(bits)
    nll1 = eng.proposal_train(steps=200, batch=1024, lr=3e-3)
    assert nll1 < nll0 - 0.2
    # the entropy of the data bounds the NLL from below (empirical distribution)
    _, counts = np.unique(bits, return_counts=True)
    p = counts / counts.sum()
    assert nll1 > -np.sum(p * np.log(p)) - 0.05


@pytest.mark.parametrize("p_ar", [0.5, 1.0])
def test_mixture_sampler_replay(nqlib, p_ar):
    N, B, L, burn = 8, 96, 5, 3
    is_, eng, onet, ohilb = make(N=N, B=B, L=L, burn=burn, p_ar=p_ar)
    m = random_made(N, 31)
    eng.proposal_set_params(m.flat())
    for call in (0, 3):
        samples, bits = eng.sample(call, want_accept_bits=True)
        ref, info = omade.run_mixture(onet.log_prob, ohilb, omade.inference_copy(m), p_ar, B, L, burn,
                                      eng.passes, eng.cfg.seed, call=call, gpu_accept_bits=bits)
        assert info["mismatch"] == 0
        assert info["ambiguous"] <= max(3, info["steps"] // 10000)
        if info["ambiguous"] == 0:
            np.testing.assert_array_equal(samples, ref.astype(np.int8))
        n_ar, n_ar_acc = eng.proposal_stats()
        assert n_ar == info["ar"]
        assert abs(n_ar_acc - info["ar_accepted"]) <= info["ambiguous"]


def test_mixture_sampler_distribution(nqlib):
    """Chains of the mixture sampler (untrained q) reproduce |ψ|² (χ² test)."""
    N, B, L = 8, 2048, 40
    is_, eng, onet, ohilb = make(N=N, B=B, L=L, burn=10, p_ar=0.5, passes=3)
    m = random_made(N, 40)
    eng.proposal_set_params(m.flat())
    samples, _ = eng.sample(2)
    x = ((samples.reshape(-1, N) + 1) // 2).astype(np.int64)
    idx = omade.x_to_bits(x).astype(np.int64)
    counts = np.bincount(idx, minlength=2 ** N).astype(np.float64)
    allx = omade.bits_to_x(np.arange(2 ** N, dtype=np.uint64), N)
    lp = onet.log_prob(2 * allx - 1)
    p = np.exp(lp - lp.max())
    p /= p.sum()
    # samples are correlated along a chain: compare per-chain-thinned counts
    thin = samples[::4].reshape(-1, N)
    tidx = omade.x_to_bits(((thin + 1) // 2).astype(np.int64)).astype(np.int64)
    tc = np.bincount(tidx, minlength=2 ** N).astype(np.float64)
    n = tc.sum()
    keep = p * n >= 5
    chi2 = np.sum((tc[keep] - n * p[keep]) ** 2 / (n * p[keep]))
    dof = keep.sum() - 1
    assert chi2 < dof + 6 * np.sqrt(2 * dof)
    assert np.sum(counts) == B * L


def _ferro_engine(N, B, L, passes, seed=7):
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.05, rng=np.random.default_rng(seed))
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - 0.5 * nq.sigmax(hilb, i)
        H = H - nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    s = nq.MetropolisSampler(nq.LocalRule(), L, passes, burn=20, seed=seed)
    return nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B).engine


def test_trained_proposal_improves_mixing(nqlib):
    """Ordered ferromagnet (h = 0.5, J = -1): single flips almost never carry a
    chain from one magnetisation sector to the other.  A MADE trained on the
    chains' samples gives a high AR acceptance and decorrelates the signed
    magnetisation Σσz within a few steps; the mixture with the untrained
    network and local flips alone do not."""
    from nqcuda.stats import integrated_autocorr_time
    N, B = 16, 1024
    train = _ferro_engine(N, B, 16, N)
    for it in range(150):
        train.vmc_step(it, 0.01, 0.05)
    flat = train.get_params()
    samples, _ = train.sample(1000)
    train.proposal_init(128, 0.0, 3)
    nll_untrained = train.proposal_grad(omade.x_to_bits(((samples.reshape(-1, N) + 1) // 2).astype(np.int64)))[1]
    nll = train.proposal_train(400, 2048, 3e-3)
    trained = train.proposal_get_params()
    assert nll < nll_untrained - 1.0

    def run(params, p_ar):
        eng = _ferro_engine(N, B, 64, 1)
        eng.set_params(flat)
        if params is not None:
            eng.proposal_init(128, 0.0, 3)
            if params is not False:
                eng.proposal_set_params(params)
            eng.proposal_set_mix(p_ar)
        smp, _ = eng.sample(2000)
        m = smp.sum(axis=2).astype(np.float64).T          # (chains, steps)
        acc = eng.proposal_stats() if params is not None else (0, 0)
        return integrated_autocorr_time(m), acc[1] / max(acc[0], 1)

    tau_local, _ = run(None, 0.0)
    tau_untrained, acc_untrained = run(False, 0.5)
    tau_trained, acc_trained = run(trained, 0.5)
    assert acc_trained > 0.3 and acc_trained > 2.0 * acc_untrained
    assert tau_trained < 0.5 * tau_local
    assert tau_trained < 0.5 * tau_untrained
