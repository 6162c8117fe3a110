"""Density-matrix observables (BatchedObsDMSampler, NQ_SPACE_DIAGONAL) on the
GPU against the oracle, through the C-ABI.

* the diagonal chains are the Metropolis replay of p(σ) ∝ ρ(σ,σ) on the N
  physical sites, bit-exact (near-ties |log u - Δ| < 1e-6 follow the
  device, none may disagree elsewhere);
* logρ(σ,σ) of N-site configurations (nq_logpsi on the diagonal handle):
  relative 2e-5 (FP32) / 1e-10 (FP64);
* O_loc(σ) = Σ O_σσ' ρ(σ',σ)/ρ(σ,σ) per sample: relative 2e-5 (FP32) /
  1e-10 (FP64) against the oracle on the device's own samples, and the
  Measurement against the oracle's stat_analysis of those values;
* the sampled means agree with the dense Tr(ρÔ)/Tr(ρ) within 5 error bars;
* exact sampling of the diagonal: χ² against ρ(σ,σ), p > 1e-3;
* the cost-function entry points refuse the diagonal handle, and the
  doubled-space handle refuses observables.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, \
    stats as ost, operators as oops
from oracle.hilbert import Hilbert, FOCK, SPIN

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


def dissipative(hilb, N, g=1.0, V=2.0, gamma=1.0):
    """examples/dissipative_ising1d.jl:17-31, open chain."""
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H = H + (g / 2) * nq.sigmax(hilb, i)
        Ls.append(float(np.sqrt(gamma)) * nq.sigmam(hilb, i))
    for i in range(1, N):
        H = H + (V / 4) * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    return nq.liouvillian(H, Ls)


def observables(hilb, ohilb, N):
    """(name, operator, oracle operator): Σσx, Σσz, σy σy and σz σz on a bond."""
    sx, osx = nq.LocalOperator(hilb), oops.OpSum(ohilb)
    sz, osz = nq.LocalOperator(hilb), oops.OpSum(ohilb)
    for i in range(1, N + 1):
        sx = sx + nq.sigmax(hilb, i)
        osx = osx + oops.sigmax(ohilb, i - 1)
        sz = sz + nq.sigmaz(hilb, i)
        osz = osz + oops.sigmaz(ohilb, i - 1)
    yy = nq.sigmay(hilb, 1) * nq.sigmay(hilb, 2)
    oyy = oops.OpSum(ohilb) + oops.prod(oops.sigmay(ohilb, 0), oops.sigmay(ohilb, 1))
    zz = nq.sigmaz(hilb, 2) * nq.sigmaz(hilb, N)
    ozz = oops.OpSum(ohilb) + oops.prod(oops.sigmaz(ohilb, 1), oops.sigmaz(ohilb, N - 1))
    return [("sx", sx, osx), ("sz", sz, osz), ("yy", yy, oyy), ("zz", zz, ozz)]


def make(N=4, ah=1, aa=2, act=nq.af_softplus, B=64, L=4, burn=5, passes=None, sigma=0.3 ** 2, seed=3,
         prec=nq._lib.NQ_EVAL_F32, kind="fock", exact=False, quirks=False):
    hilb = nq.HomogeneousFock(N) if kind == "fock" else nq.HomogeneousSpin(N)
    net = nq.NDM(np.float64, N, ah, aa, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    lv = dissipative(hilb, N)
    if exact:
        smp = nq.ExactSampler(L, seed=seed + 100)
    else:
        smp = nq.MetropolisSampler(nq.LocalRule(), L, passes or N, burn=burn, seed=seed + 100)
    obs = nq.BatchedObsDMSampler(net, smp, lv.hilb, batch_sz=B, eval_precision=prec, reference_quirks=quirks)
    ohilb = Hilbert(N, FOCK if kind == "fock" else SPIN)
    onet = onw.NDM(N, ah, aa, onw.SOFTPLUS if act == nq.af_softplus else onw.LOGCOSH)
    onet.set_flat(net.flat())
    return obs, hilb, net, onet, ohilb


@pytest.mark.parametrize("kind", ["fock", "spin"])
def test_diagonal_sampler_bitexact(nqlib, kind):
    N, B, L, burn = 5, 96, 4, 3
    obs, _, _, onet, ohilb = make(N=N, B=B, L=L, burn=burn, sigma=0.4 ** 2, kind=kind)
    eng = obs.engine
    assert eng.nsites == N
    lp = lambda x: np.real(onet.logpsi(x, x))
    for call in (0, 7):
        samples, bits = eng.sample(call, want_accept_bits=True)
        assert samples.shape == (L, B, N)
        ref, info = osm.run(lp, ohilb, B, L, burn, eng.passes, eng.cfg.seed, call=call,
                            gpu_accept_bits=bits)
        assert info["mismatch"] == 0
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


def test_diagonal_sampler_stale_last_slot(nqlib):
    N, B, L, burn = 4, 32, 3, 2
    obs, _, _, onet, ohilb = make(N=N, B=B, L=L, burn=burn, quirks=True)
    eng = obs.engine
    lp = lambda x: np.real(onet.logpsi(x, x))
    samples, bits = eng.sample(0, want_accept_bits=True)
    assert np.all(samples[L - 1] == 0)                 # state() fill of the Fock space
    ref, info = osm.run(lp, ohilb, B, L, burn, eng.passes, eng.cfg.seed, call=0, stale_last_slot=True,
                        prev_samples=samples.astype(np.float64), gpu_accept_bits=bits)
    assert info["mismatch"] == 0
    np.testing.assert_array_equal(samples.astype(np.float64), ref)


@pytest.mark.parametrize("act", [nq.af_softplus, nq.af_logcosh])
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_diagonal_logrho(nqlib, act, prec, tol):
    N = 5
    obs, _, _, onet, _ = make(N=N, act=act, prec=prec)
    sig = np.random.default_rng(2).integers(0, 2, size=(200, N)).astype(np.int8)
    lp, g = obs.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig.astype(float), sig.astype(float))
    assert rel(lp, olp) < tol
    assert np.max(np.abs(lp.imag)) < tol * np.max(np.abs(olp))
    assert rel(g, og) < tol


@pytest.mark.parametrize("act", [nq.af_softplus, nq.af_logcosh])
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_dm_local_observables_against_oracle(nqlib, act, prec, tol):
    N, B, L = 5, 64, 6
    obs, hilb, _, onet, ohilb = make(N=N, B=B, L=L, burn=6, act=act, prec=prec, kind="spin")
    eng = obs.engine
    samples, _ = eng.sample(3)
    flat = samples.reshape(-1, N).astype(np.float64)
    for name, op, oop in observables(hilb, ohilb, N):
        m, loc = eng.observable(nq.op_table(op), want_loc=True)
        ref = oest.local_observable_dm(onet, oop, flat)
        assert rel(loc.reshape(-1), ref) < tol, name
        st = ost.stat_analysis(ref.reshape(L, B).T)
        scale = max(1.0, float(np.max(np.abs(ref))))
        assert abs(complex(m.mean_re, m.mean_im) - st["mean"]) < 10 * tol * scale, name
        assert abs(m.error - st["error"]) < 1e-4 * max(1.0, st["error"]), name


def test_dm_observables_match_dense_trace(nqlib):
    """compute_observables on fresh chains: each mean within 5 error bars of
    Tr(ρÔ)/Tr(ρ) from the dense density matrix."""
    N = 4
    obs, hilb, net, onet, ohilb = make(N=N, ah=1, aa=1, B=4096, L=8, burn=40, sigma=0.5 ** 2, seed=11,
                                       kind="spin")
    ops = observables(hilb, ohilb, N)
    for name, op, _ in ops:
        nq.add_observable_(obs, name, op)
    res = nq.compute_observables(obs)
    assert set(res) == {name for name, _, _ in ops}
    for name, _, oop in ops:
        ex = oex.dm_expectation(onet, oop)
        m = res[name]
        assert abs(ex.imag) < 1e-10
        assert abs(m.mean.real - ex.real) < 5 * m.error + 1e-6, (name, m.mean, m.error, ex)
        assert abs(m.mean.imag) < 5 * m.error + 1e-6, name


def test_dm_exact_sampler_chi_square(nqlib):
    from scipy.stats import chisquare
    N, B, L = 5, 512, 16
    obs, _, _, onet, ohilb = make(N=N, B=B, L=L, sigma=0.4 ** 2, exact=True)
    samples, _ = obs.engine.sample(0)
    idx = ohilb.index_of_state(samples.reshape(-1, N).astype(np.float64))
    counts = np.bincount(idx, minlength=ohilb.dim)
    p = oex.diagonal_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3, (stat, pval)


def test_dm_handles_refuse_the_other_path(nqlib):
    N = 4
    obs, hilb, net, _, _ = make(N=N)
    eng = obs.engine
    lv = dissipative(hilb, N)
    for call in (lambda: eng.set_operator(nq.op_table(lv)), lambda: eng.estimate(),
                 lambda: eng.vmc_step(0, 0.01, 0.01), lambda: eng.precondition(0, 0.01),
                 lambda: eng.update_descent(0.01)):
        with pytest.raises(nq._lib.NqError) as e:
            call()
        assert e.value.status == nq._lib.NQ_ERR_UNSUPPORTED
    smp = nq.MetropolisSampler(nq.LocalRule(), 2, N, burn=1, seed=1)
    is_ = nq.BatchedSampler(net, smp, lv, nq.SR(eps=0.01), batch_sz=16)
    is_.engine.sample(0)
    with pytest.raises(nq._lib.NqError) as e:
        is_.engine.observable(nq.op_table(nq.sigmax(hilb, 1)))
    assert e.value.status == nq._lib.NQ_ERR_UNSUPPORTED
