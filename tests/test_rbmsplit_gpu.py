"""RBMSplit density matrix (src/Networks/MixedDensityMatrix/RBMSplit.jl) on
the doubled-space path against the FP64 oracle, through the C-ABI.

Tolerances: logρ, ∇logρ, L_loc relative 2e-5 (FP32) / 1e-10 (FP64); the
doubled-space chains bit-exact against the Philox replay (near-ties
|log u - Δ| < 1e-6 follow the device); F 1e-4; S 1e-4 (FP32 S, complex
parameters: S = conj(O_c O_c†)/Ns, SRDirect.jl:38-44); Δw 2e-3; the
diagonal observables as for the NDM (2e-5 FP32 per sample, dense trace
within 5 error bars).
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, \
    sr as osr, stats as ost, operators as oops
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


def make(N=4, alpha=2, act=nq.af_logcosh, B=64, L=4, burn=5, sigma=0.1 ** 2, seed=3,
         prec=nq._lib.NQ_EVAL_F32, sp=nq._lib.NQ_S_F32, kind="fock"):
    hilb = nq.HomogeneousFock(N) if kind == "fock" else nq.HomogeneousSpin(N)
    net = nq.RBMSplit(np.complex64, N, alpha, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    lv = dissipative(hilb, N)
    smp = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=burn, seed=seed + 100)
    is_ = nq.BatchedSampler(net, smp, lv, nq.SR(eps=0.01), batch_sz=B, eval_precision=prec, s_precision=sp)
    ohilb = Hilbert(N, FOCK if kind == "fock" else SPIN)
    onet = onw.RBMSplit(N, net.M, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    oH, oL = oex.dissipative_ising(ohilb, 1.0, 2.0)
    olv = oops.liouvillian(oH, oL)
    return is_, net, onet, olv, ohilb


@pytest.mark.parametrize("act", [nq.af_logcosh, nq.af_softplus])
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_rbmsplit_logrho_and_grad(nqlib, act, prec, tol):
    N = 4
    is_, net, onet, _, _ = make(N=N, act=act, prec=prec, sigma=0.3 ** 2)
    assert is_.engine.P == 2 * N + net.M + 2 * net.M * N
    sig = np.random.default_rng(1).integers(0, 2, size=(300, 2 * N)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig[:, :N].astype(float), sig[:, N:].astype(float))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tol
    assert rel(g, og) < tol


def test_rbmsplit_doubled_sampler_bitexact(nqlib):
    N, B, L, burn = 5, 96, 4, 3
    is_, net, onet, _, ohilb = make(N=N, B=B, L=L, burn=burn, sigma=0.4 ** 2)
    lp = lambda x: onet.log_prob(x[:, :N], x[:, N:])
    for call in (0, 7):
        samples, bits = is_.engine.sample(call, want_accept_bits=True)
        ref, info = osm.run(lp, ohilb, B, L, burn, is_.engine.passes, is_.engine.cfg.seed, call=call,
                            doubled=True, gpu_accept_bits=bits)
        assert info["mismatch"] == 0
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


@pytest.mark.parametrize("prec", [nq._lib.NQ_EVAL_F32, nq._lib.NQ_EVAL_F64])
def test_rbmsplit_liouvillian_estimator_force_S_solve(nqlib, prec):
    N, B, L = 4, 48, 5
    is_, net, onet, olv, ohilb = make(N=N, B=B, L=L, burn=8, sigma=0.2 ** 2, prec=prec)
    samples, _ = is_.engine.sample(2)
    m, loc, force = is_.engine.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    sr, sc = flat[:, :N], flat[:, N:]
    Lo, dL = oest.local_liouvillian(onet, olv, sr, sc)
    assert rel(loc.reshape(-1), Lo) < 2e-5
    _, O = onet.logpsi_and_grad(sr, sc)
    C, F = oest.force_liouvillian(Lo, dL, O)
    st = ost.stat_analysis((np.abs(Lo) ** 2).reshape(L, B).T)
    assert abs(m.mean_re - st["mean"]) < 1e-5 * max(1.0, st["mean"])
    assert abs(m.error - st["error"]) < 1e-4 * max(1.0, st["error"])
    assert rel(force, F) < 1e-4
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=False)
    assert rel(is_.engine.sr_matrix(), S) < 1e-4
    dw = is_.engine.precondition(0, 0.01)
    dwo = osr.precondition(S, F, 0.01, real_params=False)
    assert rel(dw, dwo) < 2e-3
    p0 = is_.engine.get_params()
    is_.engine.update_descent(0.01)
    np.testing.assert_allclose(is_.engine.get_params(), p0 - 0.01 * dw, rtol=0, atol=1e-12)


def test_rbmsplit_chi_square_against_exact(nqlib):
    from scipy.stats import chisquare
    N = 3
    is_, net, onet, _, ohilb = make(N=N, alpha=1, B=16384, L=1, burn=30, sigma=0.4 ** 2, seed=9)
    samples, _ = is_.engine.sample(0)
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    idx = ohilb.index_of_state(flat[:, N:]) * ohilb.dim + ohilb.index_of_state(flat[:, :N])
    counts = np.bincount(idx, minlength=ohilb.dim ** 2)
    p = oex.doubled_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval >= 1e-3, (stat, pval)


@pytest.mark.parametrize("sp", [nq._lib.NQ_S_F32, nq._lib.NQ_S_TF32X3])
def test_rbmsplit_steady_state_cost_decreases(nqlib, sp):
    """The captured whole step on the dissipative Ising chain lowers the
    Liouvillian cost mean |L_loc|²."""
    N = 4
    is_, net, _, _, _ = make(N=N, B=512, L=8, burn=10, sigma=0.05 ** 2, seed=4, sp=sp)
    costs = [is_.step(0.01).mean]
    for _ in range(60):
        costs.append(is_.step(0.01).mean)
    assert np.all(np.isfinite(costs))
    assert np.mean(costs[-5:]) < 0.9 * np.mean(costs[:5]), costs


def test_rbmsplit_diagonal_observables(nqlib):
    """BatchedObsDMSampler with an RBMSplit: per-sample O_loc against the
    oracle, and Σσx / σzσz means within 5 error bars of the exact mean of
    O_loc under p(σ) ∝ exp(Re logρ(σ,σ)).  (RBMSplit's ρ need not be
    Hermitian, so that mean is Tr(ρÔ)/Tr(ρ) only when ρ(σ,σ) > 0.)"""
    N = 4
    hilb = nq.HomogeneousSpin(N)
    ohilb = Hilbert(N, SPIN)
    net = nq.RBMSplit(np.complex64, N, 1, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.3 ** 2, rng=np.random.default_rng(21))
    onet = onw.RBMSplit(N, net.M, onw.LOGCOSH)
    onet.set_flat(net.flat())
    lv = dissipative(hilb, N)
    smp = nq.MetropolisSampler(nq.LocalRule(), 8, N, burn=40, seed=5)
    obs = nq.BatchedObsDMSampler(net, smp, lv.hilb, batch_sz=4096)
    sx, osx = nq.LocalOperator(hilb), oops.OpSum(ohilb)
    for i in range(1, N + 1):
        sx = sx + nq.sigmax(hilb, i)
        osx = osx + oops.sigmax(ohilb, i - 1)
    zz = nq.sigmaz(hilb, 1) * nq.sigmaz(hilb, 3)
    ozz = oops.OpSum(ohilb) + oops.prod(oops.sigmaz(ohilb, 0), oops.sigmaz(ohilb, 2))
    samples, _ = obs.engine.sample(0)
    flat = samples.reshape(-1, N).astype(np.float64)
    lp = obs.engine.logpsi(samples.reshape(-1, N)[:64])
    d = lp - onet.logpsi(flat[:64], flat[:64])
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) < 2e-5 * max(1.0, float(np.max(np.abs(lp))))
    p = oex.diagonal_distribution(onet, ohilb)
    st = ohilb.all_states()
    for op, oop in ((sx, osx), (zz, ozz)):
        m, loc = obs.engine.observable(nq.op_table(op), want_loc=True)
        ref = oest.local_observable_dm(onet, oop, flat)
        assert rel(loc.reshape(-1), ref) < 2e-5
        ex = np.sum(p * oest.local_observable_dm(onet, oop, st))
        mean = complex(m.mean_re, m.mean_im)
        assert abs(mean - ex) < 5 * m.error + 1e-6, (mean, m.error, ex)
