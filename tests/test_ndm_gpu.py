"""GPU parity of the NDM (purified density matrix) + Liouvillian path against
the FP64 oracle, through the C-ABI.

Tolerances: logρ, ∇logρ, L_loc: relative 2e-5 (FP32 evaluation) / 1e-10
(FP64); sampler configurations bit-exact against the Philox replay (near-ties
|log u - Δ| < 1e-6 follow the device); F: 1e-4; S: 1e-4 (FP32 S); Δw: 1e-9
against the FP64 solve of the engine's own S and F, 2e-3 against the
oracle's Δw (adds the S error).
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


def make(N=4, ah=1, aa=2, act=nq.af_softplus, B=64, L=4, burn=5, passes=None, sigma=0.1 ** 2, seed=3,
         prec=nq._lib.NQ_EVAL_F32, sp=nq._lib.NQ_S_F32, kind="fock"):
    hilb = nq.HomogeneousFock(N) if kind == "fock" else nq.HomogeneousSpin(N)
    net = nq.NDM(np.float64, N, ah, aa, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    lv = dissipative(hilb, N)
    smp = nq.MetropolisSampler(nq.LocalRule(), L, passes or 2 * N, burn=burn, seed=seed + 100)
    is_ = nq.BatchedSampler(net, smp, lv, nq.SR(eps=0.01), batch_sz=B, eval_precision=prec, s_precision=sp)
    ohilb = Hilbert(N, FOCK if kind == "fock" else SPIN)
    onet = onw.NDM(N, ah, aa, onw.SOFTPLUS if act == nq.af_softplus else onw.LOGCOSH)
    onet.set_flat(net.flat())
    oH, oL = oex.dissipative_ising(ohilb, 1.0, 2.0)
    olv = oops.liouvillian(oH, oL)
    return is_, net, onet, olv, ohilb


@pytest.mark.parametrize("act", [nq.af_softplus, nq.af_logcosh])
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_ndm_logrho_and_grad(nqlib, act, prec, tol):
    N = 4
    is_, net, onet, _, _ = make(N=N, act=act, prec=prec, sigma=0.3 ** 2)
    rng = np.random.default_rng(1)
    sig = rng.integers(0, 2, size=(300, 2 * N)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig[:, :N].astype(float), sig[:, N:].astype(float))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tol
    assert rel(g, og) < tol


def test_ndm_doubled_sampler_bitexact(nqlib):
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
def test_liouvillian_estimator_force_S_solve(nqlib, prec):
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
    assert rel(force, np.real(F)) < 1e-4
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=True)
    assert rel(is_.engine.sr_matrix(), S) < 1e-4
    dw = is_.engine.precondition(0, 0.01)
    dwo = osr.precondition(S, F, 0.01, real_params=True)
    assert rel(dw, dwo) < 2e-3
    Sg = is_.engine.sr_matrix()
    assert rel(dw, np.linalg.solve(Sg + 0.01 * np.eye(Sg.shape[0]), force)) < 1e-9
    p0 = is_.engine.get_params()
    is_.engine.update_descent(0.01)
    np.testing.assert_allclose(is_.engine.get_params(), p0 - 0.01 * dw, rtol=0, atol=1e-12)


def test_ndm_chi_square_against_exact(nqlib):
    from scipy.stats import chisquare
    N = 3
    is_, net, onet, _, ohilb = make(N=N, ah=1, aa=1, B=16384, L=1, burn=30, passes=2 * N + 1,
                                    sigma=0.4 ** 2, seed=9)
    samples, _ = is_.engine.sample(0)
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    idx = ohilb.index_of_state(flat[:, N:]) * ohilb.dim + ohilb.index_of_state(flat[:, :N])
    counts = np.bincount(idx, minlength=ohilb.dim ** 2)
    p = oex.doubled_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval >= 0.01, (stat, pval)


def test_ndm_tf32_gram_and_graph_step(nqlib):
    """3xTF32 S on the centred NDM gradients, and the captured whole step."""
    N, B, L = 5, 256, 4
    a, net, onet, olv, ohilb = make(N=N, B=B, L=L, burn=5, sp=nq._lib.NQ_S_TF32X3, sigma=0.2 ** 2)
    samples, _ = a.engine.sample(1)
    a.engine.estimate()
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    _, O = onet.logpsi_and_grad(flat[:, :N], flat[:, N:])
    Oc, _ = oest.center(O)
    assert rel(a.engine.sr_matrix(), osr.build_S(Oc, real_params=True)) < 3e-5
    costs = [a.step(lr=0.02, eps=0.01).mean for _ in range(3)]
    assert all(np.isfinite(costs))
