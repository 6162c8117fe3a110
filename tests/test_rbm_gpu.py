"""GPU parity of the RBM path against the FP64 oracle, through the C-ABI.

Tolerances (stated per quantity):
* logψ, ∇logψ, E_loc in FP32 evaluation: relative 2e-5 (of max magnitude);
  FP64 evaluation: 1e-10.
* sampler: configurations bit-exact against the Philox replay; accept
  decisions identical except near-ties |log u - Δ| < 1e-6 (counted).
* F: relative 1e-4; S (FP32 accumulation): relative 1e-4 of max |S|;
  Δw against the FP64 solve of the engine's own S and F: relative 1e-9 (the
  solve itself); against the oracle's Δw: relative 2e-3 (adds the S error).
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, \
    sr as osr, stats as ost
from oracle.hilbert import Hilbert, SPIN, FOCK

pytestmark = pytest.mark.gpu


def tfim(hilb, N, h=1.0, J=1.0):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - h * nq.sigmax(hilb, i)
        H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


def make(N=6, alpha=2, act=nq.af_logcosh, kind="spin", B=64, L=4, burn=5, passes=None,
         sigma=0.04, seed=11, eval_precision=nq._lib.NQ_EVAL_F32, quirks=False, h=1.0):
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    net = nq.RBM(np.complex64, N, alpha, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    s = nq.MetropolisSampler(nq.LocalRule(), L, passes or N, burn=burn, seed=seed * 7 + 1)
    H = tfim(hilb, N, h=h)
    is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B, eval_precision=eval_precision,
                            reference_quirks=quirks)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    onet = onw.RBM(N, net.M, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    oH = oex.tfim_1d(ohilb, h, 1.0)
    return is_, net, onet, oH, ohilb


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


@pytest.mark.parametrize("act", [nq.af_logcosh, nq.af_softplus])
@pytest.mark.parametrize("kind", ["spin", "fock"])
@pytest.mark.parametrize("prec", [nq._lib.NQ_EVAL_F32, nq._lib.NQ_EVAL_F64])
def test_logpsi_and_grad_parity(nqlib, act, kind, prec):
    is_, net, onet, _, ohilb = make(act=act, kind=kind, sigma=0.2 ** 2, eval_precision=prec)
    rng = np.random.default_rng(3)
    vals = np.array([-1, 1] if kind == "spin" else [0, 1])
    sig = rng.choice(vals, size=(257, 6)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig.astype(np.float64))
    tol = 2e-5 if prec == nq._lib.NQ_EVAL_F32 else 1e-10
    # the imaginary part of logψ is defined modulo 2π
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tol
    assert rel(g, og) < tol


@pytest.mark.parametrize("quirks", [False, True])
@pytest.mark.parametrize("kind", ["spin", "fock"])
def test_sampler_bitexact_replay(nqlib, quirks, kind):
    N, B, L, burn = 8, 96, 5, 3
    is_, net, onet, _, ohilb = make(N=N, kind=kind, B=B, L=L, burn=burn, sigma=0.3 ** 2,
                                    quirks=quirks)
    for call in (0, 5):
        samples, bits = is_.engine.sample(call, want_accept_bits=True)
        ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, is_.engine.passes,
                            is_.engine.cfg.seed, call=call, stale_last_slot=quirks,
                            gpu_accept_bits=bits)
        assert info["mismatch"] == 0
        assert info["ambiguous"] <= 3
        if quirks:
            # slot L keeps the state() fill (local index 0 everywhere)
            fill = -1 if kind == "spin" else 0
            assert np.all(samples[L - 1] == fill)
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


def test_estimator_force_S_solve(nqlib):
    N, B, L = 6, 64, 6
    is_, net, onet, oH, ohilb = make(N=N, B=B, L=L, burn=10, sigma=0.1 ** 2)
    samples, _ = is_.engine.sample(1)
    m, loc, force = is_.engine.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, N).astype(np.float64)
    E = oest.local_energy(onet, oH, flat)
    assert rel(loc.reshape(-1), E) < 2e-5
    _, O = onet.logpsi_and_grad(flat)
    F = oest.force_ket(E, O)
    assert rel(force, F) < 1e-4
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=False)
    Sg = is_.engine.sr_matrix()
    assert rel(Sg, S) < 1e-4
    st = ost.stat_analysis(E.reshape(L, B).T)
    assert abs(complex(m.mean_re, m.mean_im) - st["mean"]) < 1e-5 * max(1, abs(st["mean"]))
    for k in ("error", "variance", "tau", "R"):
        assert abs(getattr(m, k) - st[k]) <= 1e-4 * max(1.0, abs(st[k])), k
    dw = is_.engine.precondition(0, 0.01)
    dwo = osr.precondition(S, F, 0.01)
    assert rel(dw, dwo) < 2e-3
    assert rel(dw, np.linalg.solve(Sg + 0.01 * np.eye(Sg.shape[0]), force)) < 1e-9
    p0 = is_.engine.get_params()
    is_.engine.update_descent(0.05)
    p1 = is_.engine.get_params()
    np.testing.assert_allclose(p1, p0 - 0.05 * dw, rtol=0, atol=1e-12)


def test_chi_square_against_exact(nqlib):
    from scipy.stats import chisquare
    N, B = 4, 16384
    is_, net, onet, _, ohilb = make(N=N, alpha=1, B=B, L=1, burn=30, passes=N + 1,
                                    sigma=0.2 ** 2, seed=123)
    samples, _ = is_.engine.sample(0)
    idx = ohilb.index_of_state(samples.reshape(-1, N).astype(np.float64))
    counts = np.bincount(idx, minlength=ohilb.dim)
    p = oex.ket_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval >= 0.01, (stat, pval)


def test_graph_step_matches_staged(nqlib):
    kw = dict(N=8, B=128, L=4, burn=5, sigma=0.05 ** 2, seed=5)
    a, net_a, *_ = make(**kw)
    b, net_b, *_ = make(**kw)
    for it in range(3):
        ma = a.engine.vmc_step(it, 0.01, 0.02)
        b.engine.sample(it, want_samples=False)
        mb, _, _ = b.engine.estimate()
        b.engine.precondition(0, 0.01)
        b.engine.update_descent(0.02)
        assert abs(ma.mean_re - mb.mean_re) < 1e-6 * max(1, abs(mb.mean_re))
    np.testing.assert_allclose(a.engine.get_params(), b.engine.get_params(), rtol=0, atol=1e-9)
    assert a.engine.kernel_launches() > 0


def test_vmc_converges_small_tfim(nqlib):
    """A short SR run lowers the energy towards the exact ground state."""
    N = 8
    is_, net, onet, oH, ohilb = make(N=N, alpha=2, B=512, L=8, burn=20, sigma=0.01 ** 2, seed=2)
    from oracle import operators as oops
    e0 = np.linalg.eigvalsh(oops.to_matrix(oH).real)[0]
    E = []
    for it in range(150):
        m = is_.step(lr=0.05, eps=0.01)
        E.append(m.mean.real)
    assert np.mean(E[-10:]) < e0 + 0.05 * abs(e0)


@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_sampler_every_lane_layout_replays_bitexact(nqlib, lanes):
    """All instantiated lanes-per-chain layouts (the autotuner's candidates)
    reproduce the Philox replay."""
    N, B, L, burn, M = 10, 64, 3, 2, 20
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.3 ** 2, rng=np.random.default_rng(4))
    eng = nq.Engine(net, hilb, B, L, burn, N, 31, sampler_lanes=lanes)
    eng.set_params(net.flat())
    samples, bits = eng.sample(1, want_accept_bits=True)
    onet = onw.RBM(N, M, onw.LOGCOSH)
    onet.set_flat(net.flat())
    ref, info = osm.run(onet.log_prob, Hilbert(N, SPIN), B, L, burn, eng.passes, 31, call=1,
                        gpu_accept_bits=bits)
    assert info["mismatch"] == 0
    np.testing.assert_array_equal(samples.astype(np.float64), ref)
    assert eng.tuning()["sampler_lanes"] == lanes


def test_observables_match_oracle(nqlib):
    """BatchedObsKetSampler: local values of Σσx, σyσy and a σz correlator on the
    current samples (estimator kernel with another operator table) against the
    FP64 oracle; an observable equal to H reproduces the energy estimate."""
    from oracle import operators as oops, estimators as oest2
    N, B, L = 6, 128, 5
    is_, net, onet, oH, ohilb = make(N=N, B=B, L=L, sigma=0.2 ** 2)
    hilb = nq.HomogeneousSpin(N)
    samples, _ = is_.engine.sample(4)
    mE, locE, _ = is_.engine.estimate(want_loc=True)
    flat = samples.reshape(-1, N).astype(np.float64)
    cases = []
    X = nq.LocalOperator(hilb)
    oX = oops.OpSum(ohilb)
    for i in range(1, N + 1):
        X = X + nq.sigmax(hilb, i)
        oX = oX + oops.sigmax(ohilb, i - 1)
    cases.append((X, oX))
    cases.append((nq.sigmay(hilb, 2) * nq.sigmay(hilb, 3),
                  oops.OpSum(ohilb) + oops.prod(oops.sigmay(ohilb, 1), oops.sigmay(ohilb, 2))))
    cases.append((nq.sigmaz(hilb, 1) * nq.sigmaz(hilb, 4),
                  oops.OpSum(ohilb) + oops.prod(oops.sigmaz(ohilb, 0), oops.sigmaz(ohilb, 3))))
    obs = nq.BatchedObsKetSampler(is_)
    for k, (op, oop) in enumerate(cases):
        m, loc = is_.engine.observable(nq.op_table(op), want_loc=True)
        ref = oest2.local_energy(onet, oop, flat)
        assert rel(loc.reshape(-1), ref) < 2e-5
        assert abs(m.mean_re - ref.real.mean()) < 2e-5 * max(1.0, np.max(np.abs(ref)))
        nq.add_observable_(obs, f"o{k}", op)
    res = obs.compute_observables()
    assert set(res) == {"o0", "o1", "o2"}
    mH, locH = is_.engine.observable(nq.op_table(is_.prob), want_loc=True)
    np.testing.assert_allclose(locH, locE, rtol=0, atol=1e-12)
    assert mH.mean_re == mE.mean_re


def test_sr_algorithms_and_reference_multiplicative_quirk(nqlib):
    """precondition_ with SR(algorithm=sr_diag / sr_div / sr_cholesky) on the
    engine's S and F agrees with the oracle; with reference_quirks,
    sr_multiplicative + sr_cholesky / sr_div solve with S itself as the
    reference's precondition! does (SRDirect.jl:64-83): the call is the
    engine's unshifted solve (an ill-conditioned S makes that solve fragile,
    in the reference too, so it is compared with the same engine call, not
    with the oracle), while sr_diag keeps the shift."""
    N, B, L = 6, 256, 8
    for quirks in (False, True):
        is_, net, onet, oH, ohilb = make(N=N, B=B, L=L, burn=10, sigma=0.2 ** 2, quirks=quirks)
        is_.engine.sample(1)
        prec = nq.iterative.SRCache(is_)
        m, loc, force = is_.engine.estimate(want_loc=True, want_force=True)
        S = is_.engine.sr_matrix()
        for alg in (nq.sr_cholesky, nq.sr_diag, nq.sr_div):
            for kind, okind in ((nq.sr_shift, "shift"), (nq.sr_multiplicative, "multiplicative")):
                algo = nq.SR(eps=0.01, precondition_type=kind, algorithm=alg)
                if quirks and kind == nq.sr_multiplicative and alg != nq.sr_diag:
                    outs = []
                    for call in (lambda: nq.precondition_(prec, algo, 3).values,
                                 lambda: is_.engine.precondition(nq.sr_none, 0.01, it=3)):
                        try:
                            outs.append(call())
                        except nq._lib.NqError as e:
                            outs.append(e.status)
                    if isinstance(outs[0], np.ndarray):
                        np.testing.assert_array_equal(outs[0], outs[1])
                    else:
                        assert outs[0] == outs[1]
                    continue
                dw = nq.precondition_(prec, algo, 3).values
                oalg = {nq.sr_cholesky: "cholesky", nq.sr_diag: "diag", nq.sr_div: "div"}[alg]
                # the engine's own S and F, solved in FP64 by the oracle: the solve's own error
                dwo = osr.precondition(S, force, 0.01, kind=okind, it=3, algorithm=oalg)
                assert rel(dw, dwo) < 1e-9, (quirks, alg, okind)


@pytest.mark.parametrize("alpha", [1, 2])
def test_solve_at_large_P(nqlib, alpha):
    """The direct solve at P = 36 + 36 alpha + 36^2 alpha (1368 and 2700):
    the refinement stages its vectors in shared memory up to P = 2560 and
    reads them from L2 beyond; either way Δw matches the FP64 solve of the
    engine's own S and F to 1e-9."""
    N, B, L = 36, 256, 4
    is_, net, onet, oH, ohilb = make(N=N, alpha=alpha, B=B, L=L, burn=4, sigma=0.02 ** 2)
    eng = is_.engine
    assert eng.P == N + alpha * N + alpha * N * N
    eng.sample(2, want_samples=False)
    _, _, F = eng.estimate(want_force=True)
    S = eng.sr_matrix()
    dw = eng.precondition(0, 0.01)
    x = np.linalg.solve(S + 0.01 * np.eye(S.shape[0]), F)
    assert rel(dw, x) < 1e-9
    corr, bound = eng.sr_info()
    assert 1 <= corr <= 12 and bound <= 1e-13
