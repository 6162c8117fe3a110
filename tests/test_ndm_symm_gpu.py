"""NDMSymm (src/Networks/MixedDensityMatrix/NDMSymm.jl) on the doubled-space
path against the FP64 oracle, through the C-ABI.

The trainable parameters are the symmetric NDM's; the engine evaluates the
bare NDM built from them and maps the bare O onto the symmetric parameters.
Tolerances as for the NDM: logρ, ∇logρ, L_loc relative 2e-5 (FP32) / 1e-10
(FP64); chains bit-exact; F 1e-4; S 1e-4; Δw 2e-3; the update keeps the
visible biases at their mean (set_bare_params!, NDMSymm.jl:97-98).
"""
import ctypes

import numpy as np
import pytest

import nqcuda as nq
from nqcuda import _lib
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, \
    sr as osr, stats as ost, operators as oops
from oracle.hilbert import Hilbert, FOCK

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


def translations(N):
    return [[(i + t) % N for i in range(N)] for t in range(N)]


def make(N=4, ah=2, aa=1, act=nq.af_logcosh, B=64, L=4, burn=5, sigma=0.2 ** 2, seed=3,
         prec=nq._lib.NQ_EVAL_F32, sp=nq._lib.NQ_S_F32, perms=None):
    perms = translations(N) if perms is None else perms
    hilb = nq.HomogeneousFock(N)
    net = nq.NDMSymm(np.float64, N, ah, aa, perms, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    lv = dissipative(hilb, N)
    smp = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=burn, seed=seed + 100)
    is_ = nq.BatchedSampler(net, smp, lv, nq.SR(eps=0.01), batch_sz=B, eval_precision=prec, s_precision=sp)
    ohilb = Hilbert(N, FOCK)
    onet = onw.NDMSymm(N, ah, aa, perms, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    oH, oL = oex.dissipative_ising(ohilb, 1.0, 2.0)
    olv = oops.liouvillian(oH, oL)
    return is_, net, onet, olv, ohilb


@pytest.mark.parametrize("act", [nq.af_logcosh, nq.af_softplus])
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_ndm_symm_logrho_and_grad(nqlib, act, prec, tol):
    N = 4
    is_, net, onet, _, _ = make(N=N, act=act, prec=prec, sigma=0.3 ** 2)
    assert is_.engine.P == onet.n_params
    # the engine averaged the visible biases like set_bare_params!
    np.testing.assert_allclose(is_.engine.get_params(), onet.flat(), rtol=0, atol=1e-14)
    sig = np.random.default_rng(1).integers(0, 2, size=(300, 2 * N)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig[:, :N].astype(float), sig[:, N:].astype(float))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tol
    assert rel(g, og) < tol


def test_ndm_symm_sampler_bitexact(nqlib):
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
def test_ndm_symm_estimator_force_S_solve_update(nqlib, prec):
    N, B, L = 4, 48, 5
    is_, net, onet, olv, ohilb = make(N=N, B=B, L=L, burn=8, prec=prec)
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
    assert rel(force, np.real(F)) < 1e-4
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=True)
    assert rel(is_.engine.sr_matrix(), S) < 1e-4
    dw = is_.engine.precondition(0, 0.01)
    dwo = osr.precondition(S, F, 0.01, real_params=True)
    assert rel(dw, dwo) < 2e-3
    p0 = is_.engine.get_params()
    is_.engine.update_descent(0.01)
    onet.set_flat(p0 - 0.01 * dw)          # update!, then set_bare_params! (NDMSymm.jl:38-40)
    np.testing.assert_allclose(is_.engine.get_params(), onet.flat(), rtol=0, atol=1e-12)


def test_ndm_symm_graph_steps_lower_the_cost(nqlib):
    N = 4
    is_, net, _, _, _ = make(N=N, B=512, L=8, burn=10, sigma=0.05 ** 2, seed=4, sp=nq._lib.NQ_S_TF32X3)
    costs = [is_.step(0.01).mean]
    for _ in range(60):
        costs.append(is_.step(0.01).mean)
    assert np.all(np.isfinite(costs))
    assert np.mean(costs[-5:]) < 0.9 * np.mean(costs[:5]), costs


def test_ndm_symm_needs_permutations(nqlib):
    N = 4
    net = nq.NDMSymm(np.float64, N, 1, 1, translations(N))
    cfg = nq.engine.make_config(net, nq.SuperOpSpace(nq.HomogeneousFock(N)), 16, 2, 1, 3, 7)
    L = _lib.lib()
    h = ctypes.c_void_p()
    assert L.nq_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.NQ_OK
    try:
        assert L.nq_sample(h, 0, None, None) == _lib.NQ_ERR_STATE
        bad = np.ascontiguousarray([[0, 0, 1, 2]] * N, dtype=np.int32)
        assert L.nq_set_symmetry(h, N, bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == _lib.NQ_ERR_ARG
        good = np.ascontiguousarray(translations(N), dtype=np.int32)
        assert L.nq_set_symmetry(h, N, good.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == _lib.NQ_OK
        assert L.nq_sample(h, 0, None, None) == _lib.NQ_OK
    finally:
        L.nq_destroy(h)
