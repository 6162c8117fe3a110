"""θ = Wσ + b on tcgen05 (NQ_EVAL_TC_BF16X2) against the FP64 oracle and
the FP32 CUDA-core evaluation.

W is split into BF16 terms and accumulated in FP32.  With three terms
(hi + mid + lo, about 24 significant bits) θ is FP32-class: the tensor core
accumulates the N products without round-to-nearest, so its θ carries a
small bias that grows with N, where the FP32 CUDA-core path rounds every
addition.  The errors of logψ and ∇logψ against the FP64 oracle stay within
4x (logψ) and 10x (g = tanh θ, amplified near the poles of tanh for complex
θ) of the FP32 path's errors on the same inputs, or within 2e-6 and 2e-5.
With two terms (about 16 bits) logψ stays within 1e-4 relative and g within
2e-3.  Sizes cover one K step (N = 7),
two column chunks of the MMA (2M = 288 > 256) and partial tiles.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw

pytestmark = pytest.mark.gpu


def engine(N, alpha, prec, B=96, L=3, sigma=0.2 ** 2, seed=5):
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, alpha, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - 1.3 * nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    s = nq.MetropolisSampler(nq.LocalRule(), L, N, burn=4, seed=seed)
    is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B, eval_precision=prec)
    onet = onw.RBM(N, net.M, onw.LOGCOSH)
    onet.set_flat(net.flat())
    return is_.engine, onet


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


X2, X3 = nq._lib.NQ_EVAL_TC_BF16X2, nq._lib.NQ_EVAL_TC_BF16X3


def _errors(N, alpha, prec):
    eng, onet = engine(N, alpha, prec)
    rng = np.random.default_rng(N)
    sig = rng.choice([-1, 1], size=(301, N)).astype(np.int8)
    lp, g = eng.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig.astype(np.float64))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    return np.max(np.abs(d)) / np.max(np.abs(olp)), rel(g, og)


@pytest.mark.parametrize("N,alpha", [(7, 2), (20, 2), (36, 4), (33, 3)])
def test_theta_tc_logpsi_and_grad(nqlib, N, alpha):
    """Three BF16 terms are FP32-class (see the module docstring); two terms
    keep logψ within 1e-4 and g within 2e-3."""
    lp32, g32 = _errors(N, alpha, nq._lib.NQ_EVAL_F32)
    lp3, g3 = _errors(N, alpha, X3)
    lp2, g2 = _errors(N, alpha, X2)
    assert lp3 <= max(4 * lp32, 2e-6) and g3 <= max(10 * g32, 2e-5)
    assert lp2 < 1e-4 and g2 < 2e-3


@pytest.mark.parametrize("N,alpha", [(20, 2), (36, 4)])
def test_theta_tc_estimator_matches_cuda_cores(nqlib, N, alpha):
    tc, _ = engine(N, alpha, X3, B=256, L=4)
    f32, _ = engine(N, alpha, nq._lib.NQ_EVAL_F32, B=256, L=4)
    samples, _ = f32.sample(3)
    tc.set_samples(samples)
    m1, loc1, f1 = f32.estimate(want_loc=True, want_force=True)
    m2, loc2, f2 = tc.estimate(want_loc=True, want_force=True)
    assert rel(loc2, loc1) < 1e-4
    assert rel(f2, f1) < 1e-3
    assert abs(m2.mean_re - m1.mean_re) < 1e-4 * abs(m1.mean_re)


def test_theta_tc_vmc_step(nqlib):
    tc, _ = engine(20, 2, X2, B=512, L=8)
    f32, _ = engine(20, 2, nq._lib.NQ_EVAL_F32, B=512, L=8)
    for it in range(3):
        a = tc.vmc_step(it, 0.01, 0.02)
        b = f32.vmc_step(it, 0.01, 0.02)
    assert abs(a.mean_re - b.mean_re) < 5e-3 * abs(b.mean_re)
    assert rel(tc.get_params(), f32.get_params()) < 1e-2


def ndm_engine(N, ah, aa, prec, B=128, L=4, sigma=0.2 ** 2, seed=6, sp=nq._lib.NQ_S_F32):
    hilb = nq.HomogeneousSpin(N)
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H = H + 0.5 * nq.sigmax(hilb, i)
        Ls.append(nq.sigmam(hilb, i))
    for i in range(1, N):
        H = H + 0.5 * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    net = nq.NDM(np.float64, N, ah, aa, nq.af_softplus)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    s = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=4, seed=seed)
    is_ = nq.BatchedSampler(net, s, nq.liouvillian(H, Ls), nq.SR(eps=0.01), batch_sz=B, eval_precision=prec,
                            s_precision=sp)
    onet = onw.NDM(N, ah, aa, onw.SOFTPLUS)
    onet.set_flat(net.flat())
    return is_.engine, onet


@pytest.mark.parametrize("N,ah,aa", [(6, 1, 1), (12, 2, 2)])
def test_ndm_theta_tc_logrho_and_grad(nqlib, N, ah, aa):
    """The density matrix's unit pre-activations θ_u = b_u + C_u·(σ, η) on
    tcgen05 (U = 4 αN + βN units over the 2N doubled sites): logρ and ∇logρ
    against the FP64 oracle, three BF16 terms within 2e-5 (FP32 class), two
    within 1e-4 (logρ) and 2e-3 (∇logρ)."""
    rng = np.random.default_rng(N)
    sig = rng.choice([-1, 1], size=(301, 2 * N)).astype(np.int8)
    for prec, tl, tg in ((X3, 2e-5, 2e-5), (X2, 1e-4, 2e-3)):
        eng, onet = ndm_engine(N, ah, aa, prec)
        lp, g = eng.logpsi(sig, with_grad=True)
        olp, og = onet.logpsi_and_grad(sig[:, :N].astype(np.float64), sig[:, N:].astype(np.float64))
        d = lp - olp
        d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
        assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tl, prec
        assert rel(g, og) < tg, prec


def test_ndm_theta_tc_estimator_matches_cuda_cores(nqlib):
    """The precision form of the N = 12 dissipative Ising workload: L_loc, the
    cost, F and S with θ on tcgen05 (BF16 x3 and x2) against the FP32
    CUDA-core evaluation on the same samples, and one SR step from each."""
    N = 12
    f32, _ = ndm_engine(N, 2, 2, nq._lib.NQ_EVAL_F32, B=512, L=4, sp=nq._lib.NQ_S_TF32)
    samples, _ = f32.sample(2)
    m1, loc1, f1 = f32.estimate(want_loc=True, want_force=True)
    s1 = f32.sr_matrix()
    for prec, tol in ((X3, 1e-4), (X2, 2e-3)):
        tc, _ = ndm_engine(N, 2, 2, prec, B=512, L=4, sp=nq._lib.NQ_S_TF32)
        tc.set_samples(samples)
        m2, loc2, f2 = tc.estimate(want_loc=True, want_force=True)
        assert rel(loc2, loc1) < tol, prec
        assert abs(m2.mean_re - m1.mean_re) < tol * abs(m1.mean_re), prec
        assert rel(f2, f1) < 10 * tol, prec
        assert rel(tc.sr_matrix(), s1) < 10 * tol, prec
        a = tc.vmc_step(5, 0.01, 0.01)
        assert np.isfinite(a.mean_re)
