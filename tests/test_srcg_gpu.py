"""Matrix-free iterative SR (NQ_SR_CG) against the FP64 oracle and the direct
solve on the same samples.

The conjugate-gradient solve never forms S: it applies conj(O_c) O_cᵀ / Ns
from (σ, g, ⟨O⟩) each iteration.  With a tight tolerance (1e-10 relative
residual) Δw agrees with the oracle's direct solve of the FP64 S to the FP32
precision of the operator (relative 2e-3, as the direct path's test), and
the reported residual meets the tolerance.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sr as osr
from oracle.hilbert import Hilbert, SPIN

pytestmark = pytest.mark.gpu


def make(algorithm, N=6, alpha=2, B=64, L=6, sigma=0.1 ** 2, seed=11, eps=0.01, precision=1e-10):
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, alpha, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    s = nq.MetropolisSampler(nq.LocalRule(), L, N, burn=10, seed=seed * 7 + 1)
    is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=eps, algorithm=algorithm, precision=precision), batch_sz=B)
    onet = onw.RBM(N, net.M, onw.LOGCOSH)
    onet.set_flat(net.flat())
    return is_, onet, oex.tfim_1d(Hilbert(N, SPIN), 1.0, 1.0)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


@pytest.mark.parametrize("kind", [0, 1])
def test_cg_solve_matches_oracle(nqlib, kind):
    is_, onet, oH = make(nq.sr_cg)
    eng = is_.engine
    samples, _ = eng.sample(1)
    m, loc, force = eng.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, eng.N).astype(np.float64)
    E = oest.local_energy(onet, oH, flat)
    _, O = onet.logpsi_and_grad(flat)
    F = oest.force_ket(E, O)
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=False)
    if kind == 0:
        dw = eng.precondition(0, 0.01)
        A = S + 0.01 * np.eye(S.shape[0])
    else:
        lam = max(100.0 * 0.95 ** 7, 1e-4)
        dw = eng.precondition(1, 0.0, 100.0, 0.95, 1e-4, 7)
        A = S + lam * np.diag(np.diag(S))
    dwo = np.linalg.solve(A, F)
    assert rel(dw, dwo) < 2e-3
    iters, res = eng.sr_info()
    assert 0 < iters <= 10 * eng.P and res <= 1e-10
    with pytest.raises(nq._lib.NqError):
        eng.sr_matrix()


@pytest.mark.parametrize("N,alpha,B,L", [(8, 2, 256, 8), (9, 1, 1024, 8), (12, 3, 512, 16)])
def test_cg_matches_direct_on_same_samples(nqlib, N, alpha, B, L):
    """CG against the direct solve on one sample set; the shapes cover hidden
    units and sites that do not fill the adjoint's 4 x 8 register tiles
    (M = 9, N = 9 and 12) and several 32-sample tiles per CTA (Ns = 8192)."""
    direct, _, _ = make(nq.sr_cholesky, N=N, alpha=alpha, B=B, L=L)
    cg, _, _ = make(nq.sr_cg, N=N, alpha=alpha, B=B, L=L, precision=1e-9)
    samples, _ = direct.engine.sample(3)
    cg.engine.set_samples(samples)
    direct.engine.estimate()
    cg.engine.estimate()
    d1 = direct.engine.precondition(0, 0.01)
    d2 = cg.engine.precondition(0, 0.01)
    assert rel(d2, d1) < 2e-3


def test_cg_vmc_steps(nqlib):
    direct, _, _ = make(nq.sr_cholesky, N=10, B=512, L=8)
    cg, _, _ = make(nq.sr_cg, N=10, B=512, L=8, precision=1e-6)
    for it in range(5):
        a = direct.engine.vmc_step(it, 0.01, 0.02)
        b = cg.engine.vmc_step(it, 0.01, 0.02)
    assert abs(a.mean_re - b.mean_re) < 5e-3 * abs(a.mean_re)
    iters, res = cg.engine.sr_info()
    assert res <= 1e-6 and iters > 0
