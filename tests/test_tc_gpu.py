"""tcgen05 SR-matrix accumulation (kind::tf32) against the FP64 oracle and
the FP32 CUDA-core path.

Tolerances: TF32 (one product, operands rounded to 10-bit mantissa):
relative 2e-3 of max|S|; 3xTF32 (hi*hi + hi*lo + lo*hi): 2e-5; BF16
(kind::f16, operands rounded to 8-bit mantissa, FP32 accumulation): 1e-2.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import estimators as oest, sr as osr
from test_rbm_gpu import make, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sp,tol", [(nq._lib.NQ_S_TF32, 2e-3), (nq._lib.NQ_S_TF32X3, 2e-5),
                                    (nq._lib.NQ_S_BF16, 1e-2)])
@pytest.mark.parametrize("N,alpha,B,L", [(6, 2, 64, 6), (9, 1, 200, 3), (20, 2, 256, 5)])
def test_tf32_gram_matches_oracle(nqlib, sp, tol, N, alpha, B, L):
    is_, net, onet, oH, ohilb = make(N=N, alpha=alpha, B=B, L=L, burn=5, sigma=0.1 ** 2)
    eng = is_.engine
    # rebuild the engine with the requested S precision, same everything else
    eng2 = nq.Engine(net, nq.HomogeneousSpin(N), B, L, 5, N, eng.cfg.seed, s_precision=sp)
    eng2.set_params(net.flat())
    eng2.set_operator(nq.op_table(is_.prob))
    samples, _ = eng2.sample(2)
    m, loc, force = eng2.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, N).astype(np.float64)
    _, O = onet.logpsi_and_grad(flat)
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=False)
    Sg = eng2.sr_matrix()
    assert rel(Sg, S) < tol
    # Hermitian by construction
    assert np.max(np.abs(Sg - Sg.conj().T)) == 0.0
    E = oest.local_energy(onet, oH, flat)
    dw = eng2.precondition(0, 0.01)
    dwo = osr.precondition(S, oest.force_ket(E, O), 0.01)
    assert rel(dw, dwo) < {nq._lib.NQ_S_TF32: 5e-2, nq._lib.NQ_S_TF32X3: 2e-3, nq._lib.NQ_S_BF16: 2e-1}[sp]


def test_tf32x3_matches_fp32_cuda_cores_at_full_size(nqlib):
    """N=20, α=2 (P=860), 4096 chains x 20: tcgen05 3xTF32 vs the FP32 path."""
    N = 20
    res = {}
    for sp in (nq._lib.NQ_S_F32, nq._lib.NQ_S_TF32X3):
        hilb = nq.HomogeneousSpin(N)
        net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
        nq.init_random_pars_(net, sigma=0.05 ** 2, rng=np.random.default_rng(1))
        H = nq.LocalOperator(hilb)
        for i in range(1, N + 1):
            H = H - nq.sigmax(hilb, i) + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
        s = nq.MetropolisSampler(nq.LocalRule(), 20, N, burn=10, seed=77)
        is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=4096, s_precision=sp)
        is_.engine.sample(0, want_samples=False)
        is_.engine.estimate()
        res[sp] = is_.engine.sr_matrix()
    assert rel(res[nq._lib.NQ_S_TF32X3], res[nq._lib.NQ_S_F32]) < 3e-5


def test_bf16_gram_full_size_and_graph_step(nqlib):
    """N=20, α=2, 4096 chains x 20: BF16 S against the FP32 path and one
    graph-replayed SR iteration in the BF16 mode."""
    N = 20
    res, eng = {}, {}
    for sp in (nq._lib.NQ_S_F32, nq._lib.NQ_S_BF16):
        hilb = nq.HomogeneousSpin(N)
        net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
        nq.init_random_pars_(net, sigma=0.05 ** 2, rng=np.random.default_rng(1))
        H = nq.LocalOperator(hilb)
        for i in range(1, N + 1):
            H = H - nq.sigmax(hilb, i) + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
        s = nq.MetropolisSampler(nq.LocalRule(), 20, N, burn=10, seed=77)
        is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=4096, s_precision=sp)
        is_.engine.sample(0, want_samples=False)
        is_.engine.estimate()
        res[sp] = is_.engine.sr_matrix()
        eng[sp] = is_.engine
    assert rel(res[nq._lib.NQ_S_BF16], res[nq._lib.NQ_S_F32]) < 1e-2
    a = eng[nq._lib.NQ_S_BF16].vmc_step(1, 0.01, 0.01)
    b = eng[nq._lib.NQ_S_F32].vmc_step(1, 0.01, 0.01)
    assert abs(a.mean_re - b.mean_re) < 1e-3 * abs(b.mean_re)
