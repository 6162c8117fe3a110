"""Matrix-free iterative SR (NQ_SR_CG) against the FP64 oracle and the direct
solve on the same samples.

The conjugate-gradient solve never forms S: it applies conj(O_c) O_cᵀ / Ns
each iteration, from (σ, g, ⟨O⟩) for the RBM and from the centred O rows of X
for the other networks (feed-forward chains, the NDM, density-matrix chains
with complex DenseSplit or real PositiveDefR parameters).  With a tight
tolerance Δw agrees with the oracle's direct solve of the FP64 S, and with
the engine's direct solve on the same samples, to the FP32 precision of the
operator (relative 2e-3, as the direct path's test), and the reported
residual meets the tolerance.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sr as osr, operators as oops
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


def _tfim(hilb, N):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


def _dissipative(hilb, N, g=1.0, V=2.0, gamma=1.0):
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H = H + (g / 2) * nq.sigmax(hilb, i)
        Ls.append(float(np.sqrt(gamma)) * nq.sigmam(hilb, i))
    for i in range(1, N):
        H = H + (V / 4) * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    return nq.liouvillian(H, Ls)


def make_x(network, algorithm, B=128, L=8, seed=5, precision=1e-9):
    """The networks whose O the CG solve reads from X, with the oracle twin."""
    if network == "chain":          # examples/ising1d_ffnn.jl
        N = 8
        hilb = nq.HomogeneousSpin(N)
        net = nq.PureChain(N, nq.Dense(np.complex64, N, 2 * N, nq.af_logcosh), nq.sum_autobatch)
        nq.init_random_pars_(net, sigma=0.1 ** 2, rng=np.random.default_rng(seed))
        onet = onw.Chain(N, [("dense", N, 2 * N, onw.LOGCOSH), ("sum", 2 * N)])
        prob, nst, real = _tfim(hilb, N), N, False
    elif network == "ndm":          # examples/dissipative_ising1d.jl
        N = 4
        hilb = nq.HomogeneousSpin(N)
        net = nq.NDM(np.float64, N, 1, 1, nq.af_softplus)
        nq.init_random_pars_(net, sigma=0.1 ** 2, rng=np.random.default_rng(seed))
        onet = onw.NDM(N, 1, 1, onw.SOFTPLUS)
        prob, nst, real = _dissipative(hilb, N), 2 * N, True
    else:                           # density-matrix chains
        N = 4
        hilb = nq.HomogeneousSpin(N)
        if network == "mixed_pdr":
            first, ofirst = nq.PositiveDefR(np.float32, N, 2 * N, nq.af_logcosh), "positive_def_r"
        else:
            first, ofirst = nq.DenseSplit(np.complex64, N, 2 * N, nq.af_logcosh), "dense_split"
        net = nq.MixedStateAnsatz(nq.Chain(first, nq.sum_autobatch), N)
        nq.init_random_pars_(net, sigma=0.15 ** 2, rng=np.random.default_rng(seed))
        onet = onw.MixedChain(N, [(ofirst, N, 2 * N, onw.LOGCOSH), ("sum", 2 * N)])
        prob, nst, real = _dissipative(hilb, N), 2 * N, network == "mixed_pdr"
    onet.set_flat(net.flat())
    smp = nq.MetropolisSampler(nq.LocalRule(), L, nst, burn=10, seed=seed * 3 + 1)
    is_ = nq.BatchedSampler(net, smp, prob, nq.SR(eps=0.01, algorithm=algorithm, precision=precision),
                            batch_sz=B)
    return is_, onet, real


@pytest.mark.parametrize("network", ["chain", "ndm", "mixed_split", "mixed_pdr"])
def test_cg_over_X_matches_direct_on_same_samples(nqlib, network):
    direct, onet, real = make_x(network, nq.sr_cholesky)
    cg, _, _ = make_x(network, nq.sr_cg)
    samples, _ = direct.engine.sample(2)
    cg.engine.set_samples(samples)
    _, _, f1 = direct.engine.estimate(want_force=True)
    _, _, f2 = cg.engine.estimate(want_force=True)
    assert rel(f2, f1) < 1e-6
    d1 = direct.engine.precondition(0, 0.01)
    d2 = cg.engine.precondition(0, 0.01)
    assert rel(d2, d1) < 2e-3
    if real:
        assert np.all(np.imag(d2) == 0)
    iters, res = cg.engine.sr_info()
    assert 0 < iters <= 10 * cg.engine.P and res <= 1e-9
    with pytest.raises(nq._lib.NqError):
        cg.engine.sr_matrix()


@pytest.mark.parametrize("network", ["chain", "ndm"])
def test_cg_over_X_matches_oracle(nqlib, network):
    """Δw of the shift and the multiplicative shift against the oracle's FP64
    solve on the engine's samples."""
    is_, onet, real = make_x(network, nq.sr_cg, precision=1e-10)
    eng = is_.engine
    samples, _ = eng.sample(1)
    _, _, force = eng.estimate(want_force=True)
    if network == "chain":
        flat = samples.reshape(-1, eng.N).astype(np.float64)
        _, O = onet.logpsi_and_grad(flat)
    else:
        flat = samples.reshape(-1, 2 * eng.N).astype(np.float64)
        _, O = onet.logpsi_and_grad(flat[:, :eng.N], flat[:, eng.N:])
    S = osr.build_S(oest.center(O)[0], real_params=real)
    for kind in (0, 1):
        if kind == 0:
            dw = eng.precondition(0, 0.01)
            A = S + 0.01 * np.eye(S.shape[0])
        else:
            lam = max(100.0 * 0.95 ** 7, 1e-4)
            dw = eng.precondition(1, 0.0, 100.0, 0.95, 1e-4, 7)
            A = S + lam * np.diag(np.diag(S))
        dwo = np.linalg.solve(A, np.real(force) if real else force)
        assert rel(dw, dwo) < 2e-3, kind


def test_cg_ffnn_example_lowers_energy(nqlib):
    """examples/ising1d_ffnn.jl's solver, SR(ϵ=0.1, algorithm=sr_cg,
    precision=1e-3), on its Chain(Dense(N, 2N, af_logcosh), sum_autobatch)."""
    N = 8
    hilb = nq.HomogeneousSpin(N)
    net = nq.PureChain(N, nq.Dense(np.complex64, N, 2 * N, nq.af_logcosh), nq.sum_autobatch)
    nq.init_random_pars_(net, sigma=0.05 ** 2, rng=np.random.default_rng(3))
    smp = nq.MetropolisSampler(nq.LocalRule(), 8, N + 1, burn=10, seed=20)
    is_ = nq.BatchedSampler(net, smp, _tfim(hilb, N), nq.SR(eps=0.1, algorithm=nq.sr_cg, precision=1e-3),
                            batch_sz=512)
    e0 = oex.tfim_ground_energy_1d(N, 1.0, 1.0)
    first = is_.step(0.05)
    for _ in range(60):
        m = is_.step(0.05)
    assert m.mean.real < first.mean.real - 0.05 * abs(e0)
    assert m.mean.real > e0 - 5 * max(m.error, 1e-3)
    iters, res = is_.engine.sr_info()
    assert iters > 0 and res <= 1e-3


@pytest.mark.parametrize("algorithm", [nq.sr_cholesky, nq.sr_cg])
def test_time_evolution_solves_with_i_force(nqlib, algorithm):
    """SR(time_evo=true) (SRDirect.jl:27, SRIterative.jl:33): the solve takes
    i F.  Direct: against the FP64 solve of the engine's own S with i F; both
    solvers: i times the solve with F; switching it off restores Δw."""
    is_, onet, oH = make(algorithm, precision=1e-10)
    eng = is_.engine
    eng.sample(1)
    _, _, force = eng.estimate(want_force=True)
    dw0 = eng.precondition(0, 0.01)
    eng.set_time_evolution(True)
    dw1 = eng.precondition(0, 0.01)
    assert rel(dw1, 1j * dw0) < 1e-6
    if algorithm == nq.sr_cholesky:
        Sg = eng.sr_matrix()
        assert rel(dw1, np.linalg.solve(Sg + 0.01 * np.eye(Sg.shape[0]), 1j * force)) < 1e-9
    eng.set_time_evolution(False)
    assert rel(eng.precondition(0, 0.01), dw0) < 1e-12


def test_time_evolution_real_parameters(nqlib):
    """Real parameters (NDM): the solve takes Re(i F) = -Im F, F from the
    oracle on the engine's samples (|Im F| is ~7% of |F| here, hence 1e-2)."""
    is_, onet, real = make_x("ndm", nq.sr_cholesky)
    eng = is_.engine
    samples, _ = eng.sample(1)
    eng.estimate()
    N = eng.N
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    oH, oL = oex.dissipative_ising(Hilbert(N, SPIN), 1.0, 2.0)
    Lo, dL = oest.local_liouvillian(onet, oops.liouvillian(oH, oL), flat[:, :N], flat[:, N:])
    _, O = onet.logpsi_and_grad(flat[:, :N], flat[:, N:])
    _, F = oest.force_liouvillian(Lo, dL, O)
    eng.set_time_evolution(True)
    dw = eng.precondition(0, 0.01)
    Sg = eng.sr_matrix()
    assert np.isrealobj(dw)
    assert rel(dw, np.linalg.solve(Sg + 0.01 * np.eye(Sg.shape[0]), -np.imag(F))) < 1e-2
