"""Density-matrix chains MixedStateAnsatz(Chain(DenseSplit(N, M, f) |
PositiveDefR(N, M, f), Dense..., sum_autobatch | WSum), N)
(src/Networks/MixedDensityMatrix/MixedChainWrapper.jl,
Chains/Layers/DenseSplit.jl, Chains/Layers/PositiveDefR.jl; the chain of
test/Machines/test_grad.jl:49-50) with the dissipative Ising Liouvillian, on
the GPU against the FP64 oracle.  PositiveDefR's parameters are real, so its
chains take the reference's real SR (SRDirect.jl:11-38): S = Re(O_c O_c†)/Ns,
F real, a real Δw that leaves every imaginary part unchanged.

Tolerances: logρ, ∇logρ, L_loc relative 2e-5 (FP32) / 1e-10 (FP64); chains on
the doubled sites bit-exact against the Philox replay (near-ties
|log u - Δ| < 1e-6 follow the device); the cost mean 1e-5; F 1e-4; S 1e-4;
Δw 1e-9 against the FP64 solve of the engine's own S and F, 2e-3 against the
oracle's Δw; χ² of the doubled samples against |ρ|², p > 1e-3; SR lowers the
exact cost ⟨|Lρ|²⟩/⟨|ρ|²⟩.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, sr as osr, \
    operators as oops
from oracle.hilbert import Hilbert, SPIN, FOCK

pytestmark = pytest.mark.gpu

ACTS = {nq.af_logcosh: onw.LOGCOSH, nq.af_softplus: onw.SOFTPLUS, nq.identity: onw.IDENTITY}
SHAPES = {
    "split_sum": lambda N: [("split", 2 * N, nq.af_softplus), ("sum",)],
    "split_dense_wsum": lambda N: [("split", N + 1, nq.af_logcosh), ("dense", N + 1, N, nq.af_softplus),
                                   ("wsum",)],
    "pdr_sum": lambda N: [("pdr", 2 * N, nq.af_logcosh), ("sum",)],
    "pdr_dense_wsum": lambda N: [("pdr", N + 1, nq.af_softplus), ("dense", N + 1, N, nq.af_logcosh), ("wsum",)],
}


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


def dissipative(hilb, N, g=1.0, V=2.0, gamma=1.0):
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H = H + (g / 2) * nq.sigmax(hilb, i)
        Ls.append(float(np.sqrt(gamma)) * nq.sigmam(hilb, i))
    for i in range(1, N):
        H = H + (V / 4) * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    return nq.liouvillian(H, Ls)


def build(N, shape, sigma=0.2 ** 2, seed=4):
    layers, olayers, width = [], [], N
    for l in SHAPES[shape](N):
        if l[0] == "split":
            layers.append(nq.DenseSplit(np.complex64, N, l[1], l[2]))
            olayers.append(("dense_split", N, l[1], ACTS[l[2]]))
            width = l[1]
        elif l[0] == "pdr":
            layers.append(nq.PositiveDefR(np.float32, N, l[1], l[2]))
            olayers.append(("positive_def_r", N, l[1], ACTS[l[2]]))
            width = l[1]
        elif l[0] == "dense":
            layers.append(nq.Dense(np.complex64, l[1], l[2], l[3]))
            olayers.append(("dense", l[1], l[2], ACTS[l[3]]))
            width = l[2]
        elif l[0] == "wsum":
            layers.append(nq.WSum(np.complex64, width))
            olayers.append(("wsum", width))
        else:
            layers.append(nq.sum_autobatch)
            olayers.append(("sum", width))
    net = nq.MixedStateAnsatz(nq.Chain(*layers), N)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    onet = onw.MixedChain(N, olayers)
    onet.set_flat(net.flat())
    return net, onet


def make(N, shape, B=64, L=4, burn=3, kind="spin", prec=nq._lib.NQ_EVAL_F32, sp=nq._lib.NQ_S_F32, seed=4,
         sigma=0.2 ** 2):
    net, onet = build(N, shape, sigma, seed)
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    smp = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=burn, seed=seed + 11)
    is_ = nq.BatchedSampler(net, smp, dissipative(hilb, N), nq.SR(eps=0.01), batch_sz=B, eval_precision=prec,
                            s_precision=sp)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    oH, oL = oex.dissipative_ising(ohilb, 1.0, 2.0)
    return is_, net, onet, oops.liouvillian(oH, oL), ohilb


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_mixed_chain_logrho_and_grad(nqlib, shape, prec, tol):
    N = 4
    is_, net, onet, _, _ = make(N, shape, prec=prec)
    rng = np.random.default_rng(5)
    sig = rng.choice([-1, 1], size=(200, 2 * N)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig[:, :N].astype(np.float64), sig[:, N:].astype(np.float64))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / np.max(np.abs(olp)) < tol
    assert rel(g, og) < tol


@pytest.mark.parametrize("kind,shape", [("spin", "split_sum"), ("fock", "split_sum"), ("spin", "pdr_sum"),
                                        ("fock", "pdr_dense_wsum")])
def test_mixed_chain_doubled_sampler_bitexact(nqlib, kind, shape):
    N, B, L, burn = 4, 64, 4, 3
    is_, net, onet, _, ohilb = make(N, shape, B=B, L=L, burn=burn, kind=kind, sigma=0.4 ** 2)
    samples, bits = is_.engine.sample(2, want_accept_bits=True)
    ref, info = osm.run(lambda x: onet.log_prob(x[:, :N], x[:, N:]), ohilb, B, L, burn, is_.engine.passes,
                        is_.engine.cfg.seed, call=2, doubled=True, gpu_accept_bits=bits)
    assert info["mismatch"] == 0 and info["ambiguous"] <= 3
    np.testing.assert_array_equal(samples.astype(np.float64), ref)


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_mixed_chain_liouvillian_force_S_solve(nqlib, shape, prec, tol):
    N, B, L = 4, 48, 5
    is_, net, onet, olv, ohilb = make(N, shape, B=B, L=L, burn=6, prec=prec)
    eng = is_.engine
    samples, _ = eng.sample(1)
    m, loc, force = eng.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    sr, sc = flat[:, :N], flat[:, N:]
    Lo, dL = oest.local_liouvillian(onet, olv, sr, sc)
    assert rel(loc.reshape(-1), Lo) < tol
    _, O = onet.logpsi_and_grad(sr, sc)
    C, F = oest.force_liouvillian(Lo, dL, O)
    assert abs(m.mean_re - C) < 1e-5 * C
    if onet.real_sr:
        F = np.real(F) + 0j
        assert np.all(force.imag == 0)
    assert rel(force, F) < 1e-4
    S = osr.build_S(oest.center(O)[0], real_params=onet.real_sr)
    Sg = eng.sr_matrix()
    assert rel(Sg, S) < 1e-4
    if onet.real_sr:
        assert np.all(Sg.imag == 0)
    dw = eng.precondition(0, 0.01)
    assert rel(dw, np.linalg.solve(Sg + 0.01 * np.eye(Sg.shape[0]), force)) < 1e-9
    assert rel(dw, osr.precondition(S, F, 0.01, real_params=onet.real_sr)) < 2e-3
    if onet.real_sr:
        assert np.all(dw.imag == 0)


@pytest.mark.parametrize("shape,scale", [("split_sum", 0.4), ("pdr_sum", 0.2)])
def test_mixed_chain_chi_square_against_exact(nqlib, shape, scale):
    """Doubled samples against |ρ|²; the bins expecting fewer than 5 counts
    are pooled.  PositiveDefR is drawn at a smaller scale: at 0.4 its |ρ|²
    puts 0.94 of the weight on one doubled state, and 30 burn-in sweeps of the
    oracle's own Philox chains fail this test there too."""
    from scipy.stats import chisquare
    N = 3
    is_, net, onet, _, ohilb = make(N, shape, B=16384, L=1, burn=30, sigma=scale ** 2, seed=9)
    samples, _ = is_.engine.sample(0)
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    idx = ohilb.index_of_state(flat[:, N:]) * ohilb.dim + ohilb.index_of_state(flat[:, :N])
    counts = np.bincount(idx, minlength=ohilb.dim ** 2)
    p = oex.doubled_distribution(onet, ohilb)
    exp = p * counts.sum()
    small = exp < 5
    if small.any():
        counts = np.append(counts[~small], counts[small].sum())
        exp = np.append(exp[~small], exp[small].sum())
    stat, pval = chisquare(counts, exp)
    assert pval > 1e-3, (stat, pval)


@pytest.mark.parametrize("shape", ["split_sum", "pdr_sum"])
def test_mixed_chain_sr_lowers_the_exact_cost(nqlib, shape):
    """Steady-state SR with the captured whole step (3xTF32 S): the exact
    cost Σ|Lρ|²/Σ|ρ|² over all doubled states falls.  PositiveDefR's
    parameters stay real and ρ stays Hermitian, ρ(η, σ) = conj ρ(σ, η)."""
    N = 3
    is_, net, onet, olv, ohilb = make(N, shape, B=512, L=8, burn=20, sigma=0.1 ** 2, seed=3)
    Lm = oops.liouvillian_to_matrix(olv)
    st = ohilb.all_states()
    D = ohilb.dim
    sr = np.repeat(st[None], D, axis=0).reshape(-1, N)
    sc = np.repeat(st, D, axis=0)

    def exact_cost():
        onet.set_flat(is_.engine.get_params())
        v = np.exp(onet.logpsi(sr, sc))
        return float(np.sum(np.abs(Lm @ v) ** 2) / np.sum(np.abs(v) ** 2))

    c0 = exact_cost()
    for _ in range(80):
        m = is_.step(lr=0.02, eps=0.01)
        assert np.isfinite(m.mean)
    assert exact_cost() < 0.7 * c0
    if onet.real_sr:
        assert np.all(is_.engine.get_params().imag == 0)
        lr_, lc_ = onet.logpsi(sr, sc), onet.logpsi(sc, sr)
        np.testing.assert_allclose(np.exp(lc_), np.conj(np.exp(lr_)), rtol=1e-12, atol=0)
