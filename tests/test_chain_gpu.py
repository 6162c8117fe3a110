"""Feed-forward kets PureStateAnsatz(Chain(Dense..., sum_autobatch | WSum))
(src/Networks/Chains/) on the GPU against the FP64 oracle, through the C-ABI.

Tolerances: logψ, ∇logψ, E_loc relative 2e-5 (FP32) / 1e-10 (FP64); chains
bit-exact against the Philox replay (near-ties |log u - Δ| < 1e-6 follow the
device); F 1e-4; S 1e-4 (FP32 S); Δw 2e-3; χ² p > 1e-3; the chain of
examples/ising1d_ffnn.jl lowers the TFIM energy.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, \
    sr as osr, stats as ost, operators as oops
from oracle.hilbert import Hilbert, SPIN

pytestmark = pytest.mark.gpu

ACTS = {nq.af_logcosh: onw.LOGCOSH, nq.af_softplus: onw.SOFTPLUS, nq.identity: onw.IDENTITY}

# the chains of test/Machines/test_grad.jl:29-44 and test_batched.jl:32-46
SHAPES = {
    "dense_sum": lambda N: [("dense", N, 2 * N, nq.af_logcosh), ("sum",)],
    "two_dense_wsum": lambda N: [("dense", N, 2 * N, nq.identity), ("dense", 2 * N, 3 * N, nq.identity),
                                 ("wsum",)],
    "softplus_wsum": lambda N: [("dense", N, N - 1, nq.af_softplus), ("dense", N - 1, N - 2, nq.af_softplus),
                                ("wsum",)],
    "two_logcosh_sum": lambda N: [("dense", N, 2 * N, nq.af_logcosh), ("dense", 2 * N, N, nq.af_logcosh),
                                  ("sum",)],
}


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


def tfim(hilb, N, h=1.0, J=1.0):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - h * nq.sigmax(hilb, i)
        H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


def build(N, shape, sigma=0.3 ** 2, seed=2):
    spec = SHAPES[shape](N)
    layers, olayers, width = [], [], N
    for l in spec:
        if l[0] == "dense":
            layers.append(nq.Dense(np.complex64, l[1], l[2], l[3]))
            olayers.append(("dense", l[1], l[2], ACTS[l[3]]))
            width = l[2]
        elif l[0] == "wsum":
            layers.append(nq.WSum(np.complex64, width))
            olayers.append(("wsum", width))
        else:
            layers.append(nq.sum_autobatch)
            olayers.append(("sum", width))
    net = nq.PureChain(N, *layers)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    onet = onw.Chain(N, olayers)
    onet.set_flat(net.flat())
    return net, onet


def make(N, shape, B=64, L=4, burn=3, passes=None, sigma=0.3 ** 2, seed=2, prec=nq._lib.NQ_EVAL_F32,
         sp=nq._lib.NQ_S_F32):
    net, onet = build(N, shape, sigma, seed)
    hilb = nq.HomogeneousSpin(N)
    smp = nq.MetropolisSampler(nq.LocalRule(), L, passes or N, burn=burn, seed=seed + 17)
    is_ = nq.BatchedSampler(net, smp, tfim(hilb, N), nq.SR(eps=0.01), batch_sz=B, eval_precision=prec,
                            s_precision=sp)
    return is_, net, onet, Hilbert(N, SPIN)


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("prec,tol", [(nq._lib.NQ_EVAL_F32, 2e-5), (nq._lib.NQ_EVAL_F64, 1e-10)])
def test_chain_logpsi_and_grad(nqlib, shape, prec, tol):
    N = 6
    is_, net, onet, _ = make(N, shape, prec=prec)
    assert is_.engine.P == onet.n_params
    sig = np.random.default_rng(4).choice([-1, 1], size=(200, N)).astype(np.int8)
    lp, g = is_.engine.logpsi(sig, with_grad=True)
    olp, og = onet.logpsi_and_grad(sig.astype(float))
    d = lp - olp
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) / max(1.0, np.max(np.abs(olp))) < tol
    assert rel(g, og) < tol


@pytest.mark.parametrize("shape", ["dense_sum", "two_logcosh_sum"])
def test_chain_sampler_bitexact(nqlib, shape):
    N, B, L, burn = 6, 96, 3, 2
    is_, net, onet, ohilb = make(N, shape, B=B, L=L, burn=burn, sigma=0.4 ** 2)
    eng = is_.engine
    for call in (0, 3):
        samples, bits = eng.sample(call, want_accept_bits=True)
        ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, eng.passes, eng.cfg.seed, call=call,
                            gpu_accept_bits=bits)
        assert info["mismatch"] == 0
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


@pytest.mark.parametrize("prec", [nq._lib.NQ_EVAL_F32, nq._lib.NQ_EVAL_F64])
def test_chain_estimator_force_S_solve(nqlib, prec):
    N, B, L = 6, 64, 5
    is_, net, onet, ohilb = make(N, "two_logcosh_sum", B=B, L=L, burn=6, prec=prec, sigma=0.2 ** 2)
    samples, _ = is_.engine.sample(1)
    m, loc, force = is_.engine.estimate(want_loc=True, want_force=True)
    flat = samples.reshape(-1, N).astype(np.float64)
    H = oex.tfim_1d(ohilb, 1.0, 1.0)
    E = oest.local_energy(onet, H, flat)
    assert rel(loc.reshape(-1), E) < 2e-5
    st = ost.stat_analysis(E.reshape(L, B).T)
    assert abs(complex(m.mean_re, m.mean_im) - st["mean"]) < 1e-5 * max(1.0, abs(st["mean"]))
    _, O = onet.logpsi_and_grad(flat)
    F = oest.force_ket(E, O)
    assert rel(force, F) < 1e-4
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, real_params=False)
    assert rel(is_.engine.sr_matrix(), S) < 1e-4
    dw = is_.engine.precondition(0, 0.01)
    dwo = osr.precondition(S, F, 0.01, real_params=False)
    assert rel(dw, dwo) < 2e-3


def test_chain_chi_square(nqlib):
    from scipy.stats import chisquare
    N = 4
    is_, net, onet, ohilb = make(N, "two_logcosh_sum", B=16384, L=1, burn=40, sigma=0.3 ** 2, seed=6)
    samples, _ = is_.engine.sample(0)
    idx = ohilb.index_of_state(samples.reshape(-1, N).astype(np.float64))
    counts = np.bincount(idx, minlength=ohilb.dim)
    p = oex.ket_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3, (stat, pval)


@pytest.mark.parametrize("sp", [nq._lib.NQ_S_F32, nq._lib.NQ_S_TF32X3])
def test_chain_ffnn_vmc_lowers_energy(nqlib, sp):
    """examples/ising1d_ffnn.jl: Chain(Dense(N, 2N, af_logcosh), sum_autobatch)."""
    N = 8
    is_, net, onet, ohilb = make(N, "dense_sum", B=512, L=8, burn=10, passes=N + 1, sigma=0.05 ** 2, seed=3,
                                 sp=sp)
    e0 = oex.tfim_ground_energy_1d(N, 1.0, 1.0)
    first = is_.step(0.02)
    for _ in range(60):
        m = is_.step(0.02)
    assert m.mean.real < first.mean.real - 0.05 * abs(e0)
    assert m.mean.real > e0 - 5 * max(m.error, 1e-3)
    obs = nq.BatchedObsKetSampler(is_)
    nq.add_observable_(obs, "sx", nq.sigmax(nq.HomogeneousSpin(N), 1))
    res = obs.compute_observables()
    assert np.isfinite(res["sx"].mean.real)
