"""OperatorRule (src/Samplers/MCMCRules/OperatorRule.jl) in the θ-cache
Metropolis sampler, against the oracle, through the C-ABI.

* replay: the chains equal the oracle's OperatorRule replay (uniform
  connection of the configuration's rows, its changes, the factor
  n(σ)/n(σ')) bit for bit; near-ties |log u - Δ| < 1e-6 follow the device
  and no decision may disagree elsewhere.  Two operators: the TFIM (every
  operator's rows have one length, the constant-count path) and hopping plus
  a field (rows of 1 or 2 connections, the counted path); spin and Fock,
  logcosh and softplus;
* distribution: χ² of the samples against exact |ψ|², p > 1e-3, for both
  operators (the reference's own OperatorRule test, test_samplers.jl:60-63);
* a VMC run with the OperatorRule lowers the TFIM energy;
* a move operator without off-diagonal connections, and sampling without a
  move operator, are refused.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, exact as oex, sampler as osm, operators as oops
from oracle.hilbert import Hilbert, SPIN, FOCK

pytestmark = pytest.mark.gpu


def tfim(hilb, N, h=1.0, J=1.0):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - h * nq.sigmax(hilb, i)
        H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


def otfim(ohilb, N, h=1.0, J=1.0):
    H = oops.OpSum(ohilb)
    for i in range(N):
        H = H + oops.sigmax(ohilb, i).scale(-h)
        H = H + oops.prod(oops.sigmaz(ohilb, i), oops.sigmaz(ohilb, (i + 1) % N)).scale(J)
    return H


def hopping(hilb, N, t=1.0, g=0.4):
    H = nq.LocalOperator(hilb)
    for i in range(1, N):
        H = H + t * (nq.sigmap(hilb, i) * nq.sigmam(hilb, i + 1))
        H = H + t * (nq.sigmam(hilb, i) * nq.sigmap(hilb, i + 1))
    for i in range(1, N + 1):
        H = H + g * nq.sigmax(hilb, i)
    return H


def ohopping(ohilb, N, t=1.0, g=0.4):
    H = oops.OpSum(ohilb)
    for i in range(N - 1):
        H = H + oops.prod(oops.sigmap(ohilb, i), oops.sigmam(ohilb, i + 1)).scale(t)
        H = H + oops.prod(oops.sigmam(ohilb, i), oops.sigmap(ohilb, i + 1)).scale(t)
    for i in range(N):
        H = H + oops.sigmax(ohilb, i).scale(g)
    return H


def make(N, which, kind="spin", act=nq.af_logcosh, B=64, L=4, burn=3, passes=5, sigma=0.3 ** 2, seed=5):
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    net = nq.RBM(np.complex64, N, 2, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    move = tfim(hilb, N) if which == "tfim" else hopping(hilb, N)
    omove = otfim(ohilb, N) if which == "tfim" else ohopping(ohilb, N)
    smp = nq.MetropolisSampler(nq.OperatorRule(move), L, passes, burn=burn, seed=seed + 11)
    is_ = nq.BatchedSampler(net, smp, tfim(hilb, N), nq.SR(eps=0.01), batch_sz=B)
    onet = onw.RBM(N, net.M, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    return is_, onet, ohilb, omove


@pytest.mark.parametrize("which", ["tfim", "hopping"])
@pytest.mark.parametrize("kind,act", [("spin", nq.af_logcosh), ("fock", nq.af_softplus)])
def test_operator_rule_replays_bitexact(nqlib, which, kind, act):
    N, B, L, burn = 6, 64, 3, 2
    is_, onet, ohilb, omove = make(N, which, kind, act, B=B, L=L, burn=burn, sigma=0.4 ** 2)
    eng = is_.engine
    for call in (0, 5):
        samples, bits = eng.sample(call, want_accept_bits=True)
        ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, eng.passes, eng.cfg.seed, call=call,
                            gpu_accept_bits=bits, move_op=omove)
        assert info["mismatch"] == 0
        assert info["ambiguous"] <= 3
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


@pytest.mark.parametrize("which", ["tfim", "hopping"])
def test_operator_rule_chi_square(nqlib, which):
    from scipy.stats import chisquare
    N = 4
    is_, onet, ohilb, _ = make(N, which, B=16384, L=1, burn=60, passes=5, sigma=0.3 ** 2, seed=8)
    samples, _ = is_.engine.sample(0)
    idx = ohilb.index_of_state(samples.reshape(-1, N).astype(np.float64))
    counts = np.bincount(idx, minlength=ohilb.dim)
    p = oex.ket_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3, (stat, pval)


def test_vmc_with_operator_rule_lowers_energy(nqlib):
    N = 8
    is_, _, _, _ = make(N, "tfim", B=512, L=8, burn=10, passes=N + 1, sigma=0.01 ** 2, seed=3)
    e0 = oex.tfim_ground_energy_1d(N, 1.0, 1.0)
    first = is_.step(0.05)
    for _ in range(60):
        m = is_.step(0.05)
    assert m.mean.real < first.mean.real - 0.05 * abs(e0)
    assert m.mean.real > e0 - 5 * max(m.error, 1e-3)


def test_operator_rule_refusals(nqlib):
    N = 4
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, 1, nq.af_logcosh)
    diag = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        diag = diag + nq.sigmaz(hilb, i)
    smp = nq.MetropolisSampler(nq.OperatorRule(diag), 2, 3, burn=1, seed=1)
    with pytest.raises(nq._lib.NqError) as e:
        nq.BatchedSampler(net, smp, tfim(hilb, N), nq.SR(eps=0.01), batch_sz=16)
    assert e.value.status == nq._lib.NQ_ERR_ARG
    eng = nq.Engine(net, hilb, 16, 2, 1, 3, 7, rule=nq._lib.NQ_RULE_OPERATOR)
    eng.set_params(net.flat())
    with pytest.raises(nq._lib.NqError) as e:
        eng.sample(0)
    assert e.value.status == nq._lib.NQ_ERR_STATE
