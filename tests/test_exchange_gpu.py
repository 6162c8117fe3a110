"""ExchangeRule (src/Samplers/MCMCRules/ExchangeRule.jl) in the θ-cache
sampler against the oracle replay.

* replay: configurations bit-exact against ``oracle.sampler.run`` with the
  same couplings and Philox draws; accept decisions identical except
  near-ties |log u - Δ| < 1e-6 (counted);
* conservation: a chain's magnetisation never changes;
* distribution: within the magnetisation sector of each chain, χ² against
  |ψ|² restricted to that sector (p > 1e-3);
* couplings: ExchangeRule(H) takes the 2-site terms of H in term order.
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, exact as oex, sampler as osm
from oracle.hilbert import Hilbert, SPIN, FOCK

pytestmark = pytest.mark.gpu


def tfim(hilb, N, h=1.0, J=1.0):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - h * nq.sigmax(hilb, i)
        H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


def make(N=8, alpha=2, act=nq.af_logcosh, kind="spin", B=96, L=5, burn=3, passes=None, sigma=0.3 ** 2,
         seed=21):
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    net = nq.RBM(np.complex64, N, alpha, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    H = tfim(hilb, N)
    rule = nq.ExchangeRule(H)
    s = nq.MetropolisSampler(rule, L, passes or N, burn=burn, seed=seed * 3 + 1)
    is_ = nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    onet = onw.RBM(N, net.M, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    return is_, rule, onet, ohilb


def test_exchange_couplings_from_operator(nqlib):
    hilb = nq.HomogeneousSpin(4)
    rule = nq.ExchangeRule(tfim(hilb, 4))
    assert rule.couplings == [(0, 1), (1, 2), (2, 3), (0, 3)]


@pytest.mark.parametrize("kind", ["spin", "fock"])
@pytest.mark.parametrize("act", [nq.af_logcosh, nq.af_softplus])
def test_exchange_sampler_bitexact_replay(nqlib, kind, act):
    N, B, L, burn = 8, 96, 5, 3
    is_, rule, onet, ohilb = make(N=N, kind=kind, act=act, B=B, L=L, burn=burn)
    for call in (0, 4):
        samples, bits = is_.engine.sample(call, want_accept_bits=True)
        ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, is_.engine.passes, is_.engine.cfg.seed,
                            call=call, gpu_accept_bits=bits, couplings=rule.couplings)
        assert info["mismatch"] == 0
        assert info["ambiguous"] <= 3
        np.testing.assert_array_equal(samples.astype(np.float64), ref)


def test_exchange_conserves_magnetisation_and_samples_the_sector(nqlib):
    from scipy.stats import chisquare
    N, B, L = 6, 4096, 8
    is_, rule, onet, ohilb = make(N=N, B=B, L=L, burn=20, passes=4 * N + 1, sigma=0.3 ** 2, seed=5)
    samples, _ = is_.engine.sample(0)
    mag = samples.sum(axis=2)                                   # (L, B)
    assert np.all(mag == mag[0][None, :])
    # the most populated sector: |ψ|² restricted to it
    vals, counts = np.unique(mag[0], return_counts=True)
    m0 = vals[np.argmax(counts)]
    sel = samples[:, mag[0] == m0, :].reshape(-1, N).astype(np.float64)
    states = ohilb.all_states()
    in_sector = states.sum(axis=1) == m0
    p = oex.ket_distribution(onet, ohilb)[in_sector]
    p = p / p.sum()
    idx_all = ohilb.index_of_state(sel)
    sector_index = -np.ones(ohilb.dim, dtype=np.int64)
    sector_index[np.nonzero(in_sector)[0]] = np.arange(in_sector.sum())
    counts = np.bincount(sector_index[idx_all], minlength=int(in_sector.sum()))
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3
