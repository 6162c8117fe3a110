"""Exact sampler (NQ_SAMPLER_EXACT, src/Samplers/Exact.jl) on the GPU against
the oracle.

* replay: every draw is the oracle's inverse-CDF draw of the same Philox
  uniform on the FP64 distribution, except draws whose uniform lies within
  1e-6 of a CDF boundary (the GPU's CDF comes from FP32 log-probabilities);
  those may land on the neighbouring configuration and are counted (at most
  one in a thousand draws);
* distribution: χ² of the draws against exact |ψ|² (RBM) and |ρ(σ,η)|²
  (NDM doubled space), p > 1e-3;
* the stale-last-slot quirk keeps slot L-1 as for the Metropolis sampler;
* a VMC run with exact sampling lowers the energy of a small TFIM toward the
  exact ground state.
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


def make_rbm(N=8, alpha=2, act=nq.af_logcosh, kind="spin", B=64, L=6, sigma=0.3 ** 2, seed=13,
             quirks=False):
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    net = nq.RBM(np.complex64, N, alpha, act)
    nq.init_random_pars_(net, sigma=sigma, rng=np.random.default_rng(seed))
    s = nq.ExactSampler(L, seed=seed * 5 + 3)
    is_ = nq.BatchedSampler(net, s, tfim(hilb, N), nq.SR(eps=0.01), batch_sz=B, reference_quirks=quirks)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    onet = onw.RBM(N, net.M, onw.LOGCOSH if act == nq.af_logcosh else onw.SOFTPLUS)
    onet.set_flat(net.flat())
    return is_, onet, ohilb


@pytest.mark.parametrize("kind", ["spin", "fock"])
@pytest.mark.parametrize("act", [nq.af_logcosh, nq.af_softplus])
def test_exact_sampler_replays_inverse_cdf(nqlib, kind, act):
    N, B, L = 8, 64, 6
    is_, onet, ohilb = make_rbm(N=N, kind=kind, act=act, B=B, L=L)
    p = oex.ket_distribution(onet, ohilb)
    for call in (0, 7):
        samples, _ = is_.engine.sample(call)
        gpu = ohilb.index_of_state(samples.astype(np.float64))          # (L, B)
        ref, ties = osm.exact_run(p, B, L, is_.engine.cfg.seed, call=call, gpu_samples=gpu)
        np.testing.assert_array_equal(gpu, ref)
        assert ties <= max(1, B * L // 1000)


def test_exact_sampler_stale_last_slot(nqlib):
    N, B, L = 6, 32, 4
    is_, onet, ohilb = make_rbm(N=N, B=B, L=L, quirks=True)
    samples, _ = is_.engine.sample(2)
    assert np.all(samples[L - 1] == -1)              # state() fill, local index 0
    p = oex.ket_distribution(onet, ohilb)
    gpu = ohilb.index_of_state(samples.astype(np.float64))
    ref, _ = osm.exact_run(p, B, L, is_.engine.cfg.seed, call=2, stale_last_slot=True,
                           prev_samples=gpu, gpu_samples=gpu)
    np.testing.assert_array_equal(gpu[:L - 1], ref[:L - 1])


def test_exact_sampler_chi_square_rbm(nqlib):
    from scipy.stats import chisquare
    N, B, L = 6, 512, 20
    is_, onet, ohilb = make_rbm(N=N, B=B, L=L, sigma=0.25 ** 2)
    samples, _ = is_.engine.sample(1)
    idx = ohilb.index_of_state(samples.reshape(-1, N).astype(np.float64))
    counts = np.bincount(idx, minlength=ohilb.dim)
    p = oex.ket_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3


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


def test_exact_sampler_chi_square_ndm(nqlib):
    from scipy.stats import chisquare
    N, B, L = 3, 512, 16
    hilb = nq.HomogeneousFock(N)
    net = nq.NDM(np.float64, N, 1, 1, nq.af_softplus)
    nq.init_random_pars_(net, sigma=0.4 ** 2, rng=np.random.default_rng(4))
    is_ = nq.BatchedSampler(net, nq.ExactSampler(L, seed=17), dissipative(hilb, N), nq.SR(eps=0.01),
                            batch_sz=B)
    samples, _ = is_.engine.sample(0)
    ohilb = Hilbert(N, FOCK)
    onet = onw.NDM(N, 1, 1, onw.SOFTPLUS)
    onet.set_flat(net.flat())
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    idx = ohilb.index_of_state(flat[:, N:]) * ohilb.dim + ohilb.index_of_state(flat[:, :N])
    counts = np.bincount(idx, minlength=ohilb.dim ** 2)
    p = oex.doubled_distribution(onet, ohilb)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3


def test_vmc_with_exact_sampler_lowers_energy(nqlib):
    N, B, L = 8, 256, 8
    is_, onet, ohilb = make_rbm(N=N, B=B, L=L, sigma=0.01 ** 2, seed=3)
    e0 = oex.tfim_ground_energy_1d(N, 1.0, 1.0)
    first = is_.step(0.05)
    for _ in range(60):
        m = is_.step(0.05)
    assert m.mean.real < first.mean.real - 0.05 * abs(e0)
    assert m.mean.real > e0 - 5 * max(m.error, 1e-3)
