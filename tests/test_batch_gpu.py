"""Many-problem SR steps (nq_batch_*) against the single-problem path.

The batched sampler, estimator and inversion run the same arithmetic per
problem as the single-problem kernels (the sampler's chains follow the same
Philox counters for any lane layout), and the grouped SR stages (one launch
per stage for all problems, the S accumulation over one stacked X) sum the
same products with another split of the sample range, so one batched step
must reproduce one step of each problem run on its own: energies to 1e-6
relative and updated parameters to 1e-5 relative of their largest magnitude.
"""
import numpy as np
import pytest

import nqcuda as nq

pytestmark = pytest.mark.gpu


def tfim2d(L, h, J=1.0):
    N = L * L
    hilb = nq.HomogeneousSpin(N)
    H = nq.LocalOperator(hilb)
    for x in range(L):
        for y in range(L):
            i = x + L * y + 1
            H = H - h * nq.sigmax(hilb, i)
            H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, (x + 1) % L + L * y + 1)
            H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, x + L * ((y + 1) % L) + 1)
    return hilb, H


def problems(spec, seed=3):
    out = []
    for k, (L, h) in enumerate(spec):
        hilb, H = tfim2d(L, h)
        net = nq.RBM(np.complex64, L * L, 1, nq.af_logcosh)
        nq.init_random_pars_(net, sigma=0.05, rng=np.random.default_rng(seed + k))
        out.append((net, hilb, H))
    return out


def test_batch_step_matches_single_problems(nqlib):
    spec = [(3, 2.5), (4, 3.1), (5, 2.2), (3, 3.9), (4, 2.0), (5, 3.5)]
    B, Lc, burn = 128, 4, 5
    probs = problems(spec)
    batch = nq.ProblemBatch(probs, B, Lc, burn, s_precision=nq._lib.NQ_S_F32)
    ms = batch.vmc_step(7, 0.01, 0.05)
    seed = 0x4E51
    for i, (net, hilb, H) in enumerate(probs):
        N = hilb.n_sites
        smp = nq.MetropolisSampler(nq.LocalRule(), Lc, N, burn=burn, seed=seed + 7919 * i)
        single = nq.BatchedSampler(net, smp, H, nq.SR(eps=0.01), batch_sz=B, s_precision=nq._lib.NQ_S_F32).engine
        m = single.vmc_step(7, 0.01, 0.05)
        assert abs(ms[i].mean_re - m.mean_re) <= 1e-6 * abs(m.mean_re)
        assert abs(ms[i].acceptance - m.acceptance) < 1e-12
        pb, ps = batch.engines[i].get_params(), single.get_params()
        assert np.max(np.abs(pb - ps)) <= 1e-5 * np.max(np.abs(ps))


def test_batch_of_64_uneven_problems_steps(nqlib):
    rng = np.random.default_rng(1)
    spec = [(int(rng.choice([3, 4, 5])), float(rng.uniform(2.0, 4.0))) for _ in range(64)]
    hs = np.array([h for _, h in spec])
    batch = nq.ProblemBatch(problems(spec), 1024, 4, 10)
    energies = []
    for it in range(6):
        ms = batch.vmc_step(it, 0.01, 0.05)
        e = np.array([m.mean_re / (L * L) for m, (L, _) in zip(ms, spec)])
        err = np.array([m.error / (L * L) for m, (L, _) in zip(ms, spec)])
        assert np.all(np.isfinite(e))
        # variational bound: every site term is at least -h, every bond term at least -J
        assert np.all(e >= -(hs + 2.0) - 6 * err)
        energies.append(e)
    # SR lowers the energy of (almost) every problem
    assert np.mean(energies[-1] < energies[0]) > 0.9
    t = batch.tuning()
    assert t["sampler_lanes"] in (4, 8, 16, 32) and t["inversion_ctas"] >= 64
    assert batch.kernel_launches() > 0
    # every stage of the 64 problems is one grouped launch: a handful of kernels per step
    assert t["kernels_per_step"] <= 20, t
