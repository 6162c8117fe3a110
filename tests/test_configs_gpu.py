"""Parity at the configurations the measurements are quoted on, against the
FP64 oracle (never GPU against GPU).

* 1D TFIM N = 20, complex RBM α = 2, 4096 chains x 20 samples (the bench
  workload): bit-exact chains against the Philox replay of all 4096 chains;
  logψ, E_loc, F, S and Δw on all 81 920 samples.
* Dissipative Ising N = 12, NDM α = β = 2, 16384 chains x 8 samples (the
  precision-mode workload): bit-exact replay of 1024 of the chains; L_loc of
  a 4096-sample subset of the full run; S on all 131 072 samples; L_loc, the
  cost, F, S and Δw of a handle holding that subset.
* Three problems (L = 3, 4, 5) of the 64-problem 2D TFIM batch: samples,
  E_loc, F, S and Δw of the batched step itself, read back from the problem
  handles.
* Dissipative Ising N = 6, NDM α = β = 1, FP64 evaluation, 16 chains x 63
  samples, burn 100, 200 SR steps (shift 0.01, lr 0.01): every step's cost,
  F and Δw against the oracle evaluated at the engine's parameters, the cost
  curve against an oracle trajectory run from the same start on the same
  samples, bit-exact chains at the first and last step, the estimator against
  exact summation over all 4^6 doubled states, and the trained state against
  the exact steady state of the 4096-dim Liouvillian.

Tolerances are stated per assertion (relative to the largest magnitude of
the reference quantity unless said otherwise).  The SR solve is checked in
two ways: against the FP64 solve of the engine's own S and F (the solver's
own error, 1e-9) and against the oracle's Δw (which adds the error of S).
"""
import numpy as np
import pytest

import nqcuda as nq
from oracle import networks as onw, estimators as oest, exact as oex, sampler as osm, sr as osr, \
    operators as oops, stats as ost
from oracle.hilbert import Hilbert, SPIN

pytestmark = pytest.mark.gpu

SEED = 0x4E51


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b))))


def own_solve(S, F, eps):
    """FP64 solve of the shifted system the engine holds (its own S and F)."""
    return np.linalg.solve(S + eps * np.eye(S.shape[0]), F)


def tfim1d(hilb, N, h=1.0, J=1.0):
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - h * nq.sigmax(hilb, i)
        H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    return H


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


# ---------------------------------------------------------------------------
# 1D TFIM N = 20, RBM α = 2, 4096 x 20
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("sp,s_tol", [(nq._lib.NQ_S_TF32, 2e-3), (nq._lib.NQ_S_F32, 2e-5)])
def test_tfim_n20_rbm_4096x20_against_oracle(nqlib, sp, s_tol):
    N, M, B, L, burn, passes = 20, 40, 4096, 20, 50, 20
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(SEED))
    smp = nq.MetropolisSampler(nq.LocalRule(), L, passes, burn=burn, seed=SEED)
    eng = nq.BatchedSampler(net, smp, tfim1d(hilb, N), nq.SR(eps=0.01), batch_sz=B, s_precision=sp).engine
    samples, bits = eng.sample(1, want_accept_bits=True)
    onet = onw.RBM(N, M, onw.LOGCOSH)
    onet.set_flat(eng.get_params())
    ohilb = Hilbert(N, SPIN)
    # all 4096 chains bit-exact against the replay (FP32 Δ: near-ties within 1e-5 follow the device)
    ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, eng.passes, SEED, call=1, gpu_accept_bits=bits,
                        tie_tol=1e-5)
    assert info["mismatch"] == 0, info
    np.testing.assert_array_equal(samples.astype(np.float64), ref)

    m, loc, F = eng.estimate(want_loc=True, want_force=True)
    S = eng.sr_matrix()
    dw = eng.precondition(0, 0.01)
    flat = samples.reshape(-1, N).astype(np.float64)
    ns = flat.shape[0]
    sub = np.random.default_rng(1).choice(ns, 8192, replace=False)
    lp = eng.logpsi(samples.reshape(-1, N)[sub])
    d = lp - onet.logpsi(flat[sub])
    d = d.real + 1j * ((d.imag + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(np.abs(d)) < 2e-5 * np.max(np.abs(lp))                        # logψ, FP32
    oH = oex.tfim_1d(ohilb, 1.0, 1.0)
    E = oest.local_energy_batched(onet, oH, flat)
    assert rel(loc.reshape(-1), E) < 2e-5                                       # E_loc, FP32
    st = ost.stat_analysis(E.reshape(L, B).T)
    assert abs(m.mean_re - st["mean"].real) < 1e-6 * abs(st["mean"])
    assert abs(m.error - st["error"]) < 1e-3 * st["error"]
    gf = lambda a, b: onet.logpsi_and_grad(flat[a:b])[1]
    Fo = oest.force_ket_batched(E, gf, ns)
    So, _ = oest.sr_matrix_batched(gf, ns, False)
    assert rel(F, Fo) < 1e-4                                                    # F, FP32 chunks + FP64
    assert rel(S, So) < s_tol                                                   # S, per precision mode
    assert rel(dw, own_solve(S, F, 0.01)) < 1e-9                                # the solve itself: FP64
    dwo = osr.precondition(So, Fo, 0.01)
    assert rel(dw, dwo) < (0.1 if sp == nq._lib.NQ_S_TF32 else 2e-3)            # Δw with the S error


# ---------------------------------------------------------------------------
# Dissipative Ising N = 12, NDM α = β = 2, 16384 x 8
# ---------------------------------------------------------------------------
def test_dissipative_n12_ndm_16384x8_against_oracle(nqlib):
    N, B, L, burn = 12, 16384, 8, 100
    hilb = nq.HomogeneousSpin(N)
    lv = dissipative(hilb, N)
    net = nq.NDM(np.float64, N, 2, 2, nq.af_softplus)
    nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(SEED))
    smp = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=burn, seed=SEED)
    eng = nq.BatchedSampler(net, smp, lv, nq.SR(eps=0.01), batch_sz=B,
                            s_precision=nq._lib.NQ_S_TF32).engine
    samples, bits = eng.sample(3, want_accept_bits=True)
    ohilb = Hilbert(N, SPIN)
    onet = onw.NDM(N, 2, 2, onw.SOFTPLUS)
    onet.set_flat(eng.get_params())
    oH, oLs = oex.dissipative_ising(ohilb, 1.0, 2.0)
    olv = oops.liouvillian(oH, oLs)
    lp = lambda x: onet.log_prob(x[:, :N], x[:, N:])
    nrep = 1024                       # replay of the first 1024 chains (their accept bits)
    ref, info = osm.run(lp, ohilb, nrep, L, burn, eng.passes, SEED, call=3, doubled=True,
                        gpu_accept_bits=bits[:, :nrep], tie_tol=1e-5)
    assert info["mismatch"] == 0, info
    np.testing.assert_array_equal(samples[:, :nrep].astype(np.float64), ref)

    m, loc, F = eng.estimate(want_loc=True, want_force=True)
    S = eng.sr_matrix()
    flat = samples.reshape(-1, 2 * N).astype(np.float64)
    ns = flat.shape[0]
    sub = np.sort(np.random.default_rng(2).choice(ns, 4096, replace=False))
    Lsub, _, _, _ = oest.liouvillian_force_batched(onet, olv, flat[sub, :N], flat[sub, N:])
    assert rel(loc.reshape(-1)[sub], Lsub) < 2e-5                                # L_loc, FP32
    gf = lambda a, b: onet.logpsi_and_grad(flat[a:b, :N], flat[a:b, N:])[1]
    So, _ = oest.sr_matrix_batched(gf, ns, True)
    assert rel(S, So) < 2e-3                                                     # S, TF32, all samples
    dw = eng.precondition(0, 0.01)
    assert rel(dw, own_solve(S, F, 0.01)) < 1e-9                                 # the solve itself

    # the whole estimate on the 4096-sample subset, on a handle holding it
    eng2 = nq.BatchedSampler(net, nq.MetropolisSampler(nq.LocalRule(), 8, 2 * N, burn=burn, seed=SEED), lv,
                             nq.SR(eps=0.01), batch_sz=512, s_precision=nq._lib.NQ_S_F32).engine
    eng2.set_params(eng.get_params())
    eng2.set_samples(flat[sub].reshape(8, 512, 2 * N).astype(np.int8))
    m2, loc2, F2 = eng2.estimate(want_loc=True, want_force=True)
    S2 = eng2.sr_matrix()
    dw2 = eng2.precondition(0, 0.01)
    Lo, C, Fo, _ = oest.liouvillian_force_batched(onet, olv, flat[sub, :N], flat[sub, N:])
    gs = lambda a, b: onet.logpsi_and_grad(flat[sub][a:b, :N], flat[sub][a:b, N:])[1]
    So2, _ = oest.sr_matrix_batched(gs, sub.size, True)
    assert rel(loc2.reshape(-1), Lo) < 2e-5
    assert abs(m2.mean_re - C) < 1e-5 * C                                        # cost, FP64 mean
    assert rel(F2, np.real(Fo)) < 1e-4
    assert rel(S2, So2) < 1e-4                                                   # FP32 S
    assert rel(dw2, own_solve(S2, F2, 0.01)) < 1e-9
    assert rel(dw2, osr.precondition(So2, Fo, 0.01, real_params=True)) < 2e-3


# ---------------------------------------------------------------------------
# Three problems of the 64-problem 2D TFIM batch
# ---------------------------------------------------------------------------
def test_batch_problems_against_oracle(nqlib):
    rng = np.random.default_rng(1)
    spec = [(int(rng.choice((3, 4, 5))), float(rng.uniform(2.0, 4.0))) for _ in range(64)]
    probs = []
    for k, (Lx, h) in enumerate(spec):
        n = Lx * Lx
        hilb = nq.HomogeneousSpin(n)
        H = nq.LocalOperator(hilb)
        for x in range(Lx):
            for y in range(Lx):
                i = x + Lx * y + 1
                H = H - h * nq.sigmax(hilb, i)
                H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, (x + 1) % Lx + Lx * y + 1)
                H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, x + Lx * ((y + 1) % Lx) + 1)
        net = nq.RBM(np.complex64, n, 1, nq.af_logcosh)
        nq.init_random_pars_(net, sigma=0.01, rng=np.random.default_rng(100 + k))
        probs.append((net, hilb, H))
    B, L, burn = 1024, 20, 50
    batch = nq.ProblemBatch(probs, B, L, burn)
    picks = [next(k for k, (Lx, _) in enumerate(spec) if Lx == s) for s in (3, 4, 5)]
    p0 = {k: batch.engines[k].get_params() for k in picks}
    lr = 0.01
    batch.vmc_step(4, 0.01, lr)
    for k in picks:
        e = batch.engines[k]
        Lx, h = spec[k]
        n = Lx * Lx
        samples = e.get_samples()
        loc, F, dw = e.get_estimates()
        S = e.sr_matrix()
        onet = onw.RBM(n, n, onw.LOGCOSH)
        onet.set_flat(p0[k])
        ohilb = Hilbert(n, SPIN)
        ref, info = osm.run(onet.log_prob, ohilb, B, L, burn, e.passes, e.cfg.seed, call=4, tie_tol=1e-5)
        # without the device's accept bits: disagreements are allowed only at |log u - Δ| < 1e-5
        np.testing.assert_array_equal(samples.astype(np.float64), ref)
        flat = samples.reshape(-1, n).astype(np.float64)
        oH = oex.tfim_2d(ohilb, Lx, Lx, h, 1.0)
        E = oest.local_energy_batched(onet, oH, flat)
        assert rel(loc.reshape(-1), E) < 2e-5
        gf = lambda a, b: onet.logpsi_and_grad(flat[a:b])[1]
        Fo = oest.force_ket_batched(E, gf, flat.shape[0])
        So, _ = oest.sr_matrix_batched(gf, flat.shape[0], False)
        assert rel(F, Fo) < 1e-4
        assert rel(S, So) < 2e-3                                                 # TF32 S
        assert rel(dw, own_solve(S, F, 0.01)) < 1e-9
        np.testing.assert_allclose(e.get_params(), p0[k] - lr * dw, rtol=0, atol=1e-12)


# ---------------------------------------------------------------------------
# Dissipative Ising N = 6, NDM α = β = 1, FP64, 200 SR steps
# ---------------------------------------------------------------------------
def _exact_parts(onet, olv, ohilb, Lm):
    """ρ over all doubled states (column-major vec), (Lρ)/ρ, the exact cost."""
    D = ohilb.dim
    st = ohilb.all_states()
    sr = np.repeat(st[None], D, axis=0).reshape(-1, ohilb.n_sites)     # row index fastest
    sc = np.repeat(st, D, axis=0)
    v = np.exp(onet.logpsi(sr, sc))
    Lv = Lm @ v
    return sr, sc, v, Lv, float(np.sum(np.abs(Lv) ** 2) / np.sum(np.abs(v) ** 2))


def test_dissipative_n6_ndm_200_sr_steps(nqlib):
    N, B, L, burn, steps, eps, lr = 6, 16, 63, 100, 200, 0.01, 0.01
    hilb = nq.HomogeneousSpin(N)
    lv = dissipative(hilb, N)
    net = nq.NDM(np.float64, N, 1, 1, nq.af_softplus)
    nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(SEED))
    smp = nq.MetropolisSampler(nq.LocalRule(), L, 2 * N, burn=burn, seed=SEED)
    is_ = nq.BatchedSampler(net, smp, lv, nq.SR(eps=eps), batch_sz=B, eval_precision=nq._lib.NQ_EVAL_F64,
                            s_precision=nq._lib.NQ_S_F32)
    eng = is_.engine
    assert eng.passes == 13
    ohilb = Hilbert(N, SPIN)
    oH, oLs = oex.dissipative_ising(ohilb, 1.0, 2.0)
    olv = oops.liouvillian(oH, oLs)
    Lm = oops.liouvillian_to_matrix(olv)
    onet = onw.NDM(N, 1, 1, onw.SOFTPLUS)         # evaluated at the engine's parameters
    otraj = onw.NDM(N, 1, 1, onw.SOFTPLUS)        # independent trajectory from the same start
    otraj.set_flat(eng.get_params())
    cost_gpu, cost_traj, cost_exact = [], [], []
    worst = {"cost": 0.0, "F": 0.0, "dw": 0.0, "dw_own": 0.0, "traj_cost": 0.0}
    for k in range(steps):
        p = eng.get_params()
        onet.set_flat(p)
        want_bits = k in (0, steps - 1)
        samples, bits = eng.sample(k, want_accept_bits=want_bits)
        flat = samples.reshape(-1, 2 * N).astype(np.float64)
        if want_bits:
            ref, info = osm.run(lambda x: onet.log_prob(x[:, :N], x[:, N:]), ohilb, B, L, burn, eng.passes,
                                SEED, call=k, doubled=True, gpu_accept_bits=bits, tie_tol=1e-9)
            assert info["mismatch"] == 0, info
            np.testing.assert_array_equal(samples.astype(np.float64), ref)
        m, loc, F = eng.estimate(want_loc=True, want_force=True)
        S = eng.sr_matrix()
        dw = eng.precondition(0, eps)
        eng.update_descent(lr)
        cost_gpu.append(m.mean_re)
        # the oracle at the engine's parameters, same samples
        if k % 10 == 0 or k == steps - 1:
            Lo, C, Fo, _ = oest.liouvillian_force_batched(onet, olv, flat[:, :N], flat[:, N:])
            gf = lambda a, b: onet.logpsi_and_grad(flat[a:b, :N], flat[a:b, N:])[1]
            So, _ = oest.sr_matrix_batched(gf, flat.shape[0], True)
            worst["cost"] = max(worst["cost"], abs(m.mean_re - C) / C)
            worst["F"] = max(worst["F"], rel(F, np.real(Fo)))
            worst["dw"] = max(worst["dw"], rel(dw, osr.precondition(So, Fo, eps, real_params=True)))
            worst["dw_own"] = max(worst["dw_own"], rel(dw, own_solve(S, F, eps)))
            cost_exact.append(_exact_parts(onet, olv, ohilb, Lm)[4])
        # the oracle's own trajectory on the same samples
        To, Ct, Ft, _ = oest.liouvillian_force_batched(otraj, olv, flat[:, :N], flat[:, N:])
        gt = lambda a, b: otraj.logpsi_and_grad(flat[a:b, :N], flat[a:b, N:])[1]
        St, _ = oest.sr_matrix_batched(gt, flat.shape[0], True)
        cost_traj.append(Ct)
        worst["traj_cost"] = max(worst["traj_cost"], abs(m.mean_re - Ct) / Ct)
        otraj.set_flat(otraj.flat() - lr * osr.precondition(St, Ft, eps, real_params=True))
    print("C0 worst relative differences:", worst)
    print("C0 cost (sampled) first/last:", cost_gpu[0], cost_gpu[-1], "exact first/last:", cost_exact[0],
          cost_exact[-1])
    assert worst["cost"] < 1e-10                 # FP64 evaluation and mean
    assert worst["F"] < 1e-5                     # F: FP64 evaluation, FP32 O in the estimator's sums
    assert worst["dw_own"] < 1e-9                # the solve itself
    assert worst["dw"] < 1e-3                    # Δw with the FP32 S error
    assert worst["traj_cost"] < 1e-4             # cost curve of an independent oracle run
    np.testing.assert_allclose(eng.get_params(), otraj.flat(), rtol=0, atol=1e-4)

    # exact summation over all 4^6 doubled states at the final parameters
    onet.set_flat(eng.get_params())
    sr, sc, v, Lv, c_exact = _exact_parts(onet, olv, ohilb, Lm)
    full = nq.BatchedSampler(net, nq.MetropolisSampler(nq.LocalRule(), 64, 2 * N, burn=1, seed=1), lv,
                             nq.SR(eps=eps), batch_sz=64, eval_precision=nq._lib.NQ_EVAL_F64).engine
    full.set_params(eng.get_params())
    states = np.concatenate([sr, sc], axis=1).reshape(64, 64, 2 * N).astype(np.int8)
    full.set_samples(states)
    _, lall, _ = full.estimate(want_loc=True)
    assert rel(lall.reshape(-1), Lv / v) < 1e-10                                  # L_loc = (Lρ)/ρ
    p = np.abs(v) ** 2 / np.sum(np.abs(v) ** 2)
    assert abs(np.sum(p * np.abs(lall.reshape(-1)) ** 2) - c_exact) < 1e-10 * c_exact

    # the sampled cost of the last steps agrees with the exact cost there
    mlast = ost.stat_analysis(np.abs(loc.reshape(L, B).T) ** 2)
    assert abs(cost_gpu[-1] - cost_exact[-1]) < 6 * mlast["error"] + 1e-12
    # training lowers the exact cost and moves ρ towards the exact steady state
    assert cost_exact[-1] < 0.5 * cost_exact[0]
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    w, vec = spla.eigs(sps.csc_matrix(Lm), k=1, sigma=0.0)
    D = ohilb.dim
    rho_ss = vec[:, 0].reshape(D, D).T                                           # vec is column-major
    rho_ss = rho_ss / np.trace(rho_ss)
    rho = v.reshape(D, D).T
    rho = rho / np.trace(rho)
    rho0 = np.eye(D) / D
    d_final = np.linalg.norm(rho - rho_ss)
    d_start = np.linalg.norm(rho0 - rho_ss)
    print("C0 |ρ - ρ_ss|_F start/final:", d_start, d_final, "|λ_0| =", abs(w[0]))
    assert abs(w[0]) < 1e-8
    assert d_final < d_start
