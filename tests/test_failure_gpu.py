"""Failure paths of the C-ABI, injected from the host (no GPU fault, trap or
hang is provoked):

* non-finite parameters are refused by nq_set_params (NQ_ERR_NAN);
* finite parameters whose amplitudes overflow make the estimator's mean
  non-finite, which nq_estimate reports as NQ_ERR_NAN;
* a negative diagonal shift makes the shifted S indefinite: the inversion
  meets a non-positive pivot and nq_precondition reports NQ_ERR_NOT_PD;
* a 1 ns limit on the solve's grid-barrier waits (nq_set_wait_limit) makes
  them give up: the kernels return early and nq_precondition reports
  NQ_ERR_TIMEOUT.
After each failure the handle is used again with sane inputs and must give
the FP64 solve of its own S and F (relative 1e-9)."""
import numpy as np
import pytest

import nqcuda as nq

pytestmark = pytest.mark.gpu


def _engine(N=8, B=256, L=8):
    hilb = nq.HomogeneousSpin(N)
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.05 ** 2, rng=np.random.default_rng(8))
    s = nq.MetropolisSampler(nq.LocalRule(), L, N, burn=5, seed=21)
    return nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B, s_precision=nq._lib.NQ_S_F32).engine, net


def _sane_solve(eng):
    eng.sample(11, want_samples=False)
    _, _, F = eng.estimate(want_force=True)
    S = eng.sr_matrix()
    dw = eng.precondition(0, 0.01)
    x = np.linalg.solve(S + 0.01 * np.eye(S.shape[0]), F)
    assert np.max(np.abs(dw - x)) < 1e-9 * np.max(np.abs(x))
    corr, last = eng.sr_info()
    assert 1 <= corr <= 12 and last <= 1e-13


def _status(fn):
    try:
        fn()
    except nq._lib.NqError as e:
        return e.status
    return nq._lib.NQ_OK


def test_nonfinite_parameters_refused(nqlib):
    eng, net = _engine()
    p = net.flat().astype(np.complex128)
    for bad in (np.nan, np.inf):
        q = p.copy()
        q[3] = bad
        assert _status(lambda: eng.set_params(q)) == nq._lib.NQ_ERR_NAN
    eng.set_params(p)
    _sane_solve(eng)


def test_overflowing_amplitudes_give_nan_status(nqlib):
    eng, net = _engine()
    p = net.flat().astype(np.complex128)
    eng.set_params(p * 3e4)                     # θ ~ 1e4: ψ'/ψ overflows in the estimator
    eng.sample(3, want_samples=False)
    assert _status(lambda: eng.estimate()) == nq._lib.NQ_ERR_NAN
    eng.set_params(p)
    _sane_solve(eng)


def test_indefinite_shifted_matrix_not_pd(nqlib):
    eng, _ = _engine()
    eng.sample(5, want_samples=False)
    eng.estimate()
    assert _status(lambda: eng.precondition(0, -10.0)) == nq._lib.NQ_ERR_NOT_PD
    _sane_solve(eng)


def test_solve_wait_limit_times_out_and_recovers(nqlib):
    eng, _ = _engine()
    eng.sample(5, want_samples=False)
    eng.estimate()
    eng.set_wait_limit(1)
    assert _status(lambda: eng.precondition(0, 0.01)) == nq._lib.NQ_ERR_TIMEOUT
    eng.set_wait_limit(0)
    _sane_solve(eng)
