"""Stochastic reconfiguration and the Descent update (test infrastructure,
see ``oracle/__init__``).

* ``setup_algorithm!(SRDirectCache)`` SRDirect.jl:26-48: Sc = O_c O_c†;
  complex parameters: S = conj(Sc)/Ns, F unchanged; real parameters:
  S = real(Sc)/Ns, F = real(F).
* ``precondition!`` SRDirect.jl:51-90: ``sr_shift`` adds ϵ to the diagonal
  of S in place; ``sr_multiplicative`` forms Sprecond = S + max(λ0 bⁿ, λmin)
  diag(S); ``sr_diag`` solves with pinv(Sprecond); ``sr_cholesky`` (Cholesky of
  the upper triangle, ``Hermitian(S)``) and ``sr_div`` (``ldiv!`` with
  ``Hermitian(S)``) solve with S itself, so the reference's multiplicative
  shift reaches only ``sr_diag`` (:70-83); ``follow_reference=True`` restates
  that exactly, the default applies the preconditioned matrix to every
  algorithm.
* ``Optimisers.update!(Descent(η))`` Optimisers/apply.jl:25-32 and
  rules.jl:15-17: w .-= η Δw.
"""
import numpy as np
import scipy.linalg as sla


def build_S(O_centered, real_params):
    ns = O_centered.shape[0]
    Sc = O_centered.T @ np.conj(O_centered)          # (P, P) = O Oᴴ with O as (P, Ns)
    if real_params:
        return np.real(Sc) / ns
    return np.conj(Sc) / ns


def precondition(S, F, eps, kind="shift", lam0=100.0, b=0.95, lam_min=1e-4, it=1,
                 real_params=False, algorithm="cholesky", follow_reference=False):
    S = S.copy()
    if real_params:
        F = np.real(F)
    if kind == "shift":
        S[np.diag_indices_from(S)] += eps
    Sp = S
    if kind == "multiplicative":
        lam = max(lam0 * b ** it, lam_min)
        Sp = S + lam * np.diag(np.diag(S))
    if algorithm == "diag":
        return np.linalg.pinv(Sp) @ F
    A = S if follow_reference else Sp
    U = np.triu(A)
    Ah = U + np.conj(np.triu(A, 1)).T               # Hermitian(A) uses the upper triangle
    if algorithm == "div":
        return sla.solve(Ah, F, assume_a="her")
    c = sla.cho_factor(Ah, lower=False)
    return sla.cho_solve(c, F)


def descent(w, dw, lr):
    return w - lr * dw
