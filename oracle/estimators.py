"""Local estimators and cost gradients (test infrastructure, see
``oracle/__init__``).

* ket / Hamiltonian:  AccumulatorObsScalar.jl:52-137 -- for each connection:
  ``mel == 0`` is skipped (:92), no-change entries add ``mel`` (:97-98),
  others add ``mel * exp(logψ(σ') - logψ(σ))`` (:123-132); the cost
  gradient is BatchedValSampler.jl:97-115: F = E_loc · O_c† / Ns.
* doubled / Liouvillian: AccumulatorObsGrad.jl:39-127 -- every non-zero
  connection (including no-change ones, the ``&& false`` of :72) contributes
  ``mel ρ'/ρ`` to L_loc and ``mel ρ'/ρ O(σ')`` to ∇L_loc (no -O(σ) term,
  :113); BatchedGradSampler.jl:77-123 then forms C = mean|L_loc|^2 and
  F = conj(Σ L_s conj(∇L_s)/Ns - C conj(<O>)).
* density-matrix observables: BatchedObsDMSampler.jl:90-105 evaluates
  AccumulatorObsScalar over a doubled buffer filled with (σ, σ)
  (States.jl:131-132); a connection's changes go to the row
  (ApplyStateChanges.jl:18-21), so O_loc(σ) = Σ mel ρ(σ', σ)/ρ(σ, σ), with
  the same zero-skip and no-change rules as the ket estimator.
"""
import numpy as np

from .operators import connections_ket, connections_doubled, apply_changes


def local_energy(net, H, samples):
    """E_loc for ket samples (Ns, N); returns complex (Ns,)."""
    samples = np.atleast_2d(samples)
    ns = samples.shape[0]
    lpsi = net.logpsi(samples)
    res = np.zeros(ns, dtype=np.complex128)
    prime, owner, mels = [], [], []
    for s in range(ns):
        for mel, ch in connections_ket(H, samples[s]):
            if mel == 0:
                continue
            if len(ch) == 0:
                res[s] += mel
            else:
                prime.append(apply_changes(samples[s], ch))
                owner.append(s)
                mels.append(mel)
    if prime:
        prime = np.array(prime)
        owner = np.array(owner)
        lp = net.logpsi(prime)
        np.add.at(res, owner, np.array(mels) * np.exp(lp - lpsi[owner]))
    return res


def local_observable_dm(net, O, samples):
    """O_loc for physical samples (Ns, N) of the diagonal chain of an NDM;
    returns complex (Ns,)."""
    samples = np.atleast_2d(samples)
    ns = samples.shape[0]
    lrho = net.logpsi(samples, samples)
    res = np.zeros(ns, dtype=np.complex128)
    prime, owner, mels = [], [], []
    for s in range(ns):
        for mel, ch in connections_ket(O, samples[s]):
            if mel == 0:
                continue
            if len(ch) == 0:
                res[s] += mel
            else:
                prime.append(apply_changes(samples[s], ch))
                owner.append(s)
                mels.append(mel)
    if prime:
        prime = np.array(prime)
        owner = np.array(owner)
        lp = net.logpsi(prime, samples[owner])
        np.add.at(res, owner, np.array(mels) * np.exp(lp - lrho[owner]))
    return res


def local_liouvillian(net, lv, sr, sc, with_grad=True):
    """(L_loc (Ns,), ∇L_loc (Ns, P)) for doubled samples."""
    sr = np.atleast_2d(sr); sc = np.atleast_2d(sc)
    ns = sr.shape[0]
    lpsi = net.logpsi(sr, sc)
    pr, pc, owner, mels = [], [], [], []
    for s in range(ns):
        for mel, chl, chr_ in connections_doubled(lv, sr[s], sc[s]):
            if mel == 0:
                continue
            pr.append(apply_changes(sr[s], chl))
            pc.append(apply_changes(sc[s], chr_))
            owner.append(s)
            mels.append(mel)
    pr = np.array(pr); pc = np.array(pc); owner = np.array(owner)
    mels = np.array(mels)
    L = np.zeros(ns, dtype=np.complex128)
    if with_grad:
        lp, g = net.logpsi_and_grad(pr, pc)
    else:
        lp = net.logpsi(pr, pc)
    w = mels * np.exp(lp - lpsi[owner])
    np.add.at(L, owner, w)
    if not with_grad:
        return L, None
    dL = np.zeros((ns, g.shape[1]), dtype=np.complex128)
    np.add.at(dL, owner, w[:, None] * g)
    return L, dL


def center(O):
    """``_center_gradient!`` (BaseIterativeSampler.jl:19-26); O is (Ns, P)."""
    mean = O.mean(axis=0)
    return O - mean[None, :], mean


def force_ket(E, O):
    """F = E · O_c† / Ns (BatchedValSampler.jl:97-115); O is (Ns, P)."""
    Oc, _ = center(O)
    return (E[None, :] @ np.conj(Oc)).ravel() / O.shape[0]


def force_liouvillian(L, dL, O):
    """BatchedGradSampler.jl:99-120; returns (C, F)."""
    ns = O.shape[0]
    _, mean = center(O)
    C = np.mean(np.abs(L) ** 2)
    F = (L[None, :] @ np.conj(dL)).ravel() / ns
    F = F - C * np.conj(mean)
    return C, np.conj(F)
