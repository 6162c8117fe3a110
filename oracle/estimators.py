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


# ---------------------------------------------------------------------------
# Sample-batched forms of the same estimators.  They visit the same
# connections with the same rules (zero elements skipped; no-change entries
# add mel for kets, mel ρ/ρ for the Liouvillian), but group the samples by the
# local row of every operator, so a whole sample set (10^5 samples) is one
# vectorised pass instead of a Python loop per sample.  Summation order
# differs from the per-sample forms by FP64 rounding only.
# ---------------------------------------------------------------------------

def _rows_groups(hilb, sigma, sites):
    r = np.asarray(hilb.local_index(sigma, sites), dtype=np.int64)
    for row in np.unique(r):
        yield int(row), np.nonzero(r == row)[0]


def _apply_batch(sigma, idx, changes):
    out = sigma[idx].copy()
    for site, val in changes:
        out[:, site] = val
    return out


def local_energy_batched(net, H, samples, chunk=1 << 18):
    """``local_energy`` over a (Ns, N) sample set, vectorised over samples."""
    samples = np.atleast_2d(np.asarray(samples, dtype=np.float64))
    ns = samples.shape[0]
    lpsi = net.logpsi(samples)
    res = np.zeros(ns, dtype=np.complex128)
    primes, owners, mels = [], [], []
    for o in H.ops:
        for row, idx in _rows_groups(H.hilb, samples, o.sites):
            for mel, ch in o.conns[row]:
                if mel == 0:
                    continue
                if len(ch) == 0:
                    res[idx] += mel
                else:
                    primes.append(_apply_batch(samples, idx, ch))
                    owners.append(idx)
                    mels.append(np.full(idx.size, mel, dtype=np.complex128))
    if primes:
        pr = np.concatenate(primes)
        ow = np.concatenate(owners)
        ml = np.concatenate(mels)
        for a in range(0, pr.shape[0], chunk):
            b = min(pr.shape[0], a + chunk)
            lp = net.logpsi(pr[a:b])
            np.add.at(res, ow[a:b], ml[a:b] * np.exp(lp - lpsi[ow[a:b]]))
    return res


def _doubled_connections_batched(lv, sr, sc):
    """(owner, mel, primed row, primed column) arrays over all samples, every
    non-zero connection of ``connections_doubled``."""
    h = lv.hilb
    ows, mls, prs, pcs = [], [], [], []

    def push(idx, mel, chl, chr_):
        ows.append(idx)
        mls.append(np.full(idx.size, mel, dtype=np.complex128))
        prs.append(_apply_batch(sr, idx, chl))
        pcs.append(_apply_batch(sc, idx, chr_))

    for opl, _ in lv.HnH_l:
        for row, idx in _rows_groups(h, sr, opl.sites):
            for mel, ch in opl.conns[row]:
                if mel != 0:
                    push(idx, mel, ch, [])
    for _, opr in lv.HnH_r:
        for row, idx in _rows_groups(h, sc, opr.sites):
            for mel, ch in opr.conns[row]:
                if mel != 0:
                    push(idx, mel, [], ch)
    for opl, opr in lv.LLdag:
        rr = np.asarray(h.local_index(sr, opl.sites), dtype=np.int64)
        rc = np.asarray(h.local_index(sc, opr.sites), dtype=np.int64)
        for a in np.unique(rr):
            for b in np.unique(rc):
                idx = np.nonzero((rr == a) & (rc == b))[0]
                if idx.size == 0:
                    continue
                for ml, chl in opl.conns[int(a)]:
                    for mr, chr_ in opr.conns[int(b)]:
                        if ml * mr != 0:
                            push(idx, ml * mr, chl, chr_)
    return (np.concatenate(ows), np.concatenate(mls), np.concatenate(prs), np.concatenate(pcs))


def liouvillian_force_batched(net, lv, sr, sc, chunk=1 << 14):
    """L_loc (Ns,), the cost C = mean|L_loc|², the force F of
    ``force_liouvillian`` and <O> over a doubled sample set, vectorised over
    samples.  ∇L_loc is never stored: F accumulates Σ_s L_s conj(∇L_s) =
    Σ_{s,c} L_s conj(w_sc) conj(O(σ'_sc)) chunk by chunk, and O(σ) is only
    averaged."""
    sr = np.atleast_2d(np.asarray(sr, dtype=np.float64))
    sc = np.atleast_2d(np.asarray(sc, dtype=np.float64))
    ns = sr.shape[0]
    lpsi = net.logpsi(sr, sc)
    ow, ml, pr, pc = _doubled_connections_batched(lv, sr, sc)
    w = np.empty(ow.size, dtype=np.complex128)
    for a in range(0, ow.size, 1 << 18):
        b = min(ow.size, a + (1 << 18))
        w[a:b] = ml[a:b] * np.exp(net.logpsi(pr[a:b], pc[a:b]) - lpsi[ow[a:b]])
    L = np.zeros(ns, dtype=np.complex128)
    np.add.at(L, ow, w)
    C = np.mean(np.abs(L) ** 2)
    acc = None
    for a in range(0, ow.size, chunk):
        b = min(ow.size, a + chunk)
        _, g = net.logpsi_and_grad(pr[a:b], pc[a:b])
        coef = L[ow[a:b]] * np.conj(w[a:b])
        part = coef @ np.conj(g)
        acc = part if acc is None else acc + part
    meanO = None
    for a in range(0, ns, chunk):
        b = min(ns, a + chunk)
        _, g = net.logpsi_and_grad(sr[a:b], sc[a:b])
        s = g.sum(axis=0)
        meanO = s if meanO is None else meanO + s
    meanO = meanO / ns
    F = acc / ns - C * np.conj(meanO)
    return L, C, np.conj(F), meanO


def sr_matrix_batched(grad_fn, n, real_params, chunk=1 << 14):
    """S of ``sr.build_S`` from the centred O of n samples without holding
    O: grad_fn(a, b) returns O of samples a..b-1 as (b - a, P); two passes
    (mean, then the centred Gram)."""
    meanO = None
    for a in range(0, n, chunk):
        g = grad_fn(a, min(n, a + chunk))
        s = g.sum(axis=0)
        meanO = s if meanO is None else meanO + s
    meanO = meanO / n
    G = None
    for a in range(0, n, chunk):
        g = grad_fn(a, min(n, a + chunk)) - meanO[None, :]
        part = g.T @ np.conj(g)
        G = part if G is None else G + part
    if real_params:
        return np.real(G) / n, meanO
    return np.conj(G) / n, meanO


def force_ket_batched(E, grad_fn, n, chunk=1 << 14):
    """F = E · O_c† / Ns of ``force_ket`` without holding O."""
    meanO = None
    for a in range(0, n, chunk):
        g = grad_fn(a, min(n, a + chunk))
        s = g.sum(axis=0)
        meanO = s if meanO is None else meanO + s
    meanO = meanO / n
    F = None
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        g = grad_fn(a, b) - meanO[None, :]
        part = E[a:b] @ np.conj(g)
        F = part if F is None else F + part
    return F / n
