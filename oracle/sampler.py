"""Metropolis local-flip sampler replay (test infrastructure, see
``oracle/__init__``).

Restates src/Samplers/Metropolis.jl:101-167 with src/Samplers/MCMCRules/
LocalRule.jl:19-28 (ExchangeRule.jl:38-68 and OperatorRule.jl:42-58 as
options) and the chain bookkeeping of
src/IterativeInterface/Samplers/BaseIterativeSampler.jl:5-17, with the
reference MersenneTwister stream replaced by the Philox schema of
``oracle.philox``:

* every ``sample!`` call re-initialises all chains uniformly at random
  (``init_sampler!`` :101-115), then runs ``burn`` sweeps;
* a sweep (``samplenext!``) is ``passes`` Metropolis steps; ``passes`` is made
  odd by the constructor (:30-38);
* a step flips one uniformly chosen site per chain (sites 0..2N-1 on doubled
  states: >= N flips the column, DoubledHilbert.jl:19-27) and accepts iff
  ``u < exp(lp' - lp)`` (:148-159) with lp = 2 Re log psi;
* recorded slot k (1-based) holds the state after burn + k sweeps.  With
  ``stale_last_slot`` the reference's bookkeeping is reproduced exactly: the
  loop breaks before writing slot L, which keeps its previous contents
  (BaseIterativeSampler.jl:11-16 with ``done`` Metropolis.jl:122).
"""
import numpy as np

from . import philox
from .operators import connections_ket, apply_changes


def fix_passes(passes):
    return passes + 1 if passes % 2 == 0 else passes


def init_configs(hilb, seed, call, chains, n_sites_total):
    w = philox.init_words(seed, call, chains, n_sites_total)
    top = (w >> np.uint32(31)).astype(np.int64)          # floor(u*2), u = w/2^32
    return hilb.value(top)


def run(log_prob, hilb, n_chains, chain_length, burn, passes, seed, call=0,
        doubled=False, stale_last_slot=False, prev_samples=None,
        gpu_accept_bits=None, tie_tol=1e-6, chain_offset=0, couplings=None, move_op=None):
    """Replays one ``_sample_state!`` call.

    ``couplings`` (list of 0-based site pairs) selects ExchangeRule
    (src/Samplers/MCMCRules/ExchangeRule.jl:38-68): the step's draw picks
    coupling ``(r0 * len(couplings)) >> 32`` and swaps its two values (a swap
    of equal values proposes the same state, which ``u < exp(0)`` accepts).

    ``move_op`` (an ``OpSum``) selects OperatorRule
    (src/Samplers/MCMCRules/OperatorRule.jl:42-58): the step's draw picks
    connection ``(r0 * n_f) >> 32`` of the n_f connections of the chain's
    rows (``connections_ket`` order), applies its changes, and adds
    ``log(n_f / n_b)`` with n_b counted at the new configuration.

    ``log_prob(batch)`` maps (B, nsites_total) configurations to 2 Re log psi.
    ``gpu_accept_bits`` (optional, (steps, B) bool) resolves near-tie
    decisions (|log u - Δ| < tie_tol, default 1e-6: the FP32 rounding of the
    device's Δ) the way the GPU took them and counts them; all other decisions
    must agree.  Returns (samples (L, B, nsites_total), info)."""
    N = hilb.n_sites
    nt = 2 * N if doubled else N
    chains = np.arange(n_chains) + chain_offset
    sigma = init_configs(hilb, seed, call, chains, nt)
    lp = log_prob(sigma)
    passes = fix_passes(passes)
    L = chain_length
    samples = np.empty((L, n_chains, nt))
    if prev_samples is not None:
        samples[:] = prev_samples
    else:
        samples[:] = hilb.fill_value()
    n_record = L - 1 if (stale_last_slot and L > 1) else L
    n_sweeps = burn + n_record
    if stale_last_slot and L == 1:
        n_sweeps = burn
    # max_tie_gap: the largest |log u - Δ| of a decision the device took the
    # other way (0 when every decision agrees)
    info = {"ambiguous": 0, "mismatch": 0, "accepted": 0, "steps": 0, "max_tie_gap": 0.0}
    t = 0
    for sweep in range(n_sweeps):
        for _ in range(passes):
            rows = np.arange(n_chains)
            new = sigma.copy()
            bias = 0.0
            if move_op is not None:
                r0, u = philox.mh_raw(seed, call, chains, t)
                bias = np.zeros(n_chains)
                for b in range(n_chains):
                    conns = connections_ket(move_op, sigma[b])
                    nf = len(conns)
                    ch = conns[(int(r0[b]) * nf) >> 32][1]
                    if len(ch):
                        new[b] = apply_changes(sigma[b], ch)
                        bias[b] = np.log(nf / len(connections_ket(move_op, new[b])))
            elif couplings is None:
                site, u = philox.mh_draws(seed, call, chains, t, nt)
                new[rows, site] = hilb.flip(sigma[rows, site])
            else:
                cidx, u = philox.mh_draws(seed, call, chains, t, len(couplings))
                pr = np.asarray(couplings, dtype=np.int64)[cidx]
                new[rows, pr[:, 0]] = sigma[rows, pr[:, 1]]
                new[rows, pr[:, 1]] = sigma[rows, pr[:, 0]]
            lpn = log_prob(new)
            delta = lpn - lp + bias
            with np.errstate(over="ignore", divide="ignore"):
                acc = u < np.exp(delta)
                logu = np.log(np.maximum(u, 1e-300))
            if gpu_accept_bits is not None:
                g = np.asarray(gpu_accept_bits[t], dtype=bool)
                gap = np.abs(logu - delta)
                amb = gap < tie_tol
                dis = g != acc
                info["ambiguous"] += int(np.sum(amb & dis))
                info["mismatch"] += int(np.sum(~amb & dis))
                if dis.any():
                    info["max_tie_gap"] = max(info["max_tie_gap"], float(gap[dis].max()))
                acc = np.where(amb, g, acc)
            sigma = np.where(acc[:, None], new, sigma)
            lp = np.where(acc, lpn, lp)
            info["accepted"] += int(acc.sum())
            info["steps"] += n_chains
            t += 1
        k = sweep - burn
        if k >= 0:
            samples[k] = sigma
    if stale_last_slot and L == 1:
        samples[0] = sigma          # init_sampler! writes the first slot
    return samples, info


def exact_run(p, n_chains, chain_length, seed, call=0, stale_last_slot=False, prev_samples=None,
              gpu_samples=None, tie_tol=1e-6):
    """Replays the exact sampler (src/Samplers/Exact.jl:52-82; batched
    variant :133-176): cdf = cumsum(p) / sum(p) over configuration indices,
    draw = searchsortedfirst(cdf, u) with the Philox 53-bit uniform of
    ``philox.exact_uniforms``.  Slot k of chain c holds draw k; with
    ``stale_last_slot`` slots 0..L-2 are drawn and slot L-1 keeps
    ``prev_samples`` (L = 1: one draw into slot 0), as for the Metropolis
    bookkeeping of BaseIterativeSampler.jl:11-16.

    Returns (indices [L, B], number of near-ties).  With ``gpu_samples`` a
    draw whose u lies within ``tie_tol`` of a CDF boundary takes the GPU's
    index when it is one of the two neighbours (the GPU's CDF carries FP32
    log-probabilities), and is counted."""
    cdf = np.cumsum(np.asarray(p, dtype=np.float64))
    cdf /= cdf[-1]
    L = chain_length
    n_rec = (L - 1 if L > 1 else 0) if stale_last_slot else L
    draws = n_rec + (1 if stale_last_slot and L == 1 else 0)
    out = np.zeros((L, n_chains), dtype=np.int64) if prev_samples is None else np.array(prev_samples)
    chains = np.arange(n_chains)
    ties = 0
    for t in range(draws):
        u = philox.exact_uniforms(seed, call, chains, t)
        idx = np.searchsorted(cdf, u, side="left")
        idx = np.minimum(idx, len(cdf) - 1)
        slot = t if t < n_rec else 0
        if gpu_samples is not None:
            g = np.asarray(gpu_samples)[slot]
            lo = np.where(idx > 0, cdf[np.maximum(idx - 1, 0)], 0.0)
            near = (np.abs(u - cdf[idx]) < tie_tol) | (np.abs(u - lo) < tie_tol)
            ok = near & (np.abs(g - idx) == 1)
            ties += int(ok.sum())
            idx = np.where(ok, g, idx)
        out[slot] = idx
    return out, ties
