"""Sampler descriptions of the reference API (src/Samplers/)."""


class LocalRule:
    """Single-site flip proposals (src/Samplers/MCMCRules/LocalRule.jl:12-28)."""


class ExchangeRule:
    """``ExchangeRule(H)`` (src/Samplers/MCMCRules/ExchangeRule.jl:16-35):
    the couplings (i, j) are the sites of the 2-site terms of the operator,
    in its term order; 1-site terms are skipped and terms on more than two
    sites are ignored with a warning, as in the reference.  A move draws one
    coupling uniformly and swaps the two values (:38-68)."""

    def __init__(self, op):
        import warnings
        ops = op.ops if hasattr(op, "ops") else [op]
        pairs = []
        for o in ops:
            sites = list(o.sites)
            if len(sites) == 1:
                continue
            if len(sites) > 2:
                warnings.warn("Can't exchange between 3-site couplings. This coupling is ignored")
                continue
            pairs.append((int(sites[0]), int(sites[1])))
        if not pairs:
            raise ValueError("the operator has no 2-site terms")
        self.couplings = pairs           # 0-based sites

    def __repr__(self):
        return f"ExchangeRule({len(self.couplings)} couplings)"


class OperatorRule:
    """``OperatorRule(Ô)`` (src/Samplers/MCMCRules/OperatorRule.jl:9-58): a
    move draws one connection of the configuration's rows in Ô's tables
    uniformly (the diagonal entries included, which propose the same state)
    and applies its changes; the acceptance carries the factor n(σ)/n(σ') of
    the numbers of connections."""

    def __init__(self, op):
        self.operator = op

    def __repr__(self):
        return "OperatorRule()"


class MetropolisSampler:
    """``MetropolisSampler(rule, chain_length, passes; burn=0, seed)``
    (src/Samplers/Metropolis.jl:26-40).  An even number of passes is raised
    by one, as the reference constructor does."""

    def __init__(self, rule, chain_length, passes, burn=0, seed=None):
        if passes < 1 or chain_length < 1:
            raise ValueError("passes and chain_length must be positive")
        if passes % 2 == 0:
            passes += 1
        self.rule = rule
        self.kind = 0     # NQ_SAMPLER_METROPOLIS
        self.chain_length = int(chain_length)
        self.passes = int(passes)
        self.burn_length = int(burn)
        self.seed = 0x4E51 if seed is None else int(seed)

    def __repr__(self):
        return (f"MetropolisSampler(chain_length={self.chain_length}, burn={self.burn_length}, "
                f"passes={self.passes}, seed={self.seed})")


class ExactSampler:
    """``ExactSampler(n_samples; seed)`` (src/Samplers/Exact.jl:16-27): every
    sample call enumerates the 2^N configurations, builds the cumulative
    distribution of |ψ|² and draws each of the ``batch_sz`` x ``n_samples``
    slots independently by inverse CDF.  ``chain_length`` = n_samples draws
    per batch entry, as the batched reference sampler takes one draw per
    entry per step; burn and passes do not apply."""

    kind = 1          # NQ_SAMPLER_EXACT

    def __init__(self, n_samples, seed=None):
        if n_samples < 1:
            raise ValueError("n_samples must be positive")
        self.chain_length = int(n_samples)
        self.passes = 1
        self.burn_length = 0
        self.seed = 0x4E51 if seed is None else int(seed)

    def __repr__(self):
        return f"ExactSampler(n_samples={self.chain_length}, seed={self.seed})"
