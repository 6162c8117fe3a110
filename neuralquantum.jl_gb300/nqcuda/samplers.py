"""Sampler descriptions of the reference API (src/Samplers/)."""


class LocalRule:
    """Single-site flip proposals (src/Samplers/MCMCRules/LocalRule.jl:12-28)."""


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
        self.chain_length = int(chain_length)
        self.passes = int(passes)
        self.burn_length = int(burn)
        self.seed = 0x4E51 if seed is None else int(seed)

    def __repr__(self):
        return (f"MetropolisSampler(chain_length={self.chain_length}, burn={self.burn_length}, "
                f"passes={self.passes}, seed={self.seed})")
