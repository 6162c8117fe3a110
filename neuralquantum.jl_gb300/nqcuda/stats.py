"""``Measurement`` (src/utils/stats.jl:1-24)."""


class Measurement:
    def __init__(self, mean, error, variance, tau, R):
        self.mean, self.error, self.variance, self.tau, self.R = mean, error, variance, tau, R

    def __repr__(self):
        m = self.mean
        if isinstance(m, complex):
            sgn = "+" if m.imag >= 0 else "-"
            ms = f"{m.real:6.4f} {sgn} {abs(m.imag):6.4f} im"
        else:
            ms = f"{m:6.4f}"
        return (f"({ms}) ± {self.error:6.4f} [var={self.variance:6.4f}, tau={self.tau:6.4f}, "
                f"R={self.R:6.4f}]")
