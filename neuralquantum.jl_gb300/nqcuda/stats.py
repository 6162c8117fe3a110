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


def integrated_autocorr_time(x, window=5.0):
    """Integrated autocorrelation time of a (chains, samples) series, in
    samples, in the convention tau = 1 + 2 Σ_{t>=1} ρ(t) (tau = 1 for
    independent samples, so the effective sample size is n / tau).  ρ is the
    chain-averaged autocovariance (computed by FFT) normalised at lag 0; the
    sum stops at the first lag M with M >= window * tau (Sokal's
    self-consistent window).  The reference reports only the ``tau`` of
    ``Measurement``; this one backs the effective-sample-size figures."""
    import numpy as np
    v = np.asarray(x, dtype=np.complex128)
    v = v - v.mean(axis=1, keepdims=True)
    n = v.shape[1]
    spec = np.fft.fft(v, n=2 * n, axis=1)
    acov = np.fft.ifft(np.abs(spec) ** 2, axis=1)[:, :n].real.mean(axis=0)
    if not acov[0] > 0:
        return 1.0
    rho = acov / acov[0]
    tau = 1.0
    for lag in range(1, n):
        tau += 2.0 * rho[lag]
        if lag >= window * tau:
            break
    return max(tau, 1.0)


def autocorrelation(x, max_lag):
    """Chain-averaged normalised autocorrelation ρ(0..max_lag) of a
    (chains, samples) series (ρ(0) = 1)."""
    import numpy as np
    v = np.asarray(x, dtype=np.complex128)
    v = v - v.mean(axis=1, keepdims=True)
    n = v.shape[1]
    spec = np.fft.fft(v, n=2 * n, axis=1)
    acov = np.fft.ifft(np.abs(spec) ** 2, axis=1)[:, :n].real.mean(axis=0)
    if not acov[0] > 0:
        out = np.zeros(max_lag + 1)
        out[0] = 1.0
        return out
    return acov[:max_lag + 1] / acov[0]


def effective_sample_size(x, window=5.0):
    """Number of samples divided by the integrated autocorrelation time."""
    import numpy as np
    v = np.asarray(x)
    return v.size / integrated_autocorr_time(v, window)
