"""``Measurement`` statistics (test infrastructure, see ``oracle/__init__``).

Restates ``_single_stat_analysis`` of src/utils/stats.jl:26-50 on a
(chains x samples) matrix; Julia's ``var`` is the unbiased estimator and, for
complex data, averages |x - mean|^2.
"""
import numpy as np


def _var(x, mean, axis=None):
    d = np.abs(x - mean) ** 2
    n = d.size if axis is None else d.shape[axis]
    return d.sum(axis=axis) / (n - 1)


def stat_analysis(vals):
    vals = np.asarray(vals)
    n, L = vals.shape
    mu_chains = vals.mean(axis=1)
    mu = mu_chains.mean()
    var_chains = _var(vals, mu_chains[:, None], axis=1) if L > 1 else np.full(n, np.nan)
    var_mu_ch = _var(mu_chains, mu)
    var_mu = _var(vals.ravel(), mu)
    err = np.sqrt(var_mu_ch / n)
    variance = np.mean(var_chains)
    t = var_mu_ch / var_mu
    tau = max(0.0, 0.5 * (t * L - 1))
    R = np.sqrt((L - 1) / L + t)
    return {"mean": mu, "error": err, "variance": variance, "tau": tau, "R": R}


def integrated_autocorr_time(x, c=5.0):
    """Sokal-windowed integrated autocorrelation time, averaged over chains;
    x is (chains, samples).  Used for effective-sample-size reporting (a
    quantity the reference does not compute)."""
    x = np.asarray(x, dtype=np.complex128)
    x = x - x.mean(axis=1, keepdims=True)
    n = x.shape[1]
    f = np.fft.fft(x, n=2 * n, axis=1)
    acf = np.fft.ifft(f * np.conj(f), axis=1)[:, :n].real
    acf = acf.mean(axis=0)
    if acf[0] <= 0:
        return 0.5
    rho = acf / acf[0]
    tau = 0.5
    for m in range(1, n):
        tau += rho[m]
        if m >= c * tau:
            break
    return max(tau, 0.5)
