"""Chain diagnostics for the batched HMC and Metropolis-Hastings output (host-side analysis)."""
import numpy as np


def ess_1d(x):
    """Effective sample size of one chain: n / (1 + 2 sum rho_t), the sum truncated by
    Geyer's initial positive sequence (pairs rho_{2k} + rho_{2k+1} > 0)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    if n < 4 or np.var(x) == 0:
        return float(n)
    y = x - x.mean()
    f = np.fft.rfft(y, 2 * n)
    ac = np.fft.irfft(f * np.conj(f))[:n]
    ac = ac / ac[0]
    tau = 1.0
    for k in range(1, n // 2):
        pair = ac[2 * k - 1] + ac[2 * k]
        if pair <= 0:
            break
        tau += 2 * pair
    return float(n / tau)


def ess(chain):
    """chain [n, nchains, npar] -> ESS summed over chains, per parameter [npar]."""
    n, nc, npar = chain.shape
    return np.array([sum(ess_1d(chain[:, c, k]) for c in range(nc)) for k in range(npar)])


def gelman_rubin(chain):
    """Potential scale reduction R per parameter over chains [n, nchains, npar], the
    statistic MetropolisHastings uses as its GELMAN_RUBIN stopping rule
    (include/mcmc.hpp:486-520): B = n var(chain means) (ddof 1), W = the mean of the
    per-chain variances (ddof 1), R = sqrt(((n-1) W / n + B / n) / W); R = 1 when every
    chain is constant at one value, 100 when W = 0 but the chains differ."""
    x = np.asarray(chain, dtype=np.float64)
    n, nc, _ = x.shape
    if n < 2 or nc < 2:
        raise ValueError("needs at least 2 chains of 2 states")
    means = x.mean(axis=0)
    b = n * means.var(axis=0, ddof=1)
    w = x.var(axis=0, ddof=1).mean(axis=0)
    var = (n - 1) * w / n + b / n
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.sqrt(var / w)
    return np.where(w == 0, np.where(var == 0, 1.0, 100.0), r)
