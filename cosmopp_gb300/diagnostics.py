"""Chain diagnostics for the batched HMC output (host-side analysis)."""
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
