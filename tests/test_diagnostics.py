"""Host-side chain diagnostics used beside the batched HMC: the effective sample
size of iid draws is close to n, and of an AR(1) chain close to n (1 - phi) / (1 + phi)."""
import numpy as np

from cosmopp_gb300 import diagnostics


def test_ess_iid_close_to_n():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(20000)
    assert 0.85 * len(x) < diagnostics.ess_1d(x) < 1.15 * len(x)


def test_ess_ar1_matches_theory():
    rng = np.random.default_rng(1)
    phi, n = 0.8, 50000
    e = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = e[0]
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    expect = n * (1 - phi) / (1 + phi)
    assert 0.75 * expect < diagnostics.ess_1d(x) < 1.25 * expect


def test_ess_sums_over_chains_and_handles_constants():
    rng = np.random.default_rng(2)
    chain = rng.standard_normal((400, 3, 2))
    chain[:, :, 1] = 5.0  # a parameter that never moves: every draw counts, none is informative
    e = diagnostics.ess(chain)
    assert e.shape == (2,)
    assert 0.7 * 1200 < e[0] < 1.3 * 1200
    assert e[1] == 1200
