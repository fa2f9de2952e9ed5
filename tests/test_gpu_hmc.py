"""Batched HMC (cg_hmc_run) driven by the adjoint gradient: the recorded -2lnL
matches a fresh evaluation at the recorded point, small steps conserve the
Hamiltonian (acceptance near 1), and the FP64 and mixed paths give the same
trajectory from the same seed."""
import numpy as np
import pytest

from conftest import load_golden

import cosmopp_gb300 as cg
from cosmopp_gb300 import diagnostics

pytestmark = pytest.mark.gpu


def _setup(precision, nchains):
    g = load_golden("nside4")
    ctx = cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=4, good_pixels=g["nest_good"],
                     noise_sigma=float(g["sigma"]), max_batch=nchains, precision=precision,
                     cl_ref=g["cls"][0] if precision == "mixed" else None, recenter="auto")
    rng = np.random.default_rng(2)
    x0 = np.log(g["cls"][0][2:])[None, :] + np.log1p(rng.uniform(-0.1, 0.1, (nchains, len(g["cls"][0]) - 2)))
    return g, ctx, x0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hmc_records_consistent_states_and_accepts(precision):
    g, ctx, x0 = _setup(precision, 8)
    with ctx:
        chain, acc = ctx.hmc(g["d"], x0, g["cls"][0], niter=12, nleap=10, tau=0.02, seed=5)
        assert chain.shape == (13, 8, len(g["cls"][0]) - 1)
        assert np.all(np.isfinite(chain))
        assert acc.mean() > 0.6, acc
        cl = np.tile(g["cls"][0], (8, 1))
        cl[:, 2:] = np.exp(chain[-1, :, 1:])
        r = ctx.loglike(cl, g["d"])
        tol = 1e-6 if precision == "fp64" else 1e-3
        assert np.abs(r["m2lnl"] - chain[-1, :, 0]).max() <= tol
    ess = diagnostics.ess(chain[:, :, 1:])
    assert np.all(ess > 0)


def test_hmc_fp64_and_mixed_agree():
    g, c64, x0 = _setup("fp64", 4)
    _, cmx, _ = _setup("mixed", 4)
    with c64, cmx:
        a, acc_a = c64.hmc(g["d"], x0, g["cls"][0], niter=4, nleap=5, tau=0.02, seed=9)
        b, acc_b = cmx.hmc(g["d"], x0, g["cls"][0], niter=4, nleap=5, tau=0.02, seed=9)
    assert np.array_equal(acc_a, acc_b)
    assert np.abs(a[..., 1:] - b[..., 1:]).max() < 1e-5
    assert np.abs(a[..., 0] - b[..., 0]).max() < 1e-3


@pytest.mark.parametrize("precision,golden,nchains", [("fp64", "nside4", 8), ("mixed", "nside4", 8),
                                                      ("mixed", "nside8_lmax24", 16)])
def test_device_leapfrog_matches_the_host_loop_bit_for_bit(precision, golden, nchains):
    """cg_hmc_run's device-resident leapfrog (the default) and the host loop of cg_hmc_sample over
    the same pixel likelihood (knob hmc_device = 0) draw the same random numbers and do the same
    arithmetic, C_l = exp(x) included: identical chains, with and without step jitter."""
    g = load_golden(golden)
    ctx = cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=int(g["nside"]),
                     good_pixels=g["nest_good"], noise_sigma=float(g["sigma"]), max_batch=nchains,
                     precision=precision, cl_ref=g["cls"][0] if precision == "mixed" else None, recenter="fixed")
    rng = np.random.default_rng(4)
    x0 = np.log(g["cls"][0][2:])[None, :] + np.log1p(rng.uniform(-0.1, 0.1, (nchains, len(g["cls"][0]) - 2)))
    with ctx:
        assert ctx.tune_get("hmc_device") == 1
        for jitter in (False, True):
            dev, acc_dev = ctx.hmc(g["d"], x0, g["cls"][0], niter=5, nleap=6, tau=0.03, seed=11, jitter=jitter)
            ctx.tune_set("hmc_device", 0)
            host, acc_host = ctx.hmc(g["d"], x0, g["cls"][0], niter=5, nleap=6, tau=0.03, seed=11, jitter=jitter)
            ctx.tune_set("hmc_device", 1)
            assert np.array_equal(dev, host), np.abs(dev - host).max()
            assert np.array_equal(acc_dev, acc_host)
            assert acc_dev.mean() > 0.5
