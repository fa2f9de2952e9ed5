"""Batched Metropolis-Hastings over the pixel likelihood (cg_mh_run): the recorded
-2lnL matches a fresh evaluation at the recorded point on both paths, proposals stay
inside a uniform prior, and the FP64 and mixed paths give the same chain from the
same seed."""
import numpy as np
import pytest

from conftest import load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu


def _setup(precision, nchains):
    g = load_golden("nside4")
    ctx = cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=4, good_pixels=g["nest_good"],
                     noise_sigma=float(g["sigma"]), max_batch=nchains, precision=precision,
                     cl_ref=g["cls"][0] if precision == "mixed" else None, recenter="auto")
    rng = np.random.default_rng(3)
    x0 = np.log(g["cls"][0][2:])[None, :] + np.log1p(rng.uniform(-0.1, 0.1, (nchains, len(g["cls"][0]) - 2)))
    return g, ctx, x0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mh_records_consistent_states(precision):
    g, ctx, x0 = _setup(precision, 16)
    npar = x0.shape[1]
    lo = np.log(g["cls"][0][2:]) - 1.0
    hi = np.log(g["cls"][0][2:]) + 1.0
    priors = [("uniform", a, b) for a, b in zip(lo, hi)]
    with ctx:
        chain, acc, _ = ctx.mh(g["d"], x0, g["cls"][0], niter=30, sampling_width=0.05, priors=priors,
                               blocks=[npar // 2, npar], seed=4)
        assert chain.shape == (31, 16, npar + 1)
        assert acc.shape == (16, 2)
        assert np.all(np.isfinite(chain))
        assert acc.mean() > 0.05, acc.mean()
        assert np.all(chain[..., 1:] >= lo) and np.all(chain[..., 1:] <= hi)
        cl = np.tile(g["cls"][0], (16, 1))
        cl[:, 2:] = np.exp(chain[-1, :, 1:])
        r = ctx.loglike(cl, g["d"])
        tol = 1e-6 if precision == "fp64" else 1e-3
        assert np.abs(r["m2lnl"] - chain[-1, :, 0]).max() <= tol


def test_mh_fp64_and_mixed_agree():
    g, c64, x0 = _setup("fp64", 4)
    _, cmx, _ = _setup("mixed", 4)
    with c64, cmx:
        a, acc_a, _ = c64.mh(g["d"], x0, g["cls"][0], niter=10, sampling_width=0.03, blocks=[x0.shape[1]], seed=8)
        b, acc_b, _ = cmx.mh(g["d"], x0, g["cls"][0], niter=10, sampling_width=0.03, blocks=[x0.shape[1]], seed=8)
    assert np.array_equal(acc_a, acc_b)
    assert np.abs(a[..., 1:] - b[..., 1:]).max() < 1e-12
    assert np.abs(a[..., 0] - b[..., 0]).max() < 1e-3
