"""The large configuration: nside 32 (90% mask, ~11k pixels), lmax 95, FWHM
110', sigma 0.5.  The mixed path (FP64 reference factorisation of an 11k x 11k
covariance, whitened table over 6e7 pixel pairs and 9212 harmonics) against
the plain FP64 path, on two lognormal C_l vectors."""
import numpy as np
import pytest

import cosmopp_gb300 as cg
from cosmopp_gb300 import workload as W

pytestmark = pytest.mark.gpu


def test_nside32_mixed_matches_fp64():
    wl = W.make("nside32_lmax95_b32", batch=2)
    assert 10800 < wl.n < 11300
    kw = dict(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
              noise_sigma=wl.sigma, max_batch=2)
    with cg.Context(precision="fp64", **kw) as c64:
        c = c64.build_cmatrix(wl.cl_fid)
        n = wl.n
        full = W.packed_to_full(c, n) + wl.sigma ** 2 * np.eye(n)
        d = W.draw_data(full, wl.z)
        del full, c
        r64 = c64.loglike(wl.cl_batch, d, grad=True)
    with cg.Context(precision="mixed", cl_ref=wl.cl_fid, recenter="fixed", **kw) as cmx:
        rmx = cmx.loglike(wl.cl_batch, d, grad=True)
    assert np.all(r64["status"] == 0) and np.all(rmx["status"] == 0)
    print("nside32 |d(-2lnL)|", np.abs(rmx["m2lnl"] - r64["m2lnl"]), "d logdet", rmx["logdet"] - r64["logdet"])
    assert np.abs(rmx["m2lnl"] - r64["m2lnl"]).max() <= 1e-3, (rmx["m2lnl"], r64["m2lnl"])
    gscale = np.abs(r64["grad"]).max(axis=1, keepdims=True)
    assert (np.abs(rmx["grad"] - r64["grad"]) / gscale).max() <= 1e-4
