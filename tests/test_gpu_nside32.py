"""The large configuration: nside 32 (90% mask, ~11k pixels), lmax 95, FWHM
110', sigma 0.5.  The mixed path (FP64 reference factorisation of an 11k x 11k
covariance, whitened table over 6e7 pixel pairs and 9212 harmonics) against
the plain FP64 path on four elements (two lognormal C_l vectors and two far
points at the re-centring radius), per gradient component against the bar of
conftest.assert_grad_close; and the memory admission that sizes the batch."""
import numpy as np
import pytest

import cosmopp_gb300 as cg
from cosmopp_gb300 import workload as W
from conftest import assert_grad_close, grad_scale

pytestmark = pytest.mark.gpu


def test_nside32_mixed_matches_fp64():
    wl = W.make("nside32_lmax95_b32", batch=2)
    assert 10800 < wl.n < 11300
    L1 = wl.lmax + 1
    ell = np.arange(L1)
    far = wl.cl_fid[None, :] * np.exp(np.vstack([np.full(L1, 0.999), np.where(ell % 2 == 0, 0.999, -0.999)]))
    far[:, :2] = 0
    cls = np.vstack([wl.cl_batch, far])
    kw = dict(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
              noise_sigma=wl.sigma, max_batch=len(cls))
    with cg.Context(precision="fp64", **kw) as c64:
        c = c64.build_cmatrix(wl.cl_fid)
        n = wl.n
        full = W.packed_to_full(c, n) + wl.sigma ** 2 * np.eye(n)
        d = W.draw_data(full, wl.z)
        del full, c
        r64 = c64.loglike(cls, d, grad=True)
        s = grad_scale(c64, cls, n, wl.lmax)
    with cg.Context(precision="mixed", cl_ref=wl.cl_fid, recenter="fixed", **kw) as cmx:
        rmx = cmx.loglike(cls, d, grad=True)
    assert np.all(r64["status"] == 0) and np.all(rmx["status"] == 0)
    dm = np.abs(rmx["m2lnl"] - r64["m2lnl"])
    print("nside32 |d(-2lnL)|", dm, "d logdet", rmx["logdet"] - r64["logdet"], "d chi2", rmx["chi2"] - r64["chi2"])
    assert dm.max() <= 1e-3, (rmx["m2lnl"], r64["m2lnl"])
    assert_grad_close(rmx["grad"], r64["grad"], s, 1e-4, "nside32")


def test_memory_admission_plans_the_nside32_batch():
    """The plan against a 180 GB budget: the batch of 32 fits; the byte counts match what a context
    then allocates on the device (within allocator rounding)."""
    import torch
    wl = W.make("nside32_lmax95_b32")
    kw = dict(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
              noise_sigma=wl.sigma)
    p180 = cg.plan_memory(budget_bytes=180 * 10 ** 9, precision="mixed", max_batch=32, **kw)
    assert p180["max_batch_fit"] >= 32 and p180["chunk"] == 32
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    with cg.Context(precision="mixed", cl_ref=wl.cl_fid, recenter="fixed", max_batch=4, **kw) as cmx:
        plan = cmx.memory_plan()
        cls = W.lognormal_batch(wl.cl_fid, 4, 3)
        cmx.loglike(cls, np.ones(wl.n), grad=True)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info(0)
    used = free0 - free1
    predicted = plan["bytes_fixed"] + 4 * plan["bytes_per_element"]
    print("admission: predicted %.3f GB, device %.3f GB" % (predicted / 1e9, used / 1e9))
    assert abs(used - predicted) <= 0.02 * predicted + (256 << 20)
