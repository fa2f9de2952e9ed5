"""Parity of the batched mixed-precision path: every -2lnL within the
spec bar |delta| <= 1e-3 of the FP64 reference values (golden fixtures
from the reference's own code, and the FP64 CUDA path, itself pinned to the
reference), gradients within 1e-4 relative (of max |grad| over l) of the FP64
adjoint, on batches of lognormal C_l perturbations, one shared map or one map
per element."""
import numpy as np
import pytest

from conftest import load_golden

import cosmopp_gb300 as cg
from cosmopp_gb300 import workload as W

pytestmark = pytest.mark.gpu

TOL_M2LNL = 1e-3
TOL_GRAD = 1e-4


def _ctx(g, precision, max_batch, **kw):
    return cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=int(g["nside"]),
                      good_pixels=g["nest_good"], scheme="NEST", noise_sigma=float(g["sigma"]),
                      max_batch=max_batch, precision=precision, **kw)


@pytest.mark.parametrize("name", ["nside4", "nside8_lmax24", "nside16_lmax47"])
def test_mixed_matches_reference_golden(name):
    g = load_golden(name)
    B = len(g["cls"])
    with _ctx(g, "mixed", B) as ctx:
        r = ctx.loglike(g["cls"], g["d"], grad=False)
        assert ctx.reference_count() == 1
    assert np.all(r["status"] == 0)
    err = np.abs(r["m2lnl"] - g["m2lnl"]).max()
    assert err <= TOL_M2LNL, err
    assert np.abs(r["logdet"] - g["logdet_raw"]).max() <= TOL_M2LNL
    assert np.abs(r["chi2"] - g["chi2"]).max() <= TOL_M2LNL


@pytest.mark.parametrize("name,B", [("nside8_lmax24", 32), ("nside16_lmax47", 48)])
def test_mixed_batch_vs_fp64_path(name, B):
    g = load_golden(name)
    cls = W.lognormal_batch(g["cls"][0], B, 11)
    with _ctx(g, "fp64", B) as c64, _ctx(g, "mixed", B, cl_ref=g["cls"][0], recenter="fixed") as cmx:
        r64 = c64.loglike(cls, g["d"], grad=True)
        rmx = cmx.loglike(cls, g["d"], grad=True)
    assert np.all(rmx["status"] == 0) and np.all(r64["status"] == 0)
    dm = np.abs(rmx["m2lnl"] - r64["m2lnl"])
    assert dm.max() <= TOL_M2LNL, dm.max()
    gscale = np.abs(r64["grad"]).max(axis=1, keepdims=True)
    gerr = (np.abs(rmx["grad"] - r64["grad"]) / gscale).max()
    assert gerr <= TOL_GRAD, gerr


def test_mixed_per_element_maps_and_far_points():
    g = load_golden("nside8_lmax24")
    rng = np.random.default_rng(5)
    B = 8
    cls = np.vstack([g["cls"][0] * np.exp(rng.uniform(-0.9, 0.9, len(g["cls"][0]))) for _ in range(B)])
    maps = g["d"][None, :] * (1 + 0.2 * rng.standard_normal((B, 1)))
    with _ctx(g, "fp64", B) as c64, _ctx(g, "mixed", B, cl_ref=g["cls"][0], recenter="fixed") as cmx:
        r64 = c64.loglike(cls, maps, grad=True)
        rmx = cmx.loglike(cls, maps, grad=True)
    assert np.abs(rmx["m2lnl"] - r64["m2lnl"]).max() <= TOL_M2LNL
    gscale = np.abs(r64["grad"]).max(axis=1, keepdims=True)
    assert (np.abs(rmx["grad"] - r64["grad"]) / gscale).max() <= TOL_GRAD


def test_recentre_policies():
    g = load_golden("nside4")
    cls = W.lognormal_batch(g["cls"][0], 6, 3)
    far = cls * 5.0
    far[:, :2] = 0
    with _ctx(g, "fp64", 6) as c64:
        ref_near = c64.loglike(cls, g["d"])["m2lnl"]
        ref_far = c64.loglike(far, g["d"])["m2lnl"]
    with _ctx(g, "mixed", 6, cl_ref=g["cls"][0], recenter="auto", recenter_radius=1.0) as ctx:
        assert ctx.reference_count() == 1
        assert np.abs(ctx.loglike(cls, g["d"])["m2lnl"] - ref_near).max() <= TOL_M2LNL
        assert ctx.reference_count() == 1      # within the radius: no re-centre
        assert np.abs(ctx.loglike(far, g["d"])["m2lnl"] - ref_far).max() <= TOL_M2LNL
        assert ctx.reference_count() == 2      # ln 5 > 1: re-centred
    with _ctx(g, "mixed", 6, recenter="batch") as ctx:
        ctx.loglike(cls, g["d"])
        ctx.loglike(cls, g["d"])
        assert ctx.reference_count() == 2
    with _ctx(g, "mixed", 6, cl_ref=g["cls"][0], recenter="fixed") as ctx:
        r = ctx.loglike(far, g["d"])   # far from a fixed reference: still a correct answer (cond ~ 5)
        assert ctx.reference_count() == 1
        assert np.abs(r["m2lnl"] - ref_far).max() <= TOL_M2LNL


def test_mixed_nonfinite_status():
    g = load_golden("nside4")
    cls = np.vstack([g["cls"][0]] * 3)
    cls[1, 4] = np.inf
    with _ctx(g, "mixed", 3, cl_ref=g["cls"][0], recenter="fixed") as ctx:
        r = ctx.loglike(cls, g["d"])
    assert r["status"][0] == 0 and r["status"][2] == 0
    assert r["status"][1] == cg.CG_ERR_NONFINITE


def test_bounded_wait_reports_timeout_and_context_survives():
    """A device wait on a barrier that nothing completes gives up within its limit and reports
    CG_ERR_TIMEOUT (no fault, no hang); the same context then evaluates normally, and a
    timeout is reported on its own call only."""
    g = load_golden("nside4")
    B = len(g["cls"])
    with _ctx(g, "mixed", B) as ctx:
        assert ctx.selftest_wait_timeout() == cg.CG_ERR_TIMEOUT
        r = ctx.loglike(g["cls"], g["d"])
        assert ctx.selftest_wait_timeout() == cg.CG_ERR_TIMEOUT
        r2 = ctx.loglike(g["cls"], g["d"])
    for res in (r, r2):
        assert np.all(res["status"] == 0)
        assert np.abs(res["m2lnl"] - g["m2lnl"]).max() <= TOL_M2LNL


def test_mixed_against_oracle_nside16(oracle_mod):
    """Two elements of an nside-16 batch straight against the CPU oracle (FP64)."""
    g = load_golden("nside16_lmax47")
    cls = W.lognormal_batch(g["cls"][0], 4, 21)
    xyz = oracle_mod.unit_vectors(16, g["nest_good"], "NEST")
    with _ctx(g, "mixed", 4) as ctx:
        r = ctx.loglike(cls, g["d"], grad=True)
    for b in (0, 3):
        e = oracle_mod.evaluate(cls[b], xyz, float(g["fwhm_deg"]), float(g["sigma"]) ** 2, g["d"], grad=True)
        assert abs(r["m2lnl"][b] - e["m2lnl"]) <= TOL_M2LNL
        assert np.abs(r["grad"][b] - e["grad"]).max() <= TOL_GRAD * np.abs(e["grad"]).max()
