"""Parity of the plain FP64 CUDA path with the reference (golden fixtures made
from the reference's own code) and with the oracle restatement.

Bars: the covariance matrix is bit-identical (integer-exact comparison of
the FP64 words); -2lnL, chi2 and ln det within 1e-6 absolute of the
reference at every nside.  The FP64 rounding noise of the reference itself,
measured against an extended-precision (long double) evaluation of the same
covariance, is at most 2.4e-10 over 100 nside-16 vectors
(tests/golden/config2_nside16.npz), so 1e-6 is not below the noise floor.
The adjoint gradient is checked per component: within 1e-4 relative of the
reference's central finite differences, and within 1e-8 of the oracle's FP64
adjoint relative to max(|g_l|, s_l), s_l the gradient's minimum statistical
scatter (conftest.grad_scale)."""
import hashlib

import numpy as np
import pytest

from conftest import assert_grad_close, grad_scale, load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu

CASES = ["nside1", "nside2", "nside4", "nside8_lmax24", "nside16_lmax47"]


def _ctx(g, max_batch=4, **kw):
    return cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=int(g["nside"]),
                      good_pixels=g["nest_good"], scheme="NEST", noise_sigma=float(g["sigma"]),
                      max_batch=max_batch, precision="fp64", **kw)


@pytest.mark.parametrize("name", CASES)
def test_cmatrix_bit_identical_to_reference(name):
    g = load_golden(name)
    with _ctx(g) as ctx:
        c = ctx.build_cmatrix(g["cls"][0])
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["c_sha256"])
    assert np.array_equal(c[:len(g["c_head"])], g["c_head"])
    if "c_packed" in g:
        assert np.array_equal(c, g["c_packed"])


@pytest.mark.parametrize("name", ["fid_nside4", "fid_nside8"])
def test_fiducial_matrix_bit_identical_and_low_l_flow(name):
    """getFiducialMatrix on the GPU, bit for bit, then Likelihood(C, fiducial, N) as
    source/test_like_low.cpp:181-193 uses it."""
    g = load_golden(name)
    lmax, lmax_max = int(g["lmax"]), int(g["lmax_max"])
    with cg.Context(lmax=lmax, fwhm_deg=float(g["fwhm_deg"]), nside=int(g["nside"]), good_pixels=g["nest_good"],
                    scheme="NEST", noise_sigma=float(g["sigma"]), precision="fp64") as ctx:
        fid = ctx.fiducial_matrix(g["cl_full"], lmax_max)
        c = ctx.build_cmatrix(g["cl_full"][:lmax + 1])
        # an explicit beam table gives the same words as the context's Gaussian beam
        beam = np.array([cg.beam(l, float(g["fwhm_deg"])) for l in range(lmax_max + 1)])
        assert np.array_equal(ctx.fiducial_matrix(g["cl_full"], lmax_max, beam=beam), fid)
        with pytest.raises(cg.CGError):
            ctx.fiducial_matrix(g["cl_full"], lmax)  # lmax_max must exceed lmax
    assert hashlib.sha256(fid.tobytes()).hexdigest() == str(g["fid_sha256"])
    assert np.array_equal(fid[:len(g["fid_head"])], g["fid_head"])
    if "fid_packed" in g:
        assert np.array_equal(fid, g["fid_packed"])
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["c_sha256"])
    n = len(g["nest_good"])
    noise = np.zeros_like(c)
    idx = np.arange(n)
    noise[idx * (idx + 1) // 2 + idx] = float(g["sigma"]) ** 2
    like, chi2, logdet = cg.Likelihood(c, fid, noise, good_pixels=g["nest_good"]).calculate(g["d"])
    assert abs(chi2 - float(g["chi2"])) <= 1e-6
    assert abs(like - float(g["like_ref"])) <= 1e-6


def test_cmatrix_batched_matches_single(oracle_mod):
    g = load_golden("nside4")
    with _ctx(g) as ctx:
        cb = ctx.build_cmatrix(g["cls"])
        for k in range(len(g["cls"])):
            assert np.array_equal(cb[k], ctx.build_cmatrix(g["cls"][k]))
    xyz = oracle_mod.unit_vectors(4, g["nest_good"], "NEST")
    assert np.array_equal(cb[2], oracle_mod.cl_to_cmatrix(g["cls"][2], xyz, float(g["fwhm_deg"])))


@pytest.mark.parametrize("name", CASES)
def test_loglike_matches_reference(name):
    g = load_golden(name)
    B = len(g["cls"])
    with _ctx(g, max_batch=B) as ctx:
        r = ctx.loglike(g["cls"], g["d"], grad=False)
    assert np.all(r["status"] == 0)
    tol = 1e-6
    assert np.abs(r["logdet"] - g["logdet_raw"]).max() <= tol
    assert np.abs(r["chi2"] - g["chi2"]).max() <= tol
    assert np.abs(r["m2lnl"] - g["m2lnl"]).max() <= tol


def test_plain_fp64_workload_100_vectors_against_reference_and_extended_precision():
    """The plain FP64 workload at nside 16 (100 lognormal C_l vectors): every -2lnL within 1e-6 of
    the reference's, and of the extended-precision value of the same covariance; the fixture's own
    record of the reference's FP64 noise (strict and -ffast-math builds, restated LAPACK loops)
    against extended precision stays below 1e-8."""
    g = load_golden("config2_nside16")
    B = len(g["cls"])
    with _ctx(g, max_batch=B) as ctx:
        r = ctx.loglike(g["cls"], g["d"], grad=False)
    assert np.all(r["status"] == 0)
    d_ref = np.abs(r["m2lnl"] - g["m2lnl"]).max()
    d_ext = np.abs(r["m2lnl"] - g["m2lnl_ext"]).max()
    print("FP64 GPU, 100 vectors: max |d(-2lnL)| vs reference %.3e, vs extended %.3e" % (d_ref, d_ext))
    assert d_ref <= 1e-6 and d_ext <= 1e-6
    assert np.abs(r["chi2"] - g["chi2_ext"]).max() <= 1e-6
    assert np.abs(r["logdet"] - g["logdet_ext"]).max() <= 1e-6
    n10 = len(g["m2lnl_fastmath"])
    for key in ("m2lnl", "m2lnl_fastmath", "m2lnl_restated"):
        assert np.abs(g[key][:n10] - g["m2lnl_ext"][:n10]).max() <= 1e-8, key


@pytest.mark.parametrize("name", ["nside2", "nside4", "nside8_lmax24", "nside16_lmax47"])
def test_gradient_matches_reference_fd_and_oracle(name, oracle_mod):
    g = load_golden(name)
    with _ctx(g, max_batch=1) as ctx:
        r = ctx.loglike(g["cls"][0], g["d"], grad=True)
        s = grad_scale(ctx, g["cls"][0], len(g["nest_good"]), int(g["lmax"]))
    grad = r["grad"]
    # the reference's central differences (step 1e-4 C_l) carry its -2lnL rounding noise (< 1e-9)
    # over 2h and an O(h^2) truncation: both far below 1e-4 of every component here
    for ell, fd in zip(g["fd_ells"], g["fd_grad"]):
        assert abs(grad[ell] - fd) <= 1e-4 * abs(fd), (ell, grad[ell], fd)
    if int(g["nside"]) <= 8:
        xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
        e = oracle_mod.evaluate(g["cls"][0], xyz, float(g["fwhm_deg"]), float(g["sigma"]) ** 2, g["d"], grad=True)
        assert_grad_close(grad, e["grad"], s, 1e-8, name)


def test_batch_elements_independent_and_per_map_data():
    g = load_golden("nside4")
    rng = np.random.default_rng(3)
    B = 5
    cls = np.vstack([g["cls"][0] * np.exp(0.1 * rng.standard_normal(len(g["cls"][0]))) for _ in range(B)])
    maps = g["d"][None, :] * (1 + 0.1 * rng.standard_normal((B, 1)))
    with _ctx(g, max_batch=B) as ctx:
        rb = ctx.loglike(cls, maps, grad=True)
        for b in range(B):
            r1 = ctx.loglike(cls[b], maps[b], grad=True)
            assert r1["m2lnl"] == rb["m2lnl"][b]
            assert np.array_equal(r1["grad"], rb["grad"][b])


def test_not_positive_definite_and_nonfinite_status():
    g = load_golden("nside2")
    cls = np.vstack([g["cls"][0], -g["cls"][0], g["cls"][0]])
    cls[2, 5] = np.nan
    with cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=2, good_pixels=g["nest_good"],
                    noise_sigma=0.0, max_batch=3) as ctx:
        r = ctx.loglike(cls, g["d"])
    assert r["status"][0] == cg.CG_OK
    assert r["status"][1] == cg.CG_ERR_NOT_PD
    assert r["status"][2] == cg.CG_ERR_NONFINITE


def test_bad_arguments_raise():
    g = load_golden("nside2")
    with _ctx(g, max_batch=2) as ctx:
        with pytest.raises(cg.CGError):
            ctx.loglike(np.vstack([g["cls"][0]] * 3), g["d"])


@pytest.mark.parametrize("name", ["nside2", "nside8_lmax24"])
def test_likelihood_dropin_matches_reference(name, oracle_mod):
    g = load_golden(name)
    n = len(g["nest_good"])
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    c = oracle_mod.cl_to_cmatrix(g["cls"][0], xyz, float(g["fwhm_deg"]))
    noise = np.zeros_like(c)
    idx = np.arange(n)
    noise[idx * (idx + 1) // 2 + idx] = float(g["sigma"]) ** 2
    lik = cg.Likelihood(c, np.zeros_like(c), noise, good_pixels=g["nest_good"])
    like, chi2, logdet = lik.calculate(g["d"])
    assert abs(logdet - g["logdet_ref"][0]) <= 1e-6
    assert abs(chi2 - g["chi2"][0]) <= 1e-6
    assert abs(like - g["like_ref"][0]) <= 1e-6
    # foreground marginalisation (source/likelihood.cpp:171-177) against the oracle
    fg = np.cos(3 * xyz[:, 2]) + 0.3 * xyz[:, 0]
    lik_f = cg.Likelihood(c, None, noise, foreground=fg)
    like_f, chi2_f, logdet_f = lik_f.calculate(g["d"])
    like_o, chi2_o, logdet_o, _, st = oracle_mod.likelihood(c, noise, g["d"], foreground=fg)
    assert st == 0
    assert abs(chi2_f - chi2_o) <= 1e-6
    assert abs((logdet_f - cg.DET_OFFSET) - logdet_o) <= 1e-6


def test_likelihood_dropin_rejects_indefinite():
    c = np.array([1.0, 2.0, 1.0])
    with pytest.raises(cg.CGError) as ei:
        cg.Likelihood(c, None, np.zeros(3))
    assert ei.value.code == cg.CG_ERR_NOT_PD


def test_loglike_with_derivs_interface_caches_gradient():
    g = load_golden("nside4")
    with _ctx(g, max_batch=1) as ctx:
        like = cg.LikelihoodWithDerivs(ctx, g["d"], g["cls"][0], lmin=2, log_params=True)
        x = np.log(g["cls"][0][2:])
        v = like.calculate(x, len(x))
        d0 = like.calculateDeriv(x, len(x), 0)
        h = 1e-5
        xp = x.copy(); xp[0] += h
        xm = x.copy(); xm[0] -= h
        fd = (like.calculate(xp, len(x)) - like.calculate(xm, len(x))) / (2 * h)
        assert abs(v - g["m2lnl"][0]) < 1e-6
        assert abs(d0 - fd) <= 1e-5 * max(1.0, abs(fd))
