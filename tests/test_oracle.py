"""The oracle restatement pinned to the reference's own outputs (golden
fixtures made by tests/golden/make_golden.py from the reference compiled from
its sources) and to the reference's known-answer tests."""
import hashlib
import os

import numpy as np
import pytest

from conftest import ROOT, load_golden
from cosmopp_gb300 import workload as W

DET_OFFSET = 29677.0566


def test_reference_kats_legendre_and_matrix(oracle_mod):
    kat = load_golden("kat_reference")
    for which, idx, res, exp in zip(kat["which"], kat["index"], kat["result"], kat["expected"]):
        # the reference's own tests pass at its default precision (rel 1e-5)
        assert abs(res - exp) <= 1e-5 * max(1.0, abs(exp)), (which, idx)
    # the oracle's Legendre reproduces the reference's results exactly
    legendre_args = [(4, 2.0), (10, 0.5), (64, 0.1), (1000, -0.25), (10000, -0.5)]
    for (l, x), res in zip(legendre_args, kat["result"][:5]):
        assert oracle_mod.legendre(l, x) == res


def test_oracle_2x2_cholesky_invert_and_determinant(oracle_mod):
    # source/test_matrix.cpp:417-488: [[2,1],[1,3]] invert, [[3,2],[2,4]] determinant
    ap = np.array([2.0, 1.0, 3.0])
    u, info = oracle_mod.dpptrf(ap)
    assert info == 0
    inv, info = oracle_mod.dpptri(u)
    assert info == 0
    full = W.packed_to_full(inv, 2)
    assert np.allclose(full @ np.array([[2, 1], [1, 3.0]]), np.eye(2), atol=1e-12)
    u2, _ = oracle_mod.dpptrf(np.array([3.0, 2.0, 4.0]))
    sign = np.array([0], dtype=np.int32)
    ld = oracle_mod.lib().orc_logdet_from_chol(2, u2.ctypes.data_as(oracle_mod._dp),
                                               sign.ctypes.data_as(oracle_mod._ip))
    assert abs(np.exp(ld) - 8.0) < 1e-12


def test_oracle_not_positive_definite_reports_info(oracle_mod):
    _, info = oracle_mod.dpptrf(np.array([1.0, 2.0, 1.0]))  # [[1,2],[2,1]] is indefinite
    assert info == 2


@pytest.mark.parametrize("name", ["nside1", "nside2", "nside4", "nside8_lmax24", "nside16_lmax47"])
def test_oracle_cmatrix_matches_reference_bitwise(oracle_mod, name):
    g = load_golden(name)
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    c = oracle_mod.cl_to_cmatrix(g["cls"][0], xyz, float(g["fwhm_deg"]))
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["c_sha256"])
    if "c_packed" in g:
        assert np.array_equal(c, g["c_packed"])
    # RING indices give the same directions as their NEST images
    xyz_r = oracle_mod.unit_vectors(int(g["nside"]), g["ring_kept"], "RING")
    assert np.array_equal(xyz, xyz_r)


@pytest.mark.parametrize("name", ["fid_nside4", "fid_nside8"])
def test_oracle_fiducial_matrix_matches_reference_bitwise(oracle_mod, name):
    """getFiducialMatrix (source/c_matrix_generator.cpp:706-772) and the low-l flow that uses it."""
    g = load_golden(name)
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    fid = oracle_mod.fiducial_matrix(g["cl_full"], xyz, int(g["lmax"]), float(g["fwhm_deg"]))
    assert hashlib.sha256(fid.tobytes()).hexdigest() == str(g["fid_sha256"])
    if "fid_packed" in g:
        assert np.array_equal(fid, g["fid_packed"])
    n = len(g["nest_good"])
    c = oracle_mod.cl_to_cmatrix(g["cl_full"][:int(g["lmax"]) + 1], xyz, float(g["fwhm_deg"]))
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["c_sha256"])
    noise = np.zeros_like(c)
    idx = np.arange(n)
    noise[idx * (idx + 1) // 2 + idx] = float(g["sigma"]) ** 2
    like, chi2, ld, _, st = oracle_mod.likelihood(c, noise, g["d"], fid_packed=fid)
    assert st == 0
    assert abs(chi2 - float(g["chi2"])) <= 1e-9 * abs(float(g["chi2"]))
    assert abs((like + DET_OFFSET) - float(g["like_ref"])) <= 1e-8 * abs(float(g["like_ref"]))


@pytest.mark.parametrize("name", ["nside1", "nside2", "nside4", "nside8_lmax24"])
def test_oracle_likelihood_matches_reference(oracle_mod, name):
    g = load_golden(name)
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    for k, cl in enumerate(g["cls"]):
        e = oracle_mod.evaluate(cl, xyz, float(g["fwhm_deg"]), float(g["sigma"]) ** 2, g["d"], grad=False)
        assert e["status"] == 0
        assert abs(e["logdet"] - g["logdet_raw"][k]) <= 1e-9 * abs(g["logdet_raw"][k])
        assert abs(e["chi2"] - g["chi2"][k]) <= 1e-9 * abs(g["chi2"][k])
        assert abs((e["logdet"] + DET_OFFSET) - g["logdet_ref"][k]) <= 1e-8


@pytest.mark.parametrize("name", ["nside1", "nside2", "nside4", "nside8_lmax24"])
def test_oracle_adjoint_gradient_matches_reference_fd(oracle_mod, name):
    g = load_golden(name)
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    e = oracle_mod.evaluate(g["cls"][0], xyz, float(g["fwhm_deg"]), float(g["sigma"]) ** 2, g["d"], grad=True)
    scale = np.abs(g["fd_grad"]).max()
    for ell, fd in zip(g["fd_ells"], g["fd_grad"]):
        # central differences at step 1e-4 C_l carry O(h^2) truncation + roundoff of the reference
        assert abs(e["grad"][ell] - fd) <= 1e-5 * abs(fd) + 1e-7 * scale, (ell, e["grad"][ell], fd)


def test_single_pass_recurrence_equals_reference_restart(oracle_mod):
    g = load_golden("nside4")
    xyz = oracle_mod.unit_vectors(4, g["nest_good"], "NEST")
    a = oracle_mod.cl_to_cmatrix(g["cls"][1], xyz, float(g["fwhm_deg"]), restart=True)
    b = oracle_mod.cl_to_cmatrix(g["cls"][1], xyz, float(g["fwhm_deg"]), restart=False)
    assert np.array_equal(a, b)


def test_healpix_ring_nest_roundtrip(oracle_mod):
    for ns in (1, 2, 4, 8, 16):
        npix = 12 * ns * ns
        r = np.arange(npix)
        nest = oracle_mod.ring2nest(ns, r)
        assert sorted(nest.tolist()) == list(range(npix))
        assert np.array_equal(oracle_mod.nest2ring(ns, nest), r)
    # nside 1 base pixels: rings at z = 2/3, 0, -2/3 (Gorski et al. 2005, fig. 3)
    xyz = oracle_mod.unit_vectors(1, None, "RING")
    assert np.allclose(xyz[:4, 2], 2 / 3) and np.allclose(xyz[4:8, 2], 0) and np.allclose(xyz[8:, 2], -2 / 3)
    assert np.allclose(np.arctan2(xyz[4:8, 1], xyz[4:8, 0]) % (2 * np.pi), [0, np.pi / 2, np.pi, 3 * np.pi / 2])


def test_oracle_noise_matrix_matches_an_independent_restatement(oracle_mod):
    """calculateNoiseMatrix's averaging loop (source/c_matrix_generator.cpp:887-910) needs the
    HEALPix transforms to run as shipped, so its oracle is pinned to a second restatement:
    the same k-ordered sums formed as numpy rank-1 updates, every product and sum rounded on
    its own, then divided by the simulation count."""
    rng = np.random.default_rng(12)
    for nsims, n in ((1, 5), (37, 61), (150, 130)):
        sims = rng.standard_normal((nsims, n))
        acc = np.zeros((n, n))
        for k in range(nsims):
            acc += np.outer(sims[k], sims[k])
        acc /= nsims
        want = np.concatenate([acc[:j + 1, j] for j in range(n)])
        got, mx = oracle_mod.noise_matrix(sims)
        assert np.array_equal(got, want)
        means = np.zeros(n)
        for k in range(nsims):
            means += sims[k]
        assert mx == np.abs(means / nsims).max()


def test_oracle_legendre_table_matches_reference_file(oracle_mod):
    """The reference's LegendrePolynomialContainer, written by its own writeIntoFile
    (tests/golden/legendre_nside2_lmax8.bin), equals the oracle's table bit for bit; the
    covariance the reference computes from that file read back equals its plain one."""
    g = load_golden("legendre_nside2_lmax8")
    lmax, npix, tab = oracle_mod.read_legendre_file(os.path.join(ROOT, "tests", "golden", "legendre_nside2_lmax8.bin"))
    assert lmax == int(g["lmax"]) and npix == len(g["nest_good"])
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    assert np.array_equal(oracle_mod.legendre_table(lmax, xyz), tab)
    assert np.array_equal(g["c_lp"], g["c_plain"])


def test_oracle_pol_algebra_matches_the_reference_itself(oracle_mod):
    """The oracle's numpy restatement of LikelihoodPolarization's pixel algebra against the
    reference's own compiled class (fixture: make_golden.py, part pol; zero E-mode template)."""
    g = load_golden("pol_nside4_reference")
    rng = np.random.default_rng(int(g["seed"]))
    npix = int(g["npix"])
    size = 2 * npix
    a = rng.standard_normal((size, size)) / np.sqrt(size)
    c = a @ a.T + 0.5 * np.eye(size)
    b = rng.standard_normal((size, size)) / np.sqrt(size)
    ninv = np.ascontiguousarray(b @ b.T + 2.0 * np.eye(size))
    good = np.flatnonzero(rng.uniform(size=npix) < 0.8).astype(np.int32)
    c_packed = np.concatenate([c[:j + 1, j] for j in range(size)])
    assert np.array_equal(good, g["good"])
    for v, chi2_r, ld_r in zip(g["v"], g["chi2"], g["logdet_ref"]):
        chi2, ld = oracle_mod.likelihood_pol(c_packed, npix, good, ninv, v, np.zeros_like(v))
        assert abs(chi2 - chi2_r) <= 1e-9 * abs(chi2_r)
        assert abs((ld - float(g["det_offset"])) - ld_r) <= 1e-9 * abs(ld_r)


def test_oracle_noise_matrix_bit_identical_to_the_reference_itself(oracle_mod):
    """The oracle's averaging loop against the reference's own calculateNoiseMatrix on the 1000
    simulated maps it averaged (fixture: make_golden.py, part noise): bit-identical."""
    g = load_golden("noise_nside2_reference")
    packed, _ = oracle_mod.noise_matrix(g["sims"])
    assert np.array_equal(packed, g["noise_packed"])
