"""Host-side checks of the C-ABI library (no GPU needed): it loads, exports
every symbol include/cosmopp_gb300.h declares, its HEALPix geometry and beam
agree with the oracle's (and hence the reference's), and context creation
fails with a clear error when there is no usable device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden

import cosmopp_gb300 as cg


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "cosmopp_gb300.h")).read()
    return sorted(set(re.findall(r"\b(cg_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    L = cg.library()
    names = _declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name


def test_healpix_matches_oracle(oracle_mod):
    for ns in (1, 2, 4, 8, 16):
        npix = 12 * ns * ns
        ring = np.arange(npix)
        assert np.array_equal(cg.ring2nest(ns, ring), oracle_mod.ring2nest(ns, ring))
        assert np.array_equal(cg.nest2ring(ns, ring), oracle_mod.nest2ring(ns, ring))
        for scheme in ("RING", "NEST"):
            a = cg.pix2vec(ns, None, scheme)
            b = oracle_mod.unit_vectors(ns, None, scheme)
            assert np.array_equal(a, b)


def test_unit_vectors_bitwise_equal_to_reference_inputs(oracle_mod):
    g = load_golden("nside16_lmax47")
    a = cg.pix2vec(16, g["nest_good"], "NEST")
    b = oracle_mod.unit_vectors(16, g["nest_good"], "NEST")
    assert np.array_equal(a, b)
    assert np.array_equal(cg.pix2vec(16, g["ring_kept"], "RING"), a)


def test_beam_matches_oracle(oracle_mod):
    for fwhm in (0.0, 110 / 60, 220 / 60, 440 / 60, 10.0):
        for l in range(0, 100, 7):
            assert cg.beam(l, fwhm) == oracle_mod.beam(l, fwhm)


def test_invalid_pixel_is_rejected():
    with pytest.raises(cg.CGError):
        cg.pix2vec(2, [48], "RING")


def test_create_without_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cg.CGError) as ei:
        cg.Context(lmax=8, fwhm_deg=7.0, nside=2)
    assert ei.value.code == cg.CG_ERR_NO_DEVICE


def test_bad_config_rejected_before_device():
    with pytest.raises(cg.CGError) as ei:
        cg.Context(lmax=1, fwhm_deg=7.0, nside=2)
    assert ei.value.code == cg.CG_ERR_BAD_ARG
    with pytest.raises(cg.CGError):
        cg.Context(lmax=8, fwhm_deg=7.0, nside=2, good_pixels=[0, 1, 999])


def test_new_entry_points_reject_bad_arguments_before_the_device():
    """Argument checks of the table, noise-matrix and polarisation entry points run before any
    device work; with valid arguments and no GPU the polarisation likelihood fails loudly."""
    import ctypes
    L = cg.library()
    assert L.cg_legendre_table(None, 0, 3, None) == cg.CG_ERR_BAD_ARG
    assert L.cg_noise_matrix_from_sims(None, 10, 4, None, None, None) == cg.CG_ERR_BAD_ARG
    h = ctypes.c_void_p()
    good = np.array([0, 1], dtype=np.int32)
    gp = good.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    c = np.zeros(8 * 9 // 2)
    ninv = np.eye(8)
    assert L.cg_likelihood_pol_create(ctypes.byref(h), 0, gp, 2, cg._p(c), cg._p(ninv), 0) == cg.CG_ERR_BAD_ARG
    bad = np.array([0, 7], dtype=np.int32)  # pixel 7 of 4
    assert L.cg_likelihood_pol_create(ctypes.byref(h), 4, bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 2,
                                      cg._p(c), cg._p(ninv), 0) == cg.CG_ERR_BAD_ARG
    with pytest.raises(cg.CGError) as ei:
        cg.LikelihoodPolarization(c[:5], 4, good, ninv)
    assert ei.value.code == cg.CG_ERR_BAD_ARG
    nan_c = c.copy()
    nan_c[0] = np.nan
    with pytest.raises(cg.CGError) as ei:
        cg.LikelihoodPolarization(nan_c, 4, good, ninv)
    assert ei.value.code == cg.CG_ERR_NONFINITE
    import torch
    if not torch.cuda.is_available():
        with pytest.raises(cg.CGError) as ei:
            cg.LikelihoodPolarization(c + np.concatenate([[1.0] * 36]), 4, good, ninv)
        assert ei.value.code == cg.CG_ERR_NO_DEVICE


def test_legendre_file_reader_and_writer_match_the_reference_format(oracle_mod, tmp_path):
    """The reference's own LegendrePolynomialContainer file reads into the values the oracle
    computes, and writes back byte for byte (no device needed for file I/O)."""
    g = load_golden("legendre_nside2_lmax8")
    path = os.path.join(ROOT, "tests", "golden", "legendre_nside2_lmax8.bin")
    lp = cg.LegendrePolynomialContainer(file_name=path)
    assert lp.lmax == int(g["lmax"]) and lp.npix == len(g["nest_good"])
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    want = oracle_mod.legendre_table(lp.lmax, xyz)
    assert np.array_equal(lp.table, want)
    j, i = 20, 7
    x = float(np.clip(xyz[i] @ xyz[j], -1, 1))
    assert lp.value(3, j, i) == want[3, j * (j + 1) // 2 + i]
    assert abs(lp.value(3, j, i) - 0.5 * (5 * x ** 3 - 3 * x)) < 1e-14
    out = tmp_path / "lp.bin"
    lp.write_into_file(str(out))
    assert open(out, "rb").read() == open(path, "rb").read()
    short = tmp_path / "short.bin"
    short.write_bytes(open(path, "rb").read()[:100])
    with pytest.raises(cg.CGError):
        cg.LegendrePolynomialContainer(file_name=str(short))


def test_memory_plan_without_a_device():
    """Admission sizing against an explicit budget needs no device: the nside-32 batch of 32 fits in
    180 GB, a budget below the fixed part admits nothing, and chunks never exceed max_batch."""
    from cosmopp_gb300 import workload as W
    wl = W.make("nside32_lmax95_b32")
    kw = dict(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
              noise_sigma=wl.sigma)
    p = cg.plan_memory(180 * 10 ** 9, precision="mixed", max_batch=32, **kw)
    assert p["chunk"] == 32 and p["max_batch_fit"] >= 32
    # the whitened table alone: tiles x 4096 entries x lpad (96) x 4 bytes
    nt = 2 * ((wl.n + 127) // 128)
    assert p["bytes_fixed"] > nt * (nt + 1) // 2 * 4096 * 96 * 4
    small = cg.plan_memory(p["bytes_fixed"], precision="mixed", max_batch=32, **kw)
    assert small["max_batch_fit"] == 0 and small["chunk"] == 0
    mid = cg.plan_memory(p["bytes_fixed"] + p["bytes_reserve"] + 5 * p["bytes_per_element"] + 10 ** 9,
                         precision="mixed", max_batch=32, **kw)
    assert 1 <= mid["chunk"] < 32
    with pytest.raises(cg.CGError):
        cg.plan_memory(10 ** 9, precision="mixed", max_batch=0, **kw)
