"""The allocation-free likelihood entry point (cg_likelihood_noalloc), for
callers that cannot allocate device memory, against the allocating drop-in
(cg_likelihood_create / cg_likelihood_calculate) through the C ABI, on two
calls in a row with different sizes, so that the second call runs on the
workspace the first one left behind.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _case(name, oracle_mod, seed):
    g = load_golden(name)
    n = len(g["nest_good"])
    xyz = oracle_mod.unit_vectors(int(g["nside"]), g["nest_good"], "NEST")
    c = oracle_mod.cl_to_cmatrix(g["cls"][seed % len(g["cls"])], xyz, float(g["fwhm_deg"]))
    noise = np.zeros_like(c)
    i = np.arange(n)
    noise[i * (i + 1) // 2 + i] = float(g["sigma"]) ** 2
    t = np.asarray(g["d"]) * (1.0 + 0.05 * seed)
    return n, c, noise, t


def _noalloc(L, n, c, noise, t):
    import torch
    dev = torch.device("cuda", 0)
    dc = torch.tensor(c, dtype=torch.float64, device=dev)
    dn = torch.tensor(noise, dtype=torch.float64, device=dev)
    dt = torch.tensor(t, dtype=torch.float64, device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    st = torch.full((1,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = L.cg_likelihood_noalloc(n, ctypes.c_void_p(dc.data_ptr()), None, ctypes.c_void_p(dn.data_ptr()),
                                 ctypes.c_void_p(dt.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(st.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy(), int(st.cpu().item())


def _lib():
    L = cg.library()
    L.cg_likelihood_noalloc.restype = ctypes.c_int
    L.cg_likelihood_noalloc.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_void_p]
    return L


def test_noalloc_matches_allocating_entry_point_twice(oracle_mod):
    L = _lib()
    for name, seed in (("nside8_lmax24", 1), ("nside4", 2)):
        n, c, noise, t = _case(name, oracle_mod, seed)
        rc, out, st = _noalloc(L, n, c, noise, t)
        assert rc == 0, L.cg_last_error(None)
        assert st == 0
        lik = cg.Likelihood(c, None, noise)
        _, chi2, _ = lik.calculate(t)
        assert abs(out[0] - chi2) <= TOL * max(1.0, abs(chi2)), (name, out[0], chi2)
        assert abs(out[1] - lik.logdet_raw) <= TOL * max(1.0, abs(lik.logdet_raw)), (name, out[1], lik.logdet_raw)
        lik.close()


def test_noalloc_matches_reference_golden_and_allocates_nothing(oracle_mod):
    """Straight against the reference's own chi2 and ln det (golden fixture), and the property
    the entry point exists for: after a first call on the device, a call leaves the device's
    free memory unchanged."""
    import torch
    L = _lib()
    g = load_golden("nside8_lmax24")
    n, c, noise, t = _case("nside8_lmax24", oracle_mod, 0)
    rc, out, st = _noalloc(L, n, c, noise, t)
    assert rc == 0 and st == 0
    assert abs(out[0] - float(g["chi2"][0])) <= TOL, (out[0], g["chi2"][0])
    assert abs(out[1] - float(g["logdet_raw"][0])) <= TOL, (out[1], g["logdet_raw"][0])
    dev = torch.device("cuda", 0)
    dc = torch.tensor(c, dtype=torch.float64, device=dev)
    dn = torch.tensor(noise, dtype=torch.float64, device=dev)
    dt = torch.tensor(t, dtype=torch.float64, device=dev)
    res = torch.zeros(2, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    rc = L.cg_likelihood_noalloc(n, ctypes.c_void_p(dc.data_ptr()), None, ctypes.c_void_p(dn.data_ptr()),
                                 ctypes.c_void_p(dt.data_ptr()), ctypes.c_void_p(res.data_ptr()), None, None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert rc == 0
    assert free1 == free0, (free0, free1)
    assert np.array_equal(res.cpu().numpy(), out)


def test_noalloc_reports_not_positive_definite(oracle_mod):
    """An indefinite covariance: the call runs (CG_OK) and the device status word says
    CG_ERR_NOT_PD, as chol_diag set it."""
    L = _lib()
    n, c, noise, t = _case("nside4", oracle_mod, 0)
    rc, out, st = _noalloc(L, n, -c, noise, t)
    assert rc == 0, L.cg_last_error(None)
    assert st == cg.CG_ERR_NOT_PD
    # and the shared workspace serves a good matrix again on the next call
    rc, out, st = _noalloc(L, n, c, noise, t)
    assert rc == 0 and st == 0


def test_noalloc_rejects_sizes_beyond_its_workspace():
    L = _lib()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.cg_likelihood_noalloc(769, dummy, None, dummy, dummy, dummy, None, None)
    assert rc == cg.CG_ERR_BAD_ARG
    assert b"768" in L.cg_last_error(None)
