"""ctypes front end of the oracle restatement (oracle/cg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py`` as the checker / the timed CPU arm.  The
``cosmopp_gb300`` package never imports it.

Also loads, when it has been built here, the reference's own code compiled by
``oracle/ref/Makefile`` into ``oracle/_ref/libcg_ref.so`` (``ref()``).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libcg_oracle.so")
_REF = os.path.join(_HERE, "_ref", "libcg_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None
_ref = None


def build():
    """Compile the oracle restatement (gcc, OpenMP)."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "CC=gcc"])


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = ctypes.CDLL(_LIB)
        L.orc_legendre.restype = ctypes.c_double
        L.orc_legendre.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_beam.restype = ctypes.c_double
        L.orc_beam.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_unit_vectors.argtypes = [ctypes.c_long, ctypes.c_int, _ip, ctypes.c_int, _dp]
        L.orc_cl_to_cmatrix.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_fiducial_matrix.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_dpptrf.argtypes = [ctypes.c_int, _dp]
        L.orc_dpptri.argtypes = [ctypes.c_int, _dp]
        L.orc_logdet_from_chol.restype = ctypes.c_double
        L.orc_logdet_from_chol.argtypes = [ctypes.c_int, _dp, _ip]
        L.orc_vmv.restype = ctypes.c_double
        L.orc_vmv.argtypes = [ctypes.c_int, _dp, _dp, _dp]
        L.orc_likelihood_construct.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_likelihood_calculate.restype = ctypes.c_double
        L.orc_likelihood_calculate.argtypes = [ctypes.c_int, _dp, ctypes.c_double, _dp, _dp, _dp, _dp]
        L.orc_eval.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double, _dp, _dp, ctypes.c_int,
                               _dp, _dp, _dp, _dp]
        L.orc_adjoint.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_noise_matrix.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.orc_legendre_table.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp]
        L.orc_loglike_extended.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        L.hp_ring2nest.restype = ctypes.c_long
        L.hp_ring2nest.argtypes = [ctypes.c_long, ctypes.c_long]
        L.hp_nest2ring.restype = ctypes.c_long
        L.hp_nest2ring.argtypes = [ctypes.c_long, ctypes.c_long]
        _lib = L
    return _lib


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


def ring2nest(nside, ring):
    L = lib()
    return np.array([L.hp_ring2nest(nside, int(r)) for r in ring], dtype=np.int32)


def nest2ring(nside, nest):
    L = lib()
    return np.array([L.hp_nest2ring(nside, int(p)) for p in nest], dtype=np.int32)


def legendre(l, x):
    return lib().orc_legendre(int(l), float(x))


def beam(l, fwhm_deg):
    return lib().orc_beam(int(l), float(fwhm_deg))


def unit_vectors(nside, good=None, scheme="NEST"):
    """Pixel unit vectors [n, 3] (source/c_matrix_generator.cpp:178-185)."""
    sch = 1 if scheme.upper() == "NEST" else 0
    if good is None:
        n = 12 * nside * nside
        g = None
    else:
        g = np.ascontiguousarray(good, dtype=np.int32)
        n = len(g)
    out = np.zeros((n, 3))
    lib().orc_unit_vectors(nside, sch, None if g is None else g.ctypes.data_as(_ip), n, _p(out))
    return out


def cl_to_cmatrix(cl, xyz, fwhm_deg, restart=False):
    """Packed-upper C (source/c_matrix_generator.cpp:164-232)."""
    cl = np.ascontiguousarray(cl, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    out = np.zeros(n * (n + 1) // 2)
    lib().orc_cl_to_cmatrix(_p(cl), len(cl) - 1, _p(xyz), n, float(fwhm_deg), int(bool(restart)), _p(out))
    return out


def fiducial_matrix(cl, xyz, lmax, fwhm_deg):
    cl = np.ascontiguousarray(cl, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    out = np.zeros(n * (n + 1) // 2)
    lib().orc_fiducial_matrix(_p(cl), len(cl) - 1, _p(xyz), n, int(lmax), float(fwhm_deg), _p(out))
    return out


def dpptrf(ap):
    a = np.array(ap, dtype=np.float64)
    n = int(round((np.sqrt(8 * len(a) + 1) - 1) / 2))
    info = lib().orc_dpptrf(n, _p(a))
    return a, info


def dpptri(ap_chol):
    a = np.array(ap_chol, dtype=np.float64)
    n = int(round((np.sqrt(8 * len(a) + 1) - 1) / 2))
    info = lib().orc_dpptri(n, _p(a))
    return a, info


def likelihood(c_packed, noise_packed, t, fid_packed=None, foreground=None):
    """(like, chi2, logdet_ref_style_without_offset, logdet_raw, status) for the reference's
    Likelihood ctor + calculate (source/likelihood.cpp:69-180)."""
    c = np.ascontiguousarray(c_packed, dtype=np.float64)
    nz = np.ascontiguousarray(noise_packed, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    n = len(t)
    cinv = np.zeros_like(c)
    ldr = ctypes.c_double(0)
    fid = None if fid_packed is None else np.ascontiguousarray(fid_packed, dtype=np.float64)
    st = lib().orc_likelihood_construct(n, _p(c), _p(fid), _p(nz), _p(cinv), ctypes.byref(ldr))
    if st:
        return None, None, None, None, st
    chi2 = ctypes.c_double(0)
    ld = ctypes.c_double(0)
    fg = None if foreground is None else np.ascontiguousarray(foreground, dtype=np.float64)
    like = lib().orc_likelihood_calculate(n, _p(cinv), ldr.value, _p(t), _p(fg), ctypes.byref(chi2), ctypes.byref(ld))
    return like, chi2.value, ld.value, ldr.value, 0


def evaluate(cl, xyz, fwhm_deg, noise_var, d, grad=True, restart=False):
    """One -2lnL (+ d(-2lnL)/dC_l) evaluation: dict(m2lnl, chi2, logdet, grad, status)."""
    cl = np.ascontiguousarray(cl, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    nv = np.broadcast_to(np.asarray(noise_var, dtype=np.float64), (n,)).copy()
    d = np.ascontiguousarray(d, dtype=np.float64)
    m2 = ctypes.c_double(0)
    chi2 = ctypes.c_double(0)
    ld = ctypes.c_double(0)
    g = np.zeros(len(cl)) if grad else None
    st = lib().orc_eval(_p(cl), len(cl) - 1, _p(xyz), n, float(fwhm_deg), _p(nv), _p(d), int(bool(restart)),
                        ctypes.byref(m2), ctypes.byref(chi2), ctypes.byref(ld), _p(g))
    return dict(m2lnl=m2.value, chi2=chi2.value, logdet=ld.value, grad=g, status=st)


def loglike_extended(c_packed, noise_var, d):
    """chi2 and raw ln det of C + diag(noise_var) in extended precision (long double): the
    yardstick the FP64 paths' rounding noise is measured against.  Returns (chi2, logdet, info)."""
    c = np.ascontiguousarray(c_packed, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = len(d)
    nv = np.broadcast_to(np.asarray(noise_var, dtype=np.float64), (n,)).copy()
    chi2, ld = ctypes.c_double(0), ctypes.c_double(0)
    info = lib().orc_loglike_extended(n, _p(c), _p(nv), _p(d), ctypes.byref(chi2), ctypes.byref(ld))
    return chi2.value, ld.value, info


def adjoint(w_packed, lmax, xyz, fwhm_deg):
    w = np.ascontiguousarray(w_packed, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    g = np.zeros(lmax + 1)
    lib().orc_adjoint(_p(w), int(lmax), _p(xyz), xyz.shape[0], float(fwhm_deg), _p(g))
    return g


def legendre_table(lmax, xyz):
    """LegendrePolynomialContainer's table (source/c_matrix_generator.cpp:30-76):
    [lmax + 1, n(n+1)/2] with P_l(x_ij) at j(j+1)/2 + i."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    out = np.zeros((lmax + 1, n * (n + 1) // 2))
    lib().orc_legendre_table(int(lmax), _p(xyz), n, _p(out))
    return out


def read_legendre_file(path):
    """A LegendrePolynomialContainer file (source/c_matrix_generator.cpp:89-134): int lMax,
    int nPix, then (lMax + 1) packed tables -> (lmax, npix, [lmax + 1, npix(npix+1)/2])."""
    raw = open(path, "rb").read()
    lmax, npix = np.frombuffer(raw[:8], dtype=np.int32)
    data = np.frombuffer(raw[8:], dtype=np.float64)
    return int(lmax), int(npix), data.reshape(int(lmax) + 1, int(npix) * (int(npix) + 1) // 2)


def likelihood_pol(c_packed, npix, good, ninv, v, subtract):
    """LikelihoodPolarization's pixel-space algebra (source/likelihood.cpp:341-401,536-612) in
    numpy FP64: keep the Q and U rows / columns of the kept pixels, cInv = N^-1 + N^-1 C N^-1,
    logDet = ln det cInv (raw, without detOffset), w = v - N^-1 subtract, chi2 = w^T cInv^-1 w.
    Returns (chi2, logdet_raw)."""
    size = 2 * npix
    c = np.zeros((size, size))
    iu = np.triu_indices(size)
    c[iu[0], iu[1]] = np.asarray(c_packed)[iu[1] * (iu[1] + 1) // 2 + iu[0]]
    c = c + np.triu(c, 1).T
    idx = np.concatenate([np.asarray(good), npix + np.asarray(good)])
    cm = c[np.ix_(idx, idx)]
    nm = np.asarray(ninv).reshape(size, size)[np.ix_(idx, idx)]
    m = nm + nm @ (cm @ nm)
    sign, logdet = np.linalg.slogdet(m)
    w = np.asarray(v) - nm @ np.asarray(subtract)
    chi2 = float(w @ np.linalg.solve(m, w))
    return chi2, float(logdet) if sign > 0 else float("nan")


def noise_matrix(sims):
    """Averaging step of calculateNoiseMatrix (source/c_matrix_generator.cpp:887-910) over
    sims [nsims, n]: (packed noise matrix, max |per-pixel mean|)."""
    sims = np.ascontiguousarray(sims, dtype=np.float64)
    ns, n = sims.shape
    out = np.zeros(n * (n + 1) // 2)
    mx = ctypes.c_double(0)
    lib().orc_noise_matrix(ns, n, _p(sims), _p(out), ctypes.byref(mx))
    return out, mx.value


# ---- the reference itself, compiled here by oracle/ref/Makefile (absent on machines
#      without the reference sources) ----

def ref_available(variant=""):
    return os.path.exists(_REF.replace(".so", variant + ".so"))


def ref(variant=""):
    """The compiled reference: variant "" is the strict -O2 build, "_fastmath" the build with
    the reference's shipped -ffast-math flags (make -C oracle/ref fastmath)."""
    global _ref
    if variant:
        return _bind_ref(ctypes.CDLL(_REF.replace(".so", variant + ".so")))
    if _ref is None:
        _ref = _bind_ref(ctypes.CDLL(_REF))
    return _ref


def _bind_ref(R):
    R.ref_last_error.restype = ctypes.c_char_p
    R.ref_legendre.restype = ctypes.c_double
    R.ref_legendre.argtypes = [ctypes.c_int, ctypes.c_double]
    R.ref_beam.restype = ctypes.c_double
    R.ref_beam.argtypes = [ctypes.c_int, ctypes.c_double]
    R.ref_cl_to_cmatrix.argtypes = [_dp, ctypes.c_int, ctypes.c_long, ctypes.c_double, _ip, ctypes.c_int, _dp]
    R.ref_likelihood.argtypes = [_dp, ctypes.c_int, ctypes.c_long, ctypes.c_double, _ip, ctypes.c_int,
                                 ctypes.c_double, _dp, _dp, _dp, _dp]
    R.ref_likelihood_packed.argtypes = [_dp, _dp, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
    R.ref_fiducial_matrix.argtypes = [_dp, ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_double, _ip,
                                      ctypes.c_int, _dp]
    R.ref_pixel_window.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_double, _dp]
    R.ref_run_subtest.argtypes = [ctypes.c_char_p, ctypes.c_int, _dp, _dp]
    return R
