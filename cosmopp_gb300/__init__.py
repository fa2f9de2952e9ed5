"""cosmopp_gb300: GB300-native pixel-space CMB covariance and low-l TT likelihood.

Python front end over the C ABI (include/cosmopp_gb300.h) of the in-tree
library cosmopp_gb300/_lib/libcosmopp_gb300.so.  The Python names mirror the
reference's call surface:

* ``Context.build_cmatrix``  -- CMatrixGenerator::clToCMatrix
  (include/c_matrix_generator.hpp:53);
* ``Context.loglike``        -- Likelihood(C, 0, N, goodPixels).calculate(d)
  for a batch of C_l vectors, plus d(-2lnL)/dC_l (new);
* ``Likelihood``             -- the Likelihood class itself
  (include/likelihood.hpp:36-132) built from packed matrices;
* ``LikelihoodWithDerivs``   -- the Math::LikelihoodWithDerivs interface the
  reference's HMC consumes (include/likelihood_function.hpp:30-47).

There is no CPU fallback: if the library is missing, importing the compute
entry points raises.
"""
import ctypes
import os

import numpy as np

__all__ = ["Context", "Likelihood", "LikelihoodWithDerivs", "CGError", "library", "DET_OFFSET",
           "ring2nest", "nest2ring", "pix2vec", "beam", "mh_sample", "LegendrePolynomialContainer",
           "LikelihoodPolarization"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcosmopp_gb300.so")

# source/likelihood.cpp:127-128: the reference subtracts detOffset = -29677.0566 from ln det C
DET_OFFSET = 29677.0566
# source/likelihood.cpp:400-401: LikelihoodPolarization subtracts detOffset = 16078.083180
DET_OFFSET_POL = 16078.083180

CG_OK, CG_ERR_BAD_ARG, CG_ERR_NOT_PD, CG_ERR_NONFINITE, CG_ERR_TIMEOUT, CG_ERR_CUDA, CG_ERR_NO_DEVICE, \
    CG_ERR_ALLOC = range(8)
_STATUS_NAMES = {0: "OK", 1: "BAD_ARG", 2: "NOT_PD", 3: "NONFINITE", 4: "TIMEOUT", 5: "CUDA", 6: "NO_DEVICE",
                 7: "ALLOC"}
SCHEME = {"RING": 0, "NEST": 1}
PRECISION = {"fp64": 0, "mixed": 1}
RECENTER = {"fixed": 0, "batch": 1, "auto": 2}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class CGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cosmopp_gb300 error %s (%d): %s" % (_STATUS_NAMES.get(code, "?"), code, msg))
        self.code = code


class _Config(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_int), ("nside", ctypes.c_long), ("scheme", ctypes.c_int),
                ("good_pixels", _ip), ("n", ctypes.c_int), ("dirs", _dp), ("lmax", ctypes.c_int),
                ("fwhm_deg", ctypes.c_double), ("beam", _dp), ("noise_sigma", ctypes.c_double),
                ("noise_var", _dp), ("max_batch", ctypes.c_int), ("precision", ctypes.c_int),
                ("device", ctypes.c_int), ("cl_ref", _dp), ("recenter", ctypes.c_int),
                ("recenter_radius", ctypes.c_double)]


# int (*)(void* user, int nchains, const double* x, double* m2lnl)
_BATCH_LIKE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double))
_BATCH_LIKE_GRAD = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))

PRIOR = {"uniform": 0, "gauss": 1}

_lib = None


def library():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("cosmopp_gb300 native library not built (%s); run `python -m cosmopp_gb300.build`"
                          % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    L.cg_config_init.argtypes = [ctypes.POINTER(_Config)]
    L.cg_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_Config)]
    L.cg_destroy.argtypes = [ctypes.c_void_p]
    L.cg_last_error.restype = ctypes.c_char_p
    L.cg_last_error.argtypes = [ctypes.c_void_p]
    L.cg_get_n.argtypes = [ctypes.c_void_p]
    L.cg_unit_vectors.argtypes = [ctypes.c_void_p, _dp]
    L.cg_build_cmatrix.argtypes = [ctypes.c_void_p, _dp, _dp]
    L.cg_build_cmatrix_batched.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
    L.cg_fiducial_matrix.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp]
    L.cg_loglike.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _ip]
    L.cg_loglike_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
    L.cg_set_reference.argtypes = [ctypes.c_void_p, _dp]
    L.cg_reference_count.argtypes = [ctypes.c_void_p]
    L.cg_hmc_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int,
                             ctypes.c_double, _dp, ctypes.c_int, ctypes.c_ulonglong, _dp, _dp]
    _mh_tail = [_dp, _ip, _dp, _dp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_ulonglong, _dp, _dp, _dp]
    L.cg_mh_sample.argtypes = [ctypes.c_int, ctypes.c_int, _BATCH_LIKE, ctypes.c_void_p, _dp, ctypes.c_int] + _mh_tail
    L.cg_hmc_sample.argtypes = [ctypes.c_int, ctypes.c_int, _BATCH_LIKE_GRAD, ctypes.c_void_p, _dp, ctypes.c_int,
                                ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int, ctypes.c_ulonglong, _dp, _dp]
    L.cg_mh_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int] + _mh_tail
    L.cg_legendre_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp]
    L.cg_noise_matrix_from_sims.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    L.cg_selftest_wait_timeout.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    L.cg_probe_tf32_rate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
    L.cg_probe_fp32_rate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
    L.cg_plan_memory.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    L.cg_get_memory_plan.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.cg_tune_set.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    L.cg_tune_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _ip]
    L.cg_tune_describe.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    L.cg_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, _dp]
    L.cg_tune_load.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _ip]
    L.cg_launch_count.restype = ctypes.c_longlong
    L.cg_launch_count.argtypes = [ctypes.c_void_p]
    L.cg_graph_replays.restype = ctypes.c_longlong
    L.cg_graph_replays.argtypes = [ctypes.c_void_p]
    L.cg_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.cg_stage_times.argtypes = [ctypes.c_void_p, _dp]
    L.cg_likelihood_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int]
    L.cg_likelihood_calculate.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    L.cg_likelihood_pol_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _ip, ctypes.c_int, _dp, _dp,
                                           ctypes.c_int]
    L.cg_likelihood_pol_calculate.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
    L.cg_likelihood_logdet.restype = ctypes.c_double
    L.cg_likelihood_logdet.argtypes = [ctypes.c_void_p]
    L.cg_likelihood_destroy.argtypes = [ctypes.c_void_p]
    L.cg_likelihood_last_error.restype = ctypes.c_char_p
    L.cg_likelihood_last_error.argtypes = [ctypes.c_void_p]
    L.cg_nside2npix.restype = ctypes.c_long
    L.cg_nside2npix.argtypes = [ctypes.c_long]
    L.cg_ring2nest.restype = ctypes.c_long
    L.cg_ring2nest.argtypes = [ctypes.c_long, ctypes.c_long]
    L.cg_nest2ring.restype = ctypes.c_long
    L.cg_nest2ring.argtypes = [ctypes.c_long, ctypes.c_long]
    L.cg_pix2vec.argtypes = [ctypes.c_long, ctypes.c_int, _ip, ctypes.c_int, _dp]
    L.cg_beam.restype = ctypes.c_double
    L.cg_beam.argtypes = [ctypes.c_int, ctypes.c_double]
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---- HEALPix host helpers ---------------------------------------------------

def ring2nest(nside, ring):
    L = library()
    return np.array([L.cg_ring2nest(nside, int(r)) for r in np.atleast_1d(ring)], dtype=np.int32)


def nest2ring(nside, nest):
    L = library()
    return np.array([L.cg_nest2ring(nside, int(p)) for p in np.atleast_1d(nest)], dtype=np.int32)


def pix2vec(nside, pix=None, scheme="NEST"):
    L = library()
    if pix is None:
        n, pp = 12 * nside * nside, None
    else:
        pp = np.ascontiguousarray(pix, dtype=np.int32)
        n = len(pp)
    out = np.zeros((n, 3))
    rc = L.cg_pix2vec(nside, SCHEME[scheme.upper()], None if pp is None else pp.ctypes.data_as(_ip), n, _p(out))
    if rc:
        raise CGError(rc, "cg_pix2vec")
    return out


def beam(l, fwhm_deg):
    return library().cg_beam(int(l), float(fwhm_deg))


def _make_config(L, lmax, fwhm_deg, nside, good_pixels, scheme, dirs, beam, noise_sigma, noise_var, max_batch,
                 precision, device, cl_ref, recenter, recenter_radius):
    """A cg_config for these arguments and the arrays its pointers refer to (keep them alive)."""
    cfg = _Config()
    L.cg_config_init(ctypes.byref(cfg))
    keep = []
    if dirs is not None:
        d = _f64(dirs).reshape(-1, 3)
        keep.append(d)
        cfg.dirs = _p(d)
        cfg.n = d.shape[0]
    else:
        cfg.nside = int(nside)
        cfg.scheme = SCHEME[scheme.upper()]
        if good_pixels is not None:
            g = np.ascontiguousarray(good_pixels, dtype=np.int32)
            keep.append(g)
            cfg.good_pixels = g.ctypes.data_as(_ip)
            cfg.n = len(g)
    cfg.lmax = int(lmax)
    cfg.fwhm_deg = float(fwhm_deg)
    if beam is not None:
        b = _f64(beam)
        keep.append(b)
        cfg.beam = _p(b)
    cfg.noise_sigma = float(noise_sigma)
    if noise_var is not None:
        nv = _f64(noise_var)
        keep.append(nv)
        cfg.noise_var = _p(nv)
    cfg.max_batch = int(max_batch)
    cfg.precision = PRECISION[precision]
    cfg.device = int(device)
    if cl_ref is not None:
        cr = _f64(cl_ref)
        keep.append(cr)
        cfg.cl_ref = _p(cr)
    cfg.recenter = RECENTER[recenter]
    cfg.recenter_radius = float(recenter_radius)
    return cfg, keep


class _MemPlan(ctypes.Structure):
    _fields_ = [("bytes_fixed", ctypes.c_size_t), ("bytes_per_element", ctypes.c_size_t),
                ("bytes_budget", ctypes.c_size_t), ("bytes_reserve", ctypes.c_size_t),
                ("max_batch_fit", ctypes.c_int), ("chunk", ctypes.c_int)]


def _plan_dict(p):
    return {k: getattr(p, k) for k, _ in _MemPlan._fields_}


def plan_memory(budget_bytes=0, lmax=2, fwhm_deg=1.0, nside=None, good_pixels=None, scheme="NEST", dirs=None,
                beam=None, noise_sigma=1e-3, noise_var=None, max_batch=1, precision="fp64", device=0, cl_ref=None,
                recenter="auto", recenter_radius=1.0):
    """Memory admission of a context with these arguments, before creating it (cg_plan_memory):
    dict(bytes_fixed, bytes_per_element, bytes_budget, bytes_reserve, max_batch_fit, chunk).
    budget_bytes = 0 plans against the device's free memory, otherwise needs no device."""
    L = library()
    cfg, keep = _make_config(L, lmax, fwhm_deg, nside, good_pixels, scheme, dirs, beam, noise_sigma, noise_var,
                             max_batch, precision, device, cl_ref, recenter, recenter_radius)
    p = _MemPlan()
    rc = L.cg_plan_memory(ctypes.byref(cfg), ctypes.c_size_t(int(budget_bytes)), ctypes.byref(p))
    if rc:
        raise CGError(rc, L.cg_last_error(None).decode())
    return _plan_dict(p)


# ---- context ------------------------------------------------------------------

class Context:
    """One GPU context for a fixed pixel set, l range, beam and noise.

    precision="fp64": the plain FP64 path (bit-identical covariance, FP64
    Cholesky).  precision="mixed": the batched mixed path (FP64 reference
    factorisation, FP32 whitened factors, FP64 log-det and refinement).
    """

    def __init__(self, lmax, fwhm_deg, nside=None, good_pixels=None, scheme="NEST", dirs=None, beam=None,
                 noise_sigma=1e-3, noise_var=None, max_batch=1, precision="fp64", device=0, cl_ref=None,
                 recenter="auto", recenter_radius=1.0):
        L = library()
        cfg, keep = _make_config(L, lmax, fwhm_deg, nside, good_pixels, scheme, dirs, beam, noise_sigma, noise_var,
                                 max_batch, precision, device, cl_ref, recenter, recenter_radius)
        h = ctypes.c_void_p()
        rc = L.cg_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc:
            raise CGError(rc, L.cg_last_error(None).decode())
        self._h = h
        self._L = L
        self.lmax = int(lmax)
        self.n = L.cg_get_n(h)
        self.max_batch = int(max_batch)
        self.precision = precision

    def memory_plan(self):
        """The memory admission this context was created under (cg_get_memory_plan)."""
        p = _MemPlan()
        self._check(self._L.cg_get_memory_plan(self._h, ctypes.byref(p)))
        return _plan_dict(p)

    def close(self):
        if getattr(self, "_h", None):
            self._L.cg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            raise CGError(rc, self._L.cg_last_error(self._h).decode())

    @property
    def handle(self):
        return self._h

    def unit_vectors(self):
        out = np.zeros((self.n, 3))
        self._check(self._L.cg_unit_vectors(self._h, _p(out)))
        return out

    def build_cmatrix(self, cl):
        """Packed C (i <= j at j(j+1)/2 + i) for one C_l vector or a batch [B, lmax+1]."""
        cl = _f64(cl)
        single = cl.ndim == 1
        cl2 = cl.reshape(-1, self.lmax + 1)
        B = cl2.shape[0]
        out = np.zeros((B, self.n * (self.n + 1) // 2))
        self._check(self._L.cg_build_cmatrix_batched(self._h, B, _p(cl2), _p(out)))
        return out[0] if single else out

    def fiducial_matrix(self, cl, lmax_max, lmax=None, beam=None):
        """CMatrixGenerator::getFiducialMatrix for this context's pixels: packed sum over
        l = lmax+1 .. lmax_max (the reference uses lmax_max = 4 nside) plus the monopole/dipole
        term.  lmax defaults to the context's; cl [>= lmax_max + 1]; beam [lmax_max + 1] or None
        for the context's Gaussian beam (cg_fiducial_matrix)."""
        cl = _f64(cl)
        if cl.shape[0] < lmax_max + 1:
            raise ValueError("cl must have lmax_max + 1 entries")
        out = np.zeros(self.n * (self.n + 1) // 2)
        b = None if beam is None else _f64(beam)
        self._check(self._L.cg_fiducial_matrix(self._h, _p(cl), int(self.lmax if lmax is None else lmax),
                                               int(lmax_max), _p(b), _p(out)))
        return out

    def loglike(self, cl, d, grad=False):
        """-2lnL for a batch of C_l vectors on one map d [n] or B maps [B, n].

        Returns dict(m2lnl, chi2, logdet (raw ln det C), grad (d(-2lnL)/dC_l), status)."""
        cl = _f64(cl)
        single = cl.ndim == 1
        cl2 = cl.reshape(-1, self.lmax + 1)
        B = cl2.shape[0]
        d = _f64(d)
        stride = 0 if d.ndim == 1 else d.shape[1]
        m2 = np.zeros(B)
        chi2 = np.zeros(B)
        ld = np.zeros(B)
        st = np.zeros(B, dtype=np.int32)
        g = np.zeros((B, self.lmax + 1)) if grad else None
        self._check(self._L.cg_loglike(self._h, B, _p(cl2), _p(d), stride, _p(m2), _p(chi2), _p(ld), _p(g),
                                       st.ctypes.data_as(_ip)))
        out = dict(m2lnl=m2, chi2=chi2, logdet=ld, grad=g, status=st)
        if single:
            out = {k: (v[0] if v is not None else None) for k, v in out.items()}
        return out

    def loglike_device(self, B, cl_ptr, d_ptr, d_stride, m2lnl_ptr, chi2_ptr=None, logdet_ptr=None,
                       grad_ptr=None, status_ptr=None, stream=0):
        """Asynchronous device-pointer entry point (raw CUDA addresses, e.g. torch .data_ptr())."""
        self._check(self._L.cg_loglike_device(self._h, int(B), cl_ptr, d_ptr, int(d_stride), m2lnl_ptr, chi2_ptr,
                                              logdet_ptr, grad_ptr, status_ptr, stream))

    def set_reference(self, cl_ref):
        self._check(self._L.cg_set_reference(self._h, _p(_f64(cl_ref))))

    def reference_count(self):
        return self._L.cg_reference_count(self._h)

    def hmc(self, d, x0, cl_template, niter, nleap, tau, mass=None, jitter=False, seed=0):
        """Batched HMC over ln C_l (l = 2..lmax), one chain per row of x0 (cg_hmc_run).
        Returns (chain [niter+1, nchains, lmax]: -2lnL then x, accept_rate [nchains])."""
        x0 = _f64(x0)
        nchains, npar = x0.shape
        chain = np.zeros((niter + 1, nchains, npar + 1))
        acc = np.zeros(nchains)
        m = None if mass is None else _f64(mass)
        self._check(self._L.cg_hmc_run(self._h, _p(_f64(d)), nchains, _p(x0), _p(_f64(cl_template)), int(niter),
                                       int(nleap), float(tau), _p(m), int(bool(jitter)), int(seed), _p(chain),
                                       _p(acc)))
        return chain, acc

    def legendre_table(self, lmax, l0=0):
        """LegendrePolynomialContainer's table for this context's pixels (cg_legendre_table):
        [lmax + 1 - l0, n(n+1)/2] with P_l(n_i . n_j) at j(j+1)/2 + i."""
        n = self.n
        out = np.zeros((lmax + 1 - l0, n * (n + 1) // 2))
        self._check(self._L.cg_legendre_table(self._h, int(l0), int(lmax) + 1, _p(out)))
        return out

    def noise_matrix_from_sims(self, sims):
        """Averaging step of CMatrixGenerator::calculateNoiseMatrix
        (source/c_matrix_generator.cpp:887-910) on the device: sims [nsims, n] simulated
        noise maps at the kept pixels -> (packed noise matrix, max |per-pixel mean|)."""
        sims = _f64(sims)
        ns, n = sims.shape
        out = np.zeros(n * (n + 1) // 2)
        mx = ctypes.c_double(0)
        self._check(self._L.cg_noise_matrix_from_sims(self._h, ns, n, _p(sims), _p(out), ctypes.byref(mx)))
        return out, mx.value

    def mh(self, d, x0, cl_template, niter, sampling_width, priors=None, blocks=None, adapt=True, seed=0):
        """Batched Metropolis-Hastings over ln C_l (l = 2..lmax), one chain per row of x0
        (cg_mh_run).  Returns (chain [niter+1, nchains, lmax]: -2lnL then x,
        accept_rate [nchains, nblocks], final adaptive proposal covariance [lmax-1, lmax-1])."""
        x0 = _f64(x0)
        nchains, npar = x0.shape
        out = _mh_buffers(niter, nchains, npar, blocks)
        _keep, args = _mh_args(npar, sampling_width, priors, blocks, adapt, seed, out)
        self._check(self._L.cg_mh_run(self._h, _p(_f64(d)), nchains, _p(x0), _p(_f64(cl_template)), int(niter),
                                      *args))
        return out[0], out[1], out[2]

    def selftest_wait_timeout(self):
        """Status a bounded device wait reports when it gives up (CG_ERR_TIMEOUT expected)."""
        st = ctypes.c_int(-1)
        self._check(self._L.cg_selftest_wait_timeout(self._h, ctypes.byref(st)))
        return st.value

    TUNE_KNOBS = ("fwd", "fwd_ctas", "chol_ctas", "panel_ctas", "adj", "diag_sq", "table_bf16", "graph", "lauum", "trtri", "hmc_device", "overlap")
    ACCURACY_KNOBS = ("fwd", "diag_sq", "table_bf16")   # never changed by autotune

    def tune_set(self, knob, value):
        self._check(self._L.cg_tune_set(self._h, knob.encode(), int(value)))

    def tune_get(self, knob):
        v = ctypes.c_int(0)
        self._check(self._L.cg_tune_get(self._h, knob.encode(), ctypes.byref(v)))
        return v.value

    def tuning(self):
        """The launch-shape knobs in effect, as a dict (cg_tune_describe)."""
        buf = ctypes.create_string_buffer(512)
        self._check(self._L.cg_tune_describe(self._h, buf, 512))
        return {k: int(v) for k, v in (t.split("=") for t in buf.value.decode().split())}

    def autotune(self, B=None, path=None):
        """Coordinate search over the launch-shape knobs at batch B (default max_batch), applied
        and appended to the tuning file `path` if given (cg_autotune).  Returns the chosen
        shape's median ms per call."""
        ms = ctypes.c_double(0)
        self._check(self._L.cg_autotune(self._h, int(B or self.max_batch),
                                        None if path is None else str(path).encode(), ctypes.byref(ms)))
        return ms.value

    def tune_load(self, path):
        """Apply a tuning file's entry for this shape; True if one was found (cg_tune_load)."""
        f = ctypes.c_int(0)
        self._check(self._L.cg_tune_load(self._h, str(path).encode(), ctypes.byref(f)))
        return bool(f.value)

    def probe_fp32_rate(self, iters=1 << 14, reps=5):
        """FP32 rate (TFLOP/s) of packed two-lane FMAs, and the mean launch time (cg_probe_fp32_rate)."""
        tf, ms = ctypes.c_double(0), ctypes.c_double(0)
        self._check(self._L.cg_probe_fp32_rate(self._h, int(iters), int(reps), ctypes.byref(tf), ctypes.byref(ms)))
        return tf.value, ms.value

    def probe_tf32_rate(self, iters=1 << 16, reps=5):
        """TF32 tensor-core rate (TFLOP/s) of the MMA form the factorisation kernels issue, and
        the mean launch time (ms) (cg_probe_tf32_rate)."""
        tf, ms = ctypes.c_double(0), ctypes.c_double(0)
        self._check(self._L.cg_probe_tf32_rate(self._h, int(iters), int(reps), ctypes.byref(tf), ctypes.byref(ms)))
        return tf.value, ms.value

    def graph_replays(self):
        """Mixed calls replayed from a captured CUDA graph so far (cg_graph_replays)."""
        return int(self._L.cg_graph_replays(self._h))

    def launch_count(self):
        """Kernels this context has launched so far."""
        return int(self._L.cg_launch_count(self._h))

    def set_profiling(self, enable=True):
        self._check(self._L.cg_set_profiling(self._h, int(bool(enable))))

    STAGES = ("build", "cholesky", "trtri", "lauum", "solve", "adjoint", "end")

    def stage_times(self):
        """Per-stage device ms of the last profiled call (syncs on its last event)."""
        ms = np.zeros(7)
        self._check(self._L.cg_stage_times(self._h, _p(ms)))
        return dict(zip(self.STAGES, ms))


def _mh_buffers(niter, nchains, npar, blocks):
    nb = npar if blocks is None else len(blocks)
    return (np.zeros((niter + 1, nchains, npar + 1)), np.zeros((nchains, nb)), np.zeros((npar, npar)))


def _mh_args(npar, sampling_width, priors, blocks, adapt, seed, out):
    """priors: None (flat) or a list of (kind, p1, p2) per parameter, kind "uniform"
    (p1 = min, p2 = max) or "gauss" (p1 = mean, p2 = sigma)."""
    w = _f64(np.broadcast_to(np.asarray(sampling_width, dtype=np.float64), (npar,)))
    mode = p1 = p2 = None
    if priors is not None:
        if len(priors) != npar:
            raise ValueError("one prior per parameter")
        mode = np.array([PRIOR[k] for k, _, _ in priors], dtype=np.int32)
        p1 = _f64([a for _, a, _ in priors])
        p2 = _f64([b for _, _, b in priors])
    blk = None if blocks is None else np.ascontiguousarray(blocks, dtype=np.int32)
    keep = (w, mode, p1, p2, blk)  # the caller holds these while the call runs
    return keep, [_p(w), None if mode is None else mode.ctypes.data_as(_ip), _p(p1), _p(p2),
            0 if blk is None else len(blk), None if blk is None else blk.ctypes.data_as(_ip), int(bool(adapt)),
            int(seed), _p(out[0]), _p(out[1]), _p(out[2])]


def mh_sample(like, x0, niter, sampling_width, priors=None, blocks=None, adapt=True, seed=0):
    """Batched Metropolis-Hastings (cg_mh_sample) over a host likelihood:
    ``like(x [nchains, npar]) -> -2lnL [nchains]``, called once per block move for all
    chains.  The rules are MetropolisHastings::run's (source/mcmc.cpp:455-700); no device
    is used.  Returns (chain [niter+1, nchains, npar+1], accept_rate [nchains, nblocks],
    final adaptive proposal covariance [npar, npar])."""
    L = library()
    x0 = _f64(x0)
    nchains, npar = x0.shape
    failure = []

    def _cb(_user, nc, xp, outp):
        try:
            x = np.ctypeslib.as_array(xp, shape=(nc, npar))
            np.ctypeslib.as_array(outp, shape=(nc,))[:] = like(x.copy())
            return 0
        except Exception as e:  # surfaced after the call returns
            failure.append(e)
            return CG_ERR_BAD_ARG

    cb = _BATCH_LIKE(_cb)
    out = _mh_buffers(niter, nchains, npar, blocks)
    _keep, args = _mh_args(npar, sampling_width, priors, blocks, adapt, seed, out)
    rc = L.cg_mh_sample(nchains, npar, cb, None, _p(x0), int(niter), *args)
    if failure:
        raise failure[0]
    if rc:
        raise CGError(rc, "cg_mh_sample")
    return out


def hmc_sample(like_grad, x0, niter, nleap, tau, mass=None, jitter=False, seed=0):
    """Batched HMC (cg_hmc_sample) over a host likelihood with gradient:
    ``like_grad(x [nchains, npar]) -> (-2lnL [nchains], d(-2lnL)/dx [nchains, npar])``, called once
    per leapfrog step for all chains.  Math::HMC::run's rules and random-number order
    (source/hmc.cpp:31-126); no device is used.  Returns (chain [niter+1, nchains, npar+1]:
    -2lnL then x, accept_rate [nchains])."""
    L = library()
    x0 = _f64(x0)
    nchains, npar = x0.shape
    failure = []

    def _cb(_user, nc, xp, outp, gp):
        try:
            x = np.ctypeslib.as_array(xp, shape=(nc, npar))
            m2, g = like_grad(x.copy())
            np.ctypeslib.as_array(outp, shape=(nc,))[:] = m2
            np.ctypeslib.as_array(gp, shape=(nc, npar))[:] = g
            return 0
        except Exception as e:  # surfaced after the call returns
            failure.append(e)
            return CG_ERR_BAD_ARG

    cb = _BATCH_LIKE_GRAD(_cb)
    chain = np.zeros((niter + 1, nchains, npar + 1))
    acc = np.zeros(nchains)
    m = None if mass is None else _f64(mass)
    rc = L.cg_hmc_sample(nchains, npar, cb, None, _p(x0), int(niter), int(nleap), float(tau), _p(m),
                         int(bool(jitter)), int(seed), _p(chain), _p(acc))
    if failure:
        raise failure[0]
    if rc:
        raise CGError(rc, "cg_hmc_sample")
    return chain, acc


class LegendrePolynomialContainer:
    """The reference's LegendrePolynomialContainer (include/c_matrix_generator.hpp:10-36):
    ``LegendrePolynomialContainer(lmax, nside, good_pixels)`` builds P_l(n_i . n_j) on the GPU
    (NEST pixel indices, None = all); ``LegendrePolynomialContainer(file_name=...)`` reads the
    reference's binary file (int lMax, int nPix, then the packed table of every l)."""

    def __init__(self, lmax=None, nside=None, good_pixels=None, file_name=None, device=0):
        if file_name is not None:
            raw = open(file_name, "rb").read()
            if len(raw) < 8:
                raise CGError(CG_ERR_BAD_ARG, "truncated Legendre table in %s" % file_name)
            lm, npix = (int(v) for v in np.frombuffer(raw[:8], dtype=np.int32))
            if lm < 0 or npix < 0:
                raise CGError(CG_ERR_BAD_ARG, "invalid header in %s" % file_name)
            np_ = npix * (npix + 1) // 2
            if len(raw) < 8 + 8 * (lm + 1) * np_:
                raise CGError(CG_ERR_BAD_ARG, "truncated Legendre table in %s" % file_name)
            data = np.frombuffer(raw[8:8 + 8 * (lm + 1) * np_], dtype=np.float64)
            self.lmax, self.npix, self.table = lm, npix, data.reshape(lm + 1, np_).copy()
            return
        with Context(lmax=max(2, int(lmax)), fwhm_deg=1.0, nside=nside, good_pixels=good_pixels, scheme="NEST",
                     max_batch=1, precision="fp64", device=device) as ctx:
            self.lmax, self.npix, self.table = int(lmax), ctx.n, ctx.legendre_table(int(lmax))

    def value(self, l, j, i):
        """P_l(n_i . n_j), i <= j (source/c_matrix_generator.cpp:78-87)."""
        return float(self.table[l, j * (j + 1) // 2 + i])

    def write_into_file(self, file_name):
        """The reference's file format (source/c_matrix_generator.cpp:136-162)."""
        with open(file_name, "wb") as f:
            f.write(np.array([self.lmax, self.npix], dtype=np.int32).tobytes())
            f.write(np.ascontiguousarray(self.table, dtype=np.float64).tobytes())


class Likelihood:
    """Drop-in for the reference's Likelihood (source/likelihood.cpp:38-41,69-180):
    constructed from packed C, fiducial and noise matrices plus an optional
    foreground map; ``calculate(t)`` returns (like, chi2, logdet) with the
    reference's detOffset applied exactly as the reference does."""

    def __init__(self, c_packed, fid_packed, noise_packed, good_pixels=None, foreground=None, device=0):
        L = library()
        c = _f64(c_packed)
        n = int(round((np.sqrt(8 * len(c) + 1) - 1) / 2))
        if good_pixels is not None and len(good_pixels) != n:
            raise CGError(CG_ERR_BAD_ARG, "There are %d unmasked pixels, however the covariance matrix corresponds "
                                          "to %d." % (len(good_pixels), n))
        f = None if fid_packed is None else _f64(fid_packed)
        nz = _f64(noise_packed)
        for m in (f, nz):
            if m is not None and len(m) != len(c):
                raise CGError(CG_ERR_BAD_ARG, "matrix sizes differ")
        fg = None if foreground is None or len(foreground) == 0 else _f64(foreground)
        h = ctypes.c_void_p()
        rc = L.cg_likelihood_create(ctypes.byref(h), n, _p(c), _p(f), _p(nz), _p(fg), int(device))
        if rc:
            raise CGError(rc, L.cg_likelihood_last_error(None).decode())
        self._h, self._L, self.n = h, L, n
        self.logdet_raw = L.cg_likelihood_logdet(h)

    def calculate(self, t):
        chi2 = ctypes.c_double()
        ld = ctypes.c_double()
        t = _f64(t)
        rc = self._L.cg_likelihood_calculate(self._h, _p(t), ctypes.byref(chi2), ctypes.byref(ld))
        if rc:
            raise CGError(rc, self._L.cg_likelihood_last_error(self._h).decode())
        logdet = ld.value - (-DET_OFFSET)  # logDet_ -= detOffset (source/likelihood.cpp:127-128)
        return chi2.value + logdet, chi2.value, logdet

    def close(self):
        if getattr(self, "_h", None):
            self._L.cg_likelihood_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LikelihoodPolarization:
    """The pixel-space part of the reference's LikelihoodPolarization
    (source/likelihood.cpp:341-401,536-612): ``c_packed`` is the packed Q-then-U covariance of
    all 2 npix pixels, ``ninv`` the dense (2 npix)^2 inverse noise matrix (the contents of the
    reference's n_inv.txt), ``good_pixels`` the kept pixels.  ``calculate(v, subtract)`` takes
    v = N^-1 (Q, U) at the kept pixels and the T-correlated Q, U template at the kept pixels
    (which the reference forms from the TT a_lm by alm2map_pol) and returns (like, chi2, logdet)
    with the reference's detOffset applied."""

    def __init__(self, c_packed, npix, good_pixels, ninv, device=0):
        L = library()
        c = _f64(c_packed)
        size = 2 * int(npix)
        if len(c) != size * (size + 1) // 2:
            raise CGError(CG_ERR_BAD_ARG, "polarization c matrix includes q and u parts: %d pixels expected" % size)
        nv = _f64(ninv)
        if nv.size != size * size:
            raise CGError(CG_ERR_BAD_ARG, "the inverse noise matrix must be %d x %d" % (size, size))
        good = np.ascontiguousarray(good_pixels, dtype=np.int32)
        h = ctypes.c_void_p()
        rc = L.cg_likelihood_pol_create(ctypes.byref(h), int(npix), good.ctypes.data_as(_ip), len(good), _p(c),
                                        _p(nv), int(device))
        if rc:
            raise CGError(rc, L.cg_likelihood_last_error(None).decode())
        self._h, self._L, self.n = h, L, 2 * len(good)
        self.logdet_raw = L.cg_likelihood_logdet(h)

    def calculate(self, v, subtract):
        chi2 = ctypes.c_double()
        ld = ctypes.c_double()
        v, sub = _f64(v), _f64(subtract)
        if len(v) != self.n or len(sub) != self.n:
            raise CGError(CG_ERR_BAD_ARG, "v and subtract need 2 x (kept pixels) = %d values" % self.n)
        rc = self._L.cg_likelihood_pol_calculate(self._h, _p(v), _p(sub), ctypes.byref(chi2), ctypes.byref(ld))
        if rc:
            raise CGError(rc, self._L.cg_likelihood_last_error(self._h).decode())
        logdet = ld.value - DET_OFFSET_POL
        return chi2.value + logdet, chi2.value, logdet

    def close(self):
        if getattr(self, "_h", None):
            self._L.cg_likelihood_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LikelihoodWithDerivs:
    """The Math::LikelihoodWithDerivs interface (include/likelihood_function.hpp:30-47)
    over one data map: parameters are C_l for l = lmin..lmax (or ln C_l with
    log_params=True); ``calculate`` returns -2lnL and ``calculateDeriv(x, i)``
    the derivative of -2lnL w.r.t. parameter i, from one cached gradient per x
    (the reference's HMC asks for the n_par components one by one,
    source/hmc.cpp:158-163)."""

    def __init__(self, ctx, d, cl_template, lmin=2, log_params=True):
        self.ctx = ctx
        self.d = _f64(d)
        self.template = _f64(cl_template).copy()
        self.lmin = lmin
        self.log = log_params
        self._x = None
        self._val = None
        self._grad = None

    def _cl(self, x):
        cl = self.template.copy()
        x = np.asarray(x, dtype=np.float64)
        cl[self.lmin:self.lmin + len(x)] = np.exp(x) if self.log else x
        return cl

    def _eval(self, x):
        x = np.array(x, dtype=np.float64)
        if self._x is not None and np.array_equal(x, self._x):
            return
        cl = self._cl(x)
        r = self.ctx.loglike(cl, self.d, grad=True)
        if r["status"] != 0:
            raise CGError(int(r["status"]), "likelihood evaluation failed")
        g = r["grad"][self.lmin:self.lmin + len(x)]
        if self.log:
            g = g * cl[self.lmin:self.lmin + len(x)]
        self._x, self._val, self._grad = x, r["m2lnl"], g

    def calculate(self, params, nParams=None):
        self._eval(params)
        return self._val

    def calculateDeriv(self, params, nParams, i):
        self._eval(params)
        return self._grad[i]
