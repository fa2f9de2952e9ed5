"""Generate the golden fixtures in this folder from the reference's own code.

Runs here, where the reference sources exist: ``make -C oracle/ref`` compiles
the reference's unmodified translation units into oracle/_ref/libcg_ref.so
(project-written HEALPix / cfitsio / LAPACK shims), and this script calls
them through ctypes.  Every number stored below comes from the reference:

* Legendre and symmetric-matrix known-answer subtests (source/test_legendre.cpp,
  source/test_matrix.cpp), as (result, expected) pairs;
* clToCMatrix covariance matrices (full packed for small cases, SHA-256 plus
  samples for larger ones);
* Likelihood(C, 0, N, goodPixels).calculate(d) chi2 / logDet / -2lnL for the
  fiducial and a few lognormal-perturbed C_l vectors;
* central finite differences (step 1e-4 C_l) of the reference's -2lnL, which
  pin the adjoint gradient the reference does not have.
* getFiducialMatrix (l = lmax+1 .. 4 nside plus the monopole/dipole term) and
  the full low-l flow Likelihood(C, fiducial, N, goodPixels).calculate(d) of
  source/test_like_low.cpp:181-193 that uses it;
* a LegendrePolynomialContainer table file written by the reference's own
  writeIntoFile, and the clToCMatrix covariance computed from that file read
  back by the reference's file constructor;
* CMatrix binary and text files written by the reference's CMatrix, and what
  its Utils::readClFromFile reads from two C_l text files.

* the FP64 noise floor at nside 16: for 100 lognormal C_l vectors (the plain
  FP64 workload), the reference's Likelihood chi2 / logDet from its strict
  build, the same for the first 10 from its -ffast-math build and from the
  oracle's restated LAPACK loops, and an extended-precision (long double)
  evaluation of the same FP64 covariance, the yardstick all of them are
  measured against.

* Math::HMC's chain on an analytic Gaussian (the reference's sampler, driven by
  the reference's own code), with every leapfrog position at full precision;
* LikelihoodPolarization's chi2 and logDet for random Q/U inputs with a zero TT
  template (the shim maps zero harmonic coefficients to zero maps only);
* calculateNoiseMatrix's noise matrix and the 1000 simulated maps it averaged
  (the shim passes each map through the harmonic round trip unchanged, at one
  resolution and beam, and records it).

Usage:  python tests/golden/make_golden.py [part ...]   (parts: main, fiducial,
legendre, files, config2, hmc, pol, noise; default all)
"""
import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from cosmopp_gb300 import workload as W  # noqa: E402

dp = ctypes.POINTER(ctypes.c_double)
ip = ctypes.POINTER(ctypes.c_int)
DET_OFFSET = 29677.0566  # source/likelihood.cpp:127-128 (logDet -= -29677.0566)

CASES = [
    # name, nside, lmax, fwhm_arcmin, keep, sigma, n_perturbed, fd_ells, store_full_c
    ("nside1", 1, 4, 440.0, 1.0, 1.0, 2, "all", True),
    ("nside2", 2, 8, 440.0, 0.8, 1.0, 2, "all", True),
    ("nside4", 4, 16, 440.0, 0.8, 1.0, 2, "all", True),
    ("nside8_lmax24", 8, 24, 440.0, 0.8, 1.0, 3, [2, 3, 10, 17, 24], False),
    ("nside16_lmax47", 16, 47, 220.0, 0.8, 1.0, 2, [2, 30, 47], False),
]


FID_CASES = [
    # name, nside, lmax, fwhm_arcmin, keep, sigma, store_full
    ("fid_nside4", 4, 10, 440.0, 0.8, 1.0, True),
    ("fid_nside8", 8, 24, 440.0, 0.8, 1.0, False),
]


def ref_fiducial(R, cl, nside, lmax, fwhm, nest):
    n = len(nest)
    out = np.zeros(n * (n + 1) // 2)
    rc = R.ref_fiducial_matrix(cl.ctypes.data_as(dp), len(cl), nside, lmax, fwhm, nest.ctypes.data_as(ip), n,
                               out.ctypes.data_as(dp))
    assert rc == 0, R.ref_last_error()
    return out


def ref_like_packed(R, c, fid, noise, d):
    chi2, ld, lk = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = R.ref_likelihood_packed(c.ctypes.data_as(dp), fid.ctypes.data_as(dp), noise.ctypes.data_as(dp), len(d),
                                 d.ctypes.data_as(dp), None, ctypes.byref(chi2), ctypes.byref(ld), ctypes.byref(lk))
    assert rc == 0, R.ref_last_error()
    return chi2.value, ld.value, lk.value


def fiducial_cases(R):
    for name, nside, lmax, fwhm_am, keep, sigma, store_full in FID_CASES:
        fwhm = fwhm_am / 60.0
        ring = W.bernoulli_mask(nside, keep, 1234)
        nest = O.ring2nest(nside, ring)
        n = len(nest)
        lmax_max = 4 * nside
        cl_full = W.fiducial_cl(lmax_max)
        fid = ref_fiducial(R, cl_full, nside, lmax, fwhm, nest)
        c = ref_cmatrix(R, cl_full[:lmax + 1].copy(), nside, fwhm, nest)
        noise = np.zeros_like(c)
        noise[[j * (j + 1) // 2 + j for j in range(n)]] = sigma ** 2
        z = np.random.default_rng(0).standard_normal(n)
        full = W.packed_to_full(c + fid, n) + sigma ** 2 * np.eye(n)
        d = W.draw_data(full, z)
        chi2, ld, lk = ref_like_packed(R, c, fid, noise, d)
        out = dict(nside=nside, lmax=lmax, lmax_max=lmax_max, fwhm_deg=fwhm, sigma=sigma, ring_kept=ring,
                   nest_good=nest, cl_full=cl_full, d=d, chi2=chi2, logdet_ref=ld, like_ref=lk,
                   fid_sha256=np.array(hashlib.sha256(fid.tobytes()).hexdigest()),
                   fid_diag=np.array([fid[j * (j + 1) // 2 + j] for j in range(n)]), fid_head=fid[:4096].copy(),
                   c_sha256=np.array(hashlib.sha256(c.tobytes()).hexdigest()))
        if store_full:
            out["fid_packed"] = fid
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "n", n, "like", lk, "chi2", chi2)


LEGENDRE_CASE = ("legendre_nside2_lmax8", 2, 8, 440.0, 0.8)


def legendre_cases(R):
    name, nside, lmax, fwhm_am, keep = LEGENDRE_CASE
    fwhm = fwhm_am / 60.0
    ring = W.bernoulli_mask(nside, keep, 1234)
    nest = O.ring2nest(nside, ring)
    n = len(nest)
    path = os.path.join(HERE, name + ".bin")
    rc = R.ref_legendre_table_write(lmax, nside, nest.ctypes.data_as(ip), n, path.encode())
    assert rc == 0, R.ref_last_error()
    cl = W.fiducial_cl(lmax)
    c_lp = np.zeros(n * (n + 1) // 2)
    rc = R.ref_cl_to_cmatrix_lp_file(cl.ctypes.data_as(dp), lmax, nside, fwhm, nest.ctypes.data_as(ip), n,
                                     path.encode(), c_lp.ctypes.data_as(dp))
    assert rc == 0, R.ref_last_error()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), nside=nside, lmax=lmax, fwhm_deg=fwhm, ring_kept=ring,
                        nest_good=nest, cl=cl, c_lp=c_lp, c_plain=ref_cmatrix(R, cl, nside, fwhm, nest))
    print(name, "n", n, "bytes", os.path.getsize(path))


def file_cases(R):
    """CMatrix binary and text files written by the reference's CMatrix, and C_l text files
    (plain C_l; l-prefixed D_l) with what the reference's Utils::readClFromFile reads from them."""
    name, nside, lmax, fwhm_am, keep = LEGENDRE_CASE
    fwhm = fwhm_am / 60.0
    ring = W.bernoulli_mask(nside, keep, 1234)
    nest = O.ring2nest(nside, ring)
    n = len(nest)
    cl = W.fiducial_cl(lmax)
    binp, txtp = os.path.join(HERE, "cmatrix_nside2.bin"), os.path.join(HERE, "cmatrix_nside2.txt")
    rc = R.ref_cmatrix_write_files(cl.ctypes.data_as(dp), lmax, nside, fwhm, nest.ctypes.data_as(ip), n,
                                   b"covariance from the reference", binp.encode(), txtp.encode())
    assert rc == 0, R.ref_last_error()
    plain = os.path.join(HERE, "cl_plain.txt")
    with open(plain, "w") as f:
        f.write("".join("%.17g\n" % v for v in cl))
    ells = np.arange(lmax + 1)
    dl = np.where(ells > 0, cl * ells * (ells + 1) / (2 * np.pi), 0.0)
    withl = os.path.join(HERE, "dl_with_l.txt")
    with open(withl, "w") as f:
        f.write("".join("%d %.17g\n" % (l, v) for l, v in zip(ells, dl)))
    out = {}
    for key, path, has_l, is_dl in (("read_plain", plain, 0, 0), ("read_dl", withl, 1, 1)):
        buf = np.zeros(4096)
        k = R.ref_read_cl(path.encode(), has_l, is_dl, buf.ctypes.data_as(dp), len(buf))
        assert k > 0, R.ref_last_error()
        out[key] = buf[:k].copy()
    np.savez_compressed(os.path.join(HERE, "files_nside2.npz"), nest_good=nest, nside=nside, lmax=lmax,
                        fwhm_deg=fwhm, c_packed=ref_cmatrix(R, cl, nside, fwhm, nest), **out)
    print("files_nside2 n", n)


def ref_cmatrix(R, cl, nside, fwhm, nest):
    n = len(nest)
    out = np.zeros(n * (n + 1) // 2)
    rc = R.ref_cl_to_cmatrix(cl.ctypes.data_as(dp), len(cl) - 1, nside, fwhm, nest.ctypes.data_as(ip), n,
                             out.ctypes.data_as(dp))
    assert rc == 0, R.ref_last_error()
    return out


def ref_like(R, cl, nside, fwhm, nest, sigma, d):
    chi2, ld, lk = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = R.ref_likelihood(cl.ctypes.data_as(dp), len(cl) - 1, nside, fwhm, nest.ctypes.data_as(ip), len(nest),
                          sigma, d.ctypes.data_as(dp), ctypes.byref(chi2), ctypes.byref(ld), ctypes.byref(lk))
    assert rc == 0, R.ref_last_error()
    return chi2.value, ld.value, lk.value


def _config2_worker(args):
    """One strict-build reference evaluation in a worker process (the reference's pair loop
    is serial, so the 100 evaluations run side by side)."""
    k, cl, nside, fwhm, nest, sigma, d = args
    R = O.ref()
    return k, ref_like(R, cl, nside, fwhm, nest, sigma, d)


def config2_cases():
    """The plain FP64 workload at nside 16 (100 lognormal C_l vectors) and its noise floor."""
    import multiprocessing as mp
    g = dict(np.load(os.path.join(HERE, "nside16_lmax47.npz")))
    wl = W.make("nside16_lmax47")
    nside, fwhm, sigma = wl.nside, wl.fwhm_deg, wl.sigma
    nest = O.ring2nest(nside, wl.ring_kept)
    assert np.array_equal(nest, g["nest_good"]) and np.array_equal(wl.cl_batch[:2], g["cls"][1:3])
    d = g["d"]
    cls = wl.cl_batch
    os.environ["OMP_NUM_THREADS"] = "2"
    os.environ["OPENBLAS_NUM_THREADS"] = "2"
    with mp.get_context("spawn").Pool(4) as pool:
        rows = dict(pool.map(_config2_worker, [(k, cls[k], nside, fwhm, nest, sigma, d) for k in range(len(cls))]))
    rows = np.array([rows[k] for k in range(len(cls))])
    O.set_threads(os.cpu_count() or 1)
    xyz = O.unit_vectors(nside, nest, "NEST")
    ext = []
    for cl in cls:
        c = O.cl_to_cmatrix(cl, xyz, fwhm)
        chi2, ld, info = O.loglike_extended(c, sigma ** 2, d)
        assert info == 0
        ext.append((chi2, ld))
    ext = np.array(ext)
    nsub = 10
    Rf = O.ref("_fastmath")
    fast = np.array([ref_like(Rf, cls[k], nside, fwhm, nest, sigma, d) for k in range(nsub)])
    restated = np.array([O.evaluate(cls[k], xyz, fwhm, sigma ** 2, d, grad=False)["m2lnl"] for k in range(nsub)])
    m2 = rows[:, 0] + (rows[:, 1] - DET_OFFSET)
    m2_ext = ext[:, 0] + ext[:, 1]
    np.savez_compressed(os.path.join(HERE, "config2_nside16.npz"), nside=nside, lmax=wl.lmax, fwhm_deg=fwhm,
                        sigma=sigma, nest_good=nest, cls=cls, d=d, chi2=rows[:, 0], logdet_raw=rows[:, 1] - DET_OFFSET,
                        m2lnl=m2, chi2_ext=ext[:, 0], logdet_ext=ext[:, 1], m2lnl_ext=m2_ext,
                        m2lnl_fastmath=fast[:, 0] + (fast[:, 1] - DET_OFFSET), m2lnl_restated=restated)
    print("config2 nside16: %d vectors; |reference - extended| max %.3e; |fastmath - extended| max %.3e; "
          "|restated - extended| max %.3e" % (len(cls), np.abs(m2 - m2_ext).max(),
                                              np.abs(fast[:, 0] + fast[:, 1] - DET_OFFSET - m2_ext[:nsub]).max(),
                                              np.abs(restated - m2_ext[:nsub]).max()))


def hmc_cases():
    """Math::HMC::run (source/hmc.cpp:31-126), the reference's own code, on an analytic Gaussian:
    the leapfrog positions at full precision and the chain file it writes (6 significant digits)."""
    import tempfile
    R = O.ref()
    dp_ = ctypes.POINTER(ctypes.c_double)
    R.ref_hmc_gaussian.argtypes = [ctypes.c_int, dp_, dp_, dp_, ctypes.c_double, ctypes.c_int, ctypes.c_uint,
                                   ctypes.c_int, ctypes.c_char_p, dp_, ctypes.c_int]
    n = 5
    mu = np.array([0.3, -1.0, 2.0, 0.0, 0.5])
    sig = np.array([1.0, 0.5, 2.0, 0.3, 1.5])
    start = mu + np.array([0.5, -0.2, 1.0, 0.1, -0.7])
    out = {}
    for tag, tau, nmax, seed, iters in (("a", 0.3, 10, 12345, 50), ("b", 0.58, 12, 777, 60)):
        pts = np.zeros((20000, n))
        root = os.path.join(tempfile.mkdtemp(), "hmc")
        cnt = R.ref_hmc_gaussian(n, mu.ctypes.data_as(dp_), sig.ctypes.data_as(dp_), start.ctypes.data_as(dp_), tau,
                                 nmax, seed, iters, root.encode(), pts.ctypes.data_as(dp_), len(pts))
        assert 0 < cnt <= len(pts), R.ref_last_error()
        ch = np.loadtxt(root + ".txt")
        out.update({tag + "_tau": tau, tag + "_nmax": nmax, tag + "_seed": seed, tag + "_iters": iters,
                    tag + "_points": pts[:cnt].copy(), tag + "_chain_file": ch})
        acc = np.mean(np.any(np.diff(ch[:, 2:], axis=0) != 0, axis=1))
        print("hmc %s: %d leapfrog points, acceptance %.2f" % (tag, cnt, acc))
    np.savez_compressed(os.path.join(HERE, "hmc_gaussian_reference.npz"), mu=mu, sig=sig, start=start, **out)


def pol_case_inputs(seed, npix=192, keep=0.8):
    """The Q/U test inputs (tests/test_gpu_pol.py): a random positive-definite (2 npix)-pixel
    covariance, a random positive-definite inverse noise matrix, a Bernoulli mask."""
    rng = np.random.default_rng(seed)
    size = 2 * npix
    a = rng.standard_normal((size, size)) / np.sqrt(size)
    c = a @ a.T + 0.5 * np.eye(size)
    b = rng.standard_normal((size, size)) / np.sqrt(size)
    ninv = b @ b.T + 2.0 * np.eye(size)
    good = np.flatnonzero(rng.uniform(size=npix) < keep).astype(np.int32)
    c_packed = np.concatenate([c[:j + 1, j] for j in range(size)])
    return rng, npix, good, c_packed, ninv


def pol_cases():
    """LikelihoodPolarization's constructor and calculate (source/likelihood.cpp:341-401,536-612), the
    reference's own code, with a zero TT a_lm (zero E-mode template): chi2 and logDet of three maps."""
    import tempfile
    R = O.ref()
    dp_, ip_ = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    R.ref_likelihood_pol.argtypes = [ctypes.c_int, dp_, dp_, ip_, ctypes.c_int, ctypes.c_long, ctypes.c_int, dp_,
                                     ctypes.c_char_p, dp_, dp_]
    rng, npix, good, c_packed, ninv = pol_case_inputs(3)
    ninv = np.ascontiguousarray(ninv)
    vs, chi2s, lds = [], [], []
    for k in range(3):
        v = rng.standard_normal(2 * len(good))
        chi2, ld = ctypes.c_double(), ctypes.c_double()
        rc = R.ref_likelihood_pol(2 * npix, c_packed.ctypes.data_as(dp_), ninv.ctypes.data_as(dp_),
                                  good.ctypes.data_as(ip_), len(good), 4, 4, v.ctypes.data_as(dp_),
                                  tempfile.mkdtemp().encode(), ctypes.byref(chi2), ctypes.byref(ld))
        assert rc == 0, R.ref_last_error()
        vs.append(v)
        chi2s.append(chi2.value)
        lds.append(ld.value)
    digest = hashlib.sha256(c_packed.tobytes() + ninv.tobytes() + good.tobytes()).hexdigest()
    np.savez_compressed(os.path.join(HERE, "pol_nside4_reference.npz"), seed=3, npix=npix, good=good, v=np.array(vs),
                        chi2=np.array(chi2s), logdet_ref=np.array(lds), det_offset=16078.083180,
                        inputs_sha256=np.array(digest))
    print("pol: chi2", chi2s, "logDet", lds)


def noise_cases():
    """CMatrixGenerator::calculateNoiseMatrix (source/c_matrix_generator.cpp:789-929), the reference's
    own code, at nside 2 with equal input and output resolution and beam: the shim's harmonic
    round trip hands each of the 1000 simulated maps on unchanged and records it.  Stores the kept
    pixels, the maps at those pixels (NEST order) and the reference's noise matrix."""
    import tempfile
    R = O.ref()
    dp_ = ctypes.POINTER(ctypes.c_double)
    R.ref_noise_matrix.argtypes = [ctypes.c_long, dp_, dp_, ctypes.c_double, ctypes.c_double, ctypes.c_char_p, dp_,
                                   dp_, ctypes.c_int]
    nside, npix = 2, 48
    rng = np.random.default_rng(4)
    mask = (rng.uniform(size=npix) < 0.8).astype(float)
    nobs = rng.integers(50, 200, npix).astype(float)
    good = np.flatnonzero(mask > 0.5).astype(np.int32)
    ng = len(good)
    out = np.zeros(ng * (ng + 1) // 2)
    sims = np.zeros((1000, npix))
    k = R.ref_noise_matrix(nside, mask.ctypes.data_as(dp_), nobs.ctypes.data_as(dp_), 10.0, 7.0,
                           tempfile.mkdtemp().encode(), out.ctypes.data_as(dp_), sims.ctypes.data_as(dp_), 1000)
    assert k == 1000, R.ref_last_error()
    nest_of_ring = O.ring2nest(nside, np.arange(npix))
    sims_nest = np.zeros_like(sims)
    sims_nest[:, nest_of_ring] = sims
    np.savez_compressed(os.path.join(HERE, "noise_nside2_reference.npz"), nside=nside, good=good,
                        sims=np.ascontiguousarray(sims_nest[:, good]), noise_packed=out)
    print("noise: %d simulations x %d kept pixels" % (k, ng))


def main(parts):
    if not O.ref_available():
        raise SystemExit("build the reference first: make -C oracle/ref")
    R = O.ref()
    R.ref_legendre_table_write.argtypes = [ctypes.c_int, ctypes.c_long, ip, ctypes.c_int, ctypes.c_char_p]
    R.ref_cl_to_cmatrix_lp_file.argtypes = [dp, ctypes.c_int, ctypes.c_long, ctypes.c_double, ip, ctypes.c_int,
                                            ctypes.c_char_p, dp]
    R.ref_cmatrix_write_files.argtypes = [dp, ctypes.c_int, ctypes.c_long, ctypes.c_double, ip, ctypes.c_int,
                                          ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
    R.ref_read_cl.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int]
    if "config2" in parts:
        config2_cases()
    if "hmc" in parts:
        hmc_cases()
    if "pol" in parts:
        pol_cases()
    if "noise" in parts:
        noise_cases()
    if "legendre" in parts:
        legendre_cases(R)
    if "files" in parts:
        file_cases(R)
    if "main" not in parts:
        if "fiducial" in parts:
            fiducial_cases(R)
        return
    os.makedirs(os.path.join(HERE, "_kat", "test_files"), exist_ok=True)
    cwd = os.getcwd()
    os.chdir(os.path.join(HERE, "_kat"))  # the matrix subtests write text files under test_files/
    kat = []
    res, exp = ctypes.c_double(), ctypes.c_double()
    for which, idx in [("legendre", i) for i in range(5)] + [("matrix", 18), ("matrix", 19)]:
        rc = R.ref_run_subtest(which.encode(), idx, ctypes.byref(res), ctypes.byref(exp))
        assert rc == 0
        kat.append((which, idx, res.value, exp.value))
    os.chdir(cwd)
    np.savez(os.path.join(HERE, "kat_reference.npz"),
             which=np.array([k[0] for k in kat]), index=np.array([k[1] for k in kat]),
             result=np.array([k[2] for k in kat]), expected=np.array([k[3] for k in kat]))

    for name, nside, lmax, fwhm_am, keep, sigma, npert, fd_ells, store_full in CASES:
        fwhm = fwhm_am / 60.0
        ring = W.bernoulli_mask(nside, keep, 1234) if keep < 1 else np.arange(12 * nside * nside, dtype=np.int32)
        nest = O.ring2nest(nside, ring)
        n = len(nest)
        cl_fid = W.fiducial_cl(lmax)
        cls = np.vstack([cl_fid, W.lognormal_batch(cl_fid, npert, 7)])
        c_fid = ref_cmatrix(R, cl_fid, nside, fwhm, nest)
        z = np.random.default_rng(0).standard_normal(n)
        full = W.packed_to_full(c_fid, n) + sigma ** 2 * np.eye(n)
        d = W.draw_data(full, z)
        rows = []
        for cl in cls:
            rows.append(ref_like(R, cl, nside, fwhm, nest, sigma, d))
        rows = np.array(rows)
        ells = list(range(2, lmax + 1)) if fd_ells == "all" else list(fd_ells)
        fd = []
        for ell in ells:
            h = 1e-4 * cl_fid[ell]
            cp = cl_fid.copy(); cp[ell] += h
            cm = cl_fid.copy(); cm[ell] -= h
            fd.append((ref_like(R, cp, nside, fwhm, nest, sigma, d)[2] - ref_like(R, cm, nside, fwhm, nest, sigma, d)[2]) / (2 * h))
        out = dict(nside=nside, lmax=lmax, fwhm_deg=fwhm, sigma=sigma, ring_kept=ring, nest_good=nest,
                   cls=cls, d=d, chi2=rows[:, 0], logdet_ref=rows[:, 1], like_ref=rows[:, 2],
                   logdet_raw=rows[:, 1] - DET_OFFSET, m2lnl=rows[:, 0] + (rows[:, 1] - DET_OFFSET),
                   fd_ells=np.array(ells), fd_grad=np.array(fd),
                   c_sha256=np.array(hashlib.sha256(c_fid.tobytes()).hexdigest()),
                   c_diag=np.array([c_fid[j * (j + 1) // 2 + j] for j in range(n)]),
                   c_head=c_fid[:4096].copy())
        if store_full:
            out["c_packed"] = c_fid
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "n", n, "m2lnl", out["m2lnl"][0], "chi2", rows[0, 0])
    if "fiducial" in parts:
        fiducial_cases(R)


if __name__ == "__main__":
    main(set(sys.argv[1:]) or {"main", "fiducial", "legendre", "files", "config2", "hmc", "pol", "noise"})
