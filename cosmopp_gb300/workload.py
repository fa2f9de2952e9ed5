"""Seeded synthetic inputs for the pixel-likelihood path.

The reference's own low-l test draws its maps from CLASS spectra and HEALPix
simulations (source/test_like_low.cpp:56-177); here every input is synthetic
and seeded instead:

* pixels: HEALPix centres, Bernoulli(keep) mask drawn per RING index;
* C_l = A 2 pi / (l (l+1)) for l >= 2 (A = 1e3 muK^2), C_0 = C_1 = 0;
* batches: C_l * exp(0.1 N(0,1)) per l and per batch element;
* data: d = L z with L L^T = C_fid + sigma^2 I and z ~ N(0,1) (seed 0); the
  caller supplies L (see ``draw_data``).

Named workloads follow the five configurations the path is measured on.
"""
from dataclasses import dataclass, field

import numpy as np

WORKLOADS = {
    # name: nside, lmax, fwhm_arcmin, keep, sigma, batch
    "nside8_lmax24": dict(nside=8, lmax=24, fwhm_arcmin=440.0, keep=0.8, sigma=1.0, batch=1),
    "nside16_lmax47": dict(nside=16, lmax=47, fwhm_arcmin=220.0, keep=0.8, sigma=1.0, batch=100),
    "nside16_lmax47_b256": dict(nside=16, lmax=47, fwhm_arcmin=220.0, keep=0.8, sigma=1.0, batch=256),
    "nside16_lmax47_hmc64": dict(nside=16, lmax=47, fwhm_arcmin=220.0, keep=0.8, sigma=1.0, batch=64),
    "nside32_lmax95_b32": dict(nside=32, lmax=95, fwhm_arcmin=110.0, keep=0.9, sigma=0.5, batch=32),
}


@dataclass
class Workload:
    name: str
    nside: int
    lmax: int
    fwhm_deg: float
    sigma: float
    ring_kept: np.ndarray            # kept RING indices, ascending
    cl_fid: np.ndarray               # [lmax+1]
    cl_batch: np.ndarray             # [batch, lmax+1]
    z: np.ndarray                    # [n] N(0,1) draw for the data map
    meta: dict = field(default_factory=dict)

    @property
    def n(self):
        return len(self.ring_kept)


def fiducial_cl(lmax, amplitude=1e3):
    cl = np.zeros(lmax + 1)
    ell = np.arange(2, lmax + 1)
    cl[2:] = amplitude * 2.0 * np.pi / (ell * (ell + 1.0))
    return cl


def bernoulli_mask(nside, keep, seed):
    """Kept RING pixel indices (ascending) of a Bernoulli(keep) mask."""
    rng = np.random.default_rng(seed)
    u = rng.random(12 * nside * nside)
    return np.nonzero(u < keep)[0].astype(np.int32)


def lognormal_batch(cl_fid, batch, seed, scale=0.1):
    rng = np.random.default_rng(seed)
    f = np.exp(scale * rng.standard_normal((batch, len(cl_fid))))
    out = cl_fid[None, :] * f
    out[:, :2] = 0.0
    return out


def make(name, batch=None, mask_seed=1234, batch_seed=7, data_seed=0):
    cfg = dict(WORKLOADS[name])
    if batch is not None:
        cfg["batch"] = int(batch)
    ring = bernoulli_mask(cfg["nside"], cfg["keep"], mask_seed)
    cl = fiducial_cl(cfg["lmax"])
    cb = lognormal_batch(cl, cfg["batch"], batch_seed)
    z = np.random.default_rng(data_seed).standard_normal(len(ring))
    return Workload(name=name, nside=cfg["nside"], lmax=cfg["lmax"], fwhm_deg=cfg["fwhm_arcmin"] / 60.0,
                    sigma=cfg["sigma"], ring_kept=ring, cl_fid=cl, cl_batch=cb, z=z, meta=cfg)


def packed_to_full(ap, n):
    """Reference packed storage (i <= j at j(j+1)/2 + i) -> dense symmetric [n, n]."""
    full = np.zeros((n, n))
    # np.tril_indices walks (j, i <= j) in exactly the packed order
    jj, ii = np.tril_indices(n)
    full[ii, jj] = ap
    full[jj, ii] = ap
    return full


def full_to_packed(full):
    jj, ii = np.tril_indices(full.shape[0])
    return np.ascontiguousarray(full[ii, jj])


def draw_data(c_full_with_noise, z):
    """d = L z, L the lower Cholesky factor of the FP64 covariance (input generation only)."""
    L = np.linalg.cholesky(c_full_with_noise)
    return L @ z
