"""The pixel-space polarisation likelihood (cg_likelihood_pol_*) against the oracle's FP64
restatement of LikelihoodPolarization's construct and calculate: a random positive-definite
Q/U covariance and inverse noise over a HEALPix nside 4 sky (384 Q+U pixels) with a mask,
several maps and templates; a non-positive-definite matrix is reported."""
import numpy as np
import pytest

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu


def _case(seed, npix=192, keep=0.8):
    rng = np.random.default_rng(seed)
    size = 2 * npix
    a = rng.standard_normal((size, size)) / np.sqrt(size)
    c = a @ a.T + 0.5 * np.eye(size)
    b = rng.standard_normal((size, size)) / np.sqrt(size)
    ninv = b @ b.T + 2.0 * np.eye(size)
    good = np.flatnonzero(rng.uniform(size=npix) < keep).astype(np.int32)
    c_packed = np.concatenate([c[:j + 1, j] for j in range(size)])
    return rng, npix, good, c_packed, ninv


def test_pol_likelihood_matches_oracle(oracle_mod):
    rng, npix, good, c_packed, ninv = _case(3)
    lik = cg.LikelihoodPolarization(c_packed, npix, good, ninv)
    n2 = 2 * len(good)
    for k in range(3):
        v = rng.standard_normal(n2)
        sub = 0.3 * rng.standard_normal(n2) if k else np.zeros(n2)
        like, chi2, logdet = lik.calculate(v, sub)
        chi2_o, ld_o = oracle_mod.likelihood_pol(c_packed, npix, good, ninv, v, sub)
        assert abs(logdet - (ld_o - cg.DET_OFFSET_POL)) <= 1e-9 * max(1.0, abs(ld_o))
        assert abs(chi2 - chi2_o) <= 1e-9 * max(1.0, abs(chi2_o))
        assert abs(like - (chi2 + logdet)) <= 1e-9 * abs(like)
    lik.close()


def test_pol_likelihood_matches_the_reference_itself():
    """Against the reference's own compiled LikelihoodPolarization (fixture from make_golden.py,
    part pol: its constructor fed n_inv.txt, calculate run with a zero TT a_lm, so the E-mode
    template is zero): chi2 and the raw ln det of three maps."""
    from conftest import load_golden
    g = load_golden("pol_nside4_reference")
    _, npix, good, c_packed, ninv = _case(int(g["seed"]))
    ninv = np.ascontiguousarray(ninv)
    # the inputs come from the seeded draws; their products round alike to the last bits on each
    # machine's BLAS only, so the kept pixels (integers) are compared and the values by the bar
    assert np.array_equal(good, g["good"])
    lik = cg.LikelihoodPolarization(c_packed, npix, good, ninv)
    for v, chi2_r, ld_r in zip(g["v"], g["chi2"], g["logdet_ref"]):
        like, chi2, logdet = lik.calculate(v, np.zeros_like(v))
        assert abs(chi2 - chi2_r) <= 1e-9 * max(1.0, abs(chi2_r)), (chi2, chi2_r)
        assert abs(logdet - ld_r) <= 1e-9 * max(1.0, abs(ld_r)), (logdet, ld_r)
    lik.close()


def test_pol_likelihood_rejects_indefinite():
    _, npix, good, c_packed, ninv = _case(5, npix=48)
    with pytest.raises(cg.CGError) as e:
        cg.LikelihoodPolarization(1e-3 * c_packed, npix, good, -ninv)
    assert e.value.code == cg.CG_ERR_NOT_PD
