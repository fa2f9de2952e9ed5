"""The algebra the batched mixed path rests on, checked in FP64 numpy against the oracle (which is
pinned to the reference), with no device:
- the addition theorem: B_l^2 sum_m Y_lm Y_lm^T over real spherical harmonics at the pixels is
  l's term of clToCMatrix, (2l+1)/(4pi) B_l^2 P_l(n_i . n_j);
- whitening by the reference factor, A_b = M_ref C_b M_ref^T = I + sum_l eps_bl Ubar_l with
  Ubar_l = c_ref,l Z_l Z_l^T, Z = M_ref Y B, eps_bl = C_bl / c_ref,l - 1;
- ln det C_b = ln det C_ref + ln det A_b and chi2 = y^T A_b^-1 y with y = M_ref d;
- the gradient tr(V Ubar_l) / c_ref,l - sum_{h in l} (Z_h^T x)^2 with V = A_b^-1, x = V y equals
  the oracle's FP64 adjoint."""
import numpy as np
import pytest

from cosmopp_gb300 import workload as W

special = pytest.importorskip("scipy.special")
if not hasattr(special, "sph_harm_y"):
    pytest.skip("scipy without sph_harm_y", allow_module_level=True)

NSIDE, LMAX, FWHM, SIGMA = 2, 8, 440.0 / 60.0, 1.0


def _real_ylm(xyz, lmax):
    """Real orthonormal spherical harmonics [n, sum_{l=2}^{lmax} (2l+1)], columns l-major."""
    theta = np.arccos(np.clip(xyz[:, 2], -1, 1))
    phi = np.arctan2(xyz[:, 1], xyz[:, 0])
    cols, ells = [], []
    for l in range(2, lmax + 1):
        cols.append(special.sph_harm_y(l, 0, theta, phi).real)
        ells.append(l)
        for m in range(1, l + 1):
            y = special.sph_harm_y(l, m, theta, phi)
            cols += [np.sqrt(2) * y.real, np.sqrt(2) * y.imag]
            ells += [l, l]
    return np.stack(cols, axis=1), np.array(ells)


@pytest.fixture(scope="module")
def setup(oracle_mod):
    O = oracle_mod
    ring = W.bernoulli_mask(NSIDE, 0.8, 1234)
    nest = O.ring2nest(NSIDE, ring)
    xyz = O.unit_vectors(NSIDE, nest, "NEST")
    n = len(nest)
    beam = np.array([O.beam(l, FWHM) for l in range(LMAX + 1)])
    Y, ells = _real_ylm(xyz, LMAX)
    Yb = Y * beam[ells][None, :]
    return O, xyz, n, Yb, ells


def test_addition_theorem_gives_the_covariance_terms(setup):
    O, xyz, n, Yb, ells = setup
    for l in (2, 5, LMAX):
        cl = np.zeros(LMAX + 1)
        cl[l] = 1.0
        want = W.packed_to_full(O.cl_to_cmatrix(cl, xyz, FWHM), n)
        got = Yb[:, ells == l] @ Yb[:, ells == l].T
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_whitened_likelihood_and_gradient_match_the_oracle(setup):
    O, xyz, n, Yb, ells = setup
    cl_ref = W.fiducial_cl(LMAX)
    cref = W.packed_to_full(O.cl_to_cmatrix(cl_ref, xyz, FWHM), n) + SIGMA ** 2 * np.eye(n)
    Lref = np.linalg.cholesky(cref)
    Mref = np.linalg.inv(Lref)
    Z = Mref @ Yb
    d = W.draw_data(cref, np.random.default_rng(0).standard_normal(n))
    y = Mref @ d
    for cl in W.lognormal_batch(cl_ref, 3, 11):
        eps = cl / np.where(cl_ref > 0, cl_ref, 1.0) - 1.0
        A = np.eye(n)
        for l in range(2, LMAX + 1):
            Zl = Z[:, ells == l]
            A += eps[l] * cl_ref[l] * (Zl @ Zl.T)
        cb = W.packed_to_full(O.cl_to_cmatrix(cl, xyz, FWHM), n) + SIGMA ** 2 * np.eye(n)
        assert np.abs(A - Mref @ cb @ Mref.T).max() <= 1e-10
        ref = O.evaluate(cl, xyz, FWHM, SIGMA ** 2, d, grad=True)
        logdet = 2 * np.log(np.diag(Lref)).sum() + np.linalg.slogdet(A)[1]
        V = np.linalg.inv(A)
        x = V @ y
        assert abs(logdet - ref["logdet"]) <= 1e-9 * abs(ref["logdet"])
        assert abs(y @ x - ref["chi2"]) <= 1e-9 * abs(ref["chi2"])
        proj = Z.T @ x
        for l in range(2, LMAX + 1):
            Zl = Z[:, ells == l]
            g = np.trace(V @ (cl_ref[l] * Zl @ Zl.T)) / cl_ref[l] - (proj[ells == l] ** 2).sum()
            assert abs(g - ref["grad"][l]) <= 1e-8 * np.abs(ref["grad"][2:]).max()
