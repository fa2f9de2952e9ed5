"""The noise matrix from simulations (cg_noise_matrix_from_sims) is bit-identical to the
reference's own calculateNoiseMatrix on the 1000 simulations it averaged (fixture
noise_nside2_reference.npz), and to the oracle's restatement of its averaging loop
(source/c_matrix_generator.cpp:887-910) on ragged sizes that leave partial 64-pixel tiles and
partial 16-deep simulation slices, one simulation, and 1000 simulations at the nside 16 pixel
count."""
import numpy as np
import pytest

from conftest import load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    g = load_golden("nside4")
    c = cg.Context(lmax=int(g["lmax"]), fwhm_deg=float(g["fwhm_deg"]), nside=4, good_pixels=g["nest_good"],
                   noise_sigma=float(g["sigma"]), max_batch=1, precision="fp64")
    yield c
    c.close()


@pytest.mark.parametrize("nsims,n", [(1, 1), (1, 70), (17, 63), (33, 129), (200, 147), (1000, 2469)])
def test_noise_matrix_bit_identical(ctx, oracle_mod, nsims, n):
    rng = np.random.default_rng(nsims * 7919 + n)
    sims = rng.standard_normal((nsims, n)) * rng.uniform(0.5, 2.0, n)
    got, mx = ctx.noise_matrix_from_sims(sims)
    want, mx_ref = oracle_mod.noise_matrix(sims)
    assert np.array_equal(got, want)
    assert mx == mx_ref


def test_noise_matrix_rejects_bad_sizes(ctx):
    with pytest.raises(cg.CGError):
        ctx._check(ctx._L.cg_noise_matrix_from_sims(ctx._h, 0, 4, None, None, None))


def test_noise_matrix_bit_identical_to_the_reference_itself(ctx):
    g = load_golden("noise_nside2_reference")
    got, _ = ctx.noise_matrix_from_sims(g["sims"])
    assert np.array_equal(got, g["noise_packed"])
