"""LegendrePolynomialContainer's table on the GPU (cg_legendre_table) is bit-identical to the
table the reference itself wrote (tests/golden/legendre_nside2_lmax8.bin) and to the oracle
on a larger pixel set, for a full l range and for a sub-range."""
import os

import numpy as np
import pytest

from conftest import ROOT, load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu

REF_FILE = os.path.join(ROOT, "tests", "golden", "legendre_nside2_lmax8.bin")


def test_table_matches_reference_file(tmp_path):
    g = load_golden("legendre_nside2_lmax8")
    lp = cg.LegendrePolynomialContainer(int(g["lmax"]), int(g["nside"]), g["nest_good"])
    ref = cg.LegendrePolynomialContainer(file_name=REF_FILE)
    assert np.array_equal(lp.table, ref.table)
    out = tmp_path / "lp.bin"
    lp.write_into_file(str(out))
    assert open(out, "rb").read() == open(REF_FILE, "rb").read()


@pytest.mark.parametrize("l0", [0, 5])
def test_table_matches_oracle(oracle_mod, l0):
    g = load_golden("nside8_lmax24")
    nside, lmax = int(g["nside"]), 12
    with cg.Context(lmax=lmax, fwhm_deg=1.0, nside=nside, good_pixels=g["nest_good"], max_batch=1) as ctx:
        got = ctx.legendre_table(lmax, l0=l0)
    want = oracle_mod.legendre_table(lmax, oracle_mod.unit_vectors(nside, g["nest_good"], "NEST"))
    assert np.array_equal(got, want[l0:])
