"""The batched HMC sampler (cg_hmc_sample, the driver under cg_hmc_run) against the reference's own
Math::HMC::run (source/hmc.cpp:31-126), compiled from the reference's sources, on an analytic
Gaussian -2lnL with the same seed: every leapfrog position must be bit-identical and the chain must
match the file the reference wrote (6 significant digits).  The reference's positions are stored in
tests/golden/hmc_gaussian_reference.npz (make_golden.py, part hmc); where the compiled reference is
present it is also run live.  No device is used."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

import cosmopp_gb300 as cg
from conftest import load_golden


def _ours(g, tag):
    mu, sig = g["mu"], g["sig"]
    seen = []

    def like_grad(x):
        seen.append(x.copy())
        d = (x - mu) / sig
        return (d * d).sum(axis=1), 2 * (x - mu) / sig ** 2

    chain, acc = cg.hmc_sample(like_grad, g["start"][None, :], int(g[tag + "_iters"]), int(g[tag + "_nmax"]),
                               float(g[tag + "_tau"]), jitter=True, seed=int(g[tag + "_seed"]))
    # the first evaluation is the starting point; the reference's leapfrog record starts after it
    return np.vstack(seen)[1:], chain, acc


@pytest.mark.parametrize("tag", ["a", "b"])
def test_leapfrog_positions_bit_identical_to_the_reference(tag):
    g = load_golden("hmc_gaussian_reference")
    pts, chain, acc = _ours(g, tag)
    ref = g[tag + "_points"]
    assert pts.shape == ref.shape
    assert np.array_equal(pts, ref)
    ch = g[tag + "_chain_file"]          # columns: weight 1, -2lnL, x
    assert np.allclose(chain[:, 0, 0], ch[:, 1], rtol=1e-5, atol=1e-5)
    assert np.allclose(chain[:, 0, 1:], ch[:, 2:], rtol=1e-5, atol=1e-5)
    accepted = np.mean(np.any(np.diff(ch[:, 2:], axis=0) != 0, axis=1))
    assert abs(acc[0] - accepted) < 1e-12


def test_against_the_live_reference_when_compiled_here():
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("the reference is compiled only where its sources are")
    R = O.ref()
    dp = ctypes.POINTER(ctypes.c_double)
    R.ref_hmc_gaussian.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_uint,
                                   ctypes.c_int, ctypes.c_char_p, dp, ctypes.c_int]
    g = dict(load_golden("hmc_gaussian_reference"))
    g.update(b_seed=2024, b_iters=40)
    n = len(g["mu"])
    pts = np.zeros((20000, n))
    root = os.path.join(tempfile.mkdtemp(), "hmc")
    cnt = R.ref_hmc_gaussian(n, g["mu"].ctypes.data_as(dp), g["sig"].ctypes.data_as(dp),
                             g["start"].ctypes.data_as(dp), float(g["b_tau"]), int(g["b_nmax"]), 2024, 40,
                             root.encode(), pts.ctypes.data_as(dp), len(pts))
    ours, _, _ = _ours(g, "b")
    assert cnt == len(ours) and np.array_equal(ours, pts[:cnt])
