"""The C++ drop-in classes (include/cosmopp_gb300/cosmopp.hpp) used exactly as
the reference's own low-l test uses CMatrixGenerator / Likelihood, compiled
with g++ against the C-ABI library and compared with the golden fixtures from
the reference's code; plus a leapfrog on PixelLikelihoodWithDerivs."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

import cosmopp_gb300 as cg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cg.library()
    out = str(tmp_path_factory.mktemp("cxx") / "test_dropin")
    libdir = os.path.join(ROOT, "cosmopp_gb300", "_lib")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cxx", "test_dropin.cpp"), "-L", libdir, "-lcosmopp_gb300",
                           "-Wl,-rpath," + libdir, "-o", out])
    return out


@pytest.mark.parametrize("name", ["nside4", "nside8_lmax24"])
def test_reference_flow_through_cxx_dropin(exe, name, tmp_path):
    g = load_golden(name)
    inp = tmp_path / "in.txt"
    with open(inp, "w") as f:
        f.write("%d %d %.17g %.17g %d\n" % (int(g["nside"]), int(g["lmax"]), float(g["fwhm_deg"]),
                                            float(g["sigma"]), len(g["nest_good"])))
        f.write(" ".join(str(int(v)) for v in g["nest_good"]) + "\n")
        f.write(" ".join("%.17g" % v for v in g["cls"][0]) + "\n")
        f.write(" ".join("%.17g" % v for v in g["d"]) + "\n")
    cbin = tmp_path / "c.bin"
    p = subprocess.run([exe, str(inp), str(cbin)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    c = np.fromfile(cbin, dtype=np.float64)
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["c_sha256"])
    like, chi2, logdet = map(float, p.stdout.splitlines()[0].split())
    assert abs(logdet - g["logdet_ref"][0]) <= 1e-6
    assert abs(chi2 - g["chi2"][0]) <= 1e-6
    assert abs(like - g["like_ref"][0]) <= 1e-6
    hmc = p.stdout.splitlines()[1].split()
    assert hmc[0] == "hmc"
    # a small step size leapfrog conserves the Hamiltonian to O(tau^2)
    assert abs(float(hmc[2])) < 0.05


def test_low_l_flow_with_fiducial_matrix_through_cxx_dropin(exe, tmp_path):
    """clToCMatrix + getFiducialMatrix + noise -> Likelihood -> calculate, as
    source/test_like_low.cpp:181-193 runs it."""
    g = load_golden("fid_nside4")
    lmax = int(g["lmax"])
    inp = tmp_path / "in.txt"
    with open(inp, "w") as f:
        f.write("%d %d %.17g %.17g %d\n" % (int(g["nside"]), lmax, float(g["fwhm_deg"]), float(g["sigma"]),
                                            len(g["nest_good"])))
        f.write(" ".join(str(int(v)) for v in g["nest_good"]) + "\n")
        f.write(" ".join("%.17g" % v for v in g["cl_full"][:lmax + 1]) + "\n")
        f.write(" ".join("%.17g" % v for v in g["d"]) + "\n")
        f.write("%d\n" % int(g["lmax_max"]) + " ".join("%.17g" % v for v in g["cl_full"]) + "\n")
    cbin, fbin = tmp_path / "c.bin", tmp_path / "fid.bin"
    p = subprocess.run([exe, str(inp), str(cbin), str(fbin)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert hashlib.sha256(np.fromfile(cbin, dtype=np.float64).tobytes()).hexdigest() == str(g["c_sha256"])
    assert np.array_equal(np.fromfile(fbin, dtype=np.float64), g["fid_packed"])
    like, chi2, logdet = map(float, p.stdout.splitlines()[0].split())
    assert abs(chi2 - float(g["chi2"])) <= 1e-6
    assert abs(logdet - float(g["logdet_ref"])) <= 1e-6
    assert abs(like - float(g["like_ref"])) <= 1e-6


def test_legendre_container_and_cl_file_through_cxx_dropin(tmp_path):
    """LegendrePolynomialContainer built on the GPU writes the reference's file byte for
    byte; the reference's own file reads back to the same values; clToCMatrix with that
    table and clToCMatrix from a C_l text file give the reference's matrices."""
    g = load_golden("legendre_nside2_lmax8")
    cg.library()
    exe = str(tmp_path / "test_legendre_lp")
    libdir = os.path.join(ROOT, "cosmopp_gb300", "_lib")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cxx", "test_legendre_lp.cpp"), "-L", libdir,
                           "-lcosmopp_gb300", "-Wl,-rpath," + libdir, "-o", exe])
    inp = tmp_path / "in.txt"
    with open(inp, "w") as f:
        f.write("%d %d %.17g %d\n" % (int(g["nside"]), int(g["lmax"]), float(g["fwhm_deg"]), len(g["nest_good"])))
        f.write(" ".join(str(int(v)) for v in g["nest_good"]) + "\n")
    clf = tmp_path / "cl.txt"
    with open(clf, "w") as f:
        f.write("".join("%.17g\n" % v for v in g["cl"]))
    ref_file = os.path.join(ROOT, "tests", "golden", "legendre_nside2_lmax8.bin")
    p = subprocess.run([exe, str(inp), ref_file, str(clf), str(tmp_path)], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.split() == ["0", "refused"]
    assert open(tmp_path / "lp.bin", "rb").read() == open(ref_file, "rb").read()
    assert np.array_equal(np.fromfile(tmp_path / "c_lp.bin", dtype=np.float64), g["c_lp"])
    assert np.array_equal(np.fromfile(tmp_path / "c_file.bin", dtype=np.float64), g["c_plain"])
