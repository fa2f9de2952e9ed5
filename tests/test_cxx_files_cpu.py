"""The C++ drop-in's file formats on the CPU, against files the reference's own classes wrote
(tests/golden/make_golden.py): a CMatrix binary file reads back to the reference's matrix and
comment and writes back byte for byte; the text format is the reference's writeIntoTextFile
output byte for byte and reads back to its printed precision; a LegendrePolynomialContainer
file round-trips; Utils::readClFromFile reads what the reference reads (plain C_l, and
l-prefixed D_l converted to C_l); a missing file raises StandardException."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

import cosmopp_gb300 as cg

G = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cg.library()
    out = str(tmp_path_factory.mktemp("cxxcpu") / "test_files_cpu")
    libdir = os.path.join(ROOT, "cosmopp_gb300", "_lib")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cxx", "test_files_cpu.cpp"), "-L", libdir, "-lcosmopp_gb300",
                           "-Wl,-rpath," + libdir, "-o", out])
    return out


def test_file_formats_match_the_reference(exe, tmp_path):
    g = load_golden("files_nside2")
    p = subprocess.run([exe, os.path.join(G, "cmatrix_nside2.bin"), os.path.join(G, "legendre_nside2_lmax8.bin"),
                        os.path.join(G, "cl_plain.txt"), os.path.join(G, "dl_with_l.txt"), str(tmp_path)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.splitlines()
    assert lines[0] == "covariance from the reference"
    assert np.array_equal(np.array(lines[1].split(), dtype=float), g["read_plain"])
    assert np.array_equal(np.array(lines[2].split(), dtype=float), g["read_dl"])
    assert lines[3] == "raised"
    ref_bin = open(os.path.join(G, "cmatrix_nside2.bin"), "rb").read()
    assert open(tmp_path / "c.bin", "rb").read() == ref_bin
    n = int(np.frombuffer(ref_bin[:4], dtype=np.int32)[0])
    assert np.array_equal(np.frombuffer(ref_bin[4:4 + 8 * n * (n + 1) // 2], dtype=np.float64), g["c_packed"])
    assert open(tmp_path / "c.txt").read() == open(os.path.join(G, "cmatrix_nside2.txt")).read()
    back = np.fromfile(tmp_path / "c_from_txt.bin", dtype=np.uint8).tobytes()
    vals = np.frombuffer(back[4:4 + 8 * n * (n + 1) // 2], dtype=np.float64)
    assert np.allclose(vals, g["c_packed"], rtol=1e-5, atol=1e-9)
    assert open(tmp_path / "lp.bin", "rb").read() == open(os.path.join(G, "legendre_nside2_lmax8.bin"), "rb").read()


@pytest.mark.parametrize("src", ["test_dropin.cpp", "test_legendre_lp.cpp", "test_files_cpu.cpp"])
def test_dropin_header_compiles_as_cxx11_without_warnings(src):
    """The reference builds with -std=c++11 (CMakeLists.txt:13); code using the drop-in header
    must compile there too, warning-free under -Wall -Wextra."""
    p = subprocess.run(["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                        os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cxx", src)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
