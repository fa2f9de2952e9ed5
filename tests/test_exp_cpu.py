"""The exp used to turn ln C_l into C_l in both HMC drivers (cosmopp_gb300/csrc/cg_exp.h): within
2 ulp of the long-double exp over the range samplers visit, compiled here with the library's host
flags (the device copy is the same source; the GPU test of the drivers checks that the two agree
bit for bit)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "cosmopp_gb300", "csrc")

PROG = r"""
#include "cg_exp.h"
#include <cmath>
#include <cstdio>
int main()
{
    double worst = 0;
    for (int i = 0; i <= 400000; ++i) {
        const double x = -60.0 + 120.0 * i / 400000.0;
        const long double r = expl((long double)x);
        const double rd = (double)r;
        const double ulp = std::nextafter(rd, INFINITY) - rd;
        const double e = (double)fabsl((long double)cg::exp_same(x) - r) / ulp;
        if (e > worst) worst = e;
    }
    const bool edges = cg::exp_same(0.0) == 1.0 && cg::exp_same(800.0) == INFINITY && cg::exp_same(-800.0) == 0.0 &&
                       std::isnan(cg::exp_same(NAN));
    std::printf("%.6f %d\n", worst, edges ? 1 : 0);
    return 0;
}
"""


def test_exp_same_accuracy(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    src = tmp_path / "t.cpp"
    src.write_text(PROG)
    exe = tmp_path / "t"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    worst, edges = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert float(worst) <= 2.0
    assert edges == "1"
