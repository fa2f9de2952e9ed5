"""Compile the cosmopp_gb300 CUDA/C++ sources into the in-tree shared library
cosmopp_gb300/_lib/libcosmopp_gb300.so (sm_103a only, static CUDA runtime).

    python -m cosmopp_gb300.build        # or: from cosmopp_gb300 import build; build.build()
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcosmopp_gb300.so")

CU_SOURCES = ["k_chol.cu", "k_fp64.cu", "k_hmc.cu", "k_mixed.cu", "k_noalloc.cu", "k_tc.cu"]
CXX_SOURCES = ["cg_abi.cpp", "cg_geometry.cpp", "cg_hmc.cpp", "cg_mcmc.cpp", "cg_tune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build cosmopp_gb300")


def _cuda_include(nvcc):
    return os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "cosmopp_gb300.h"))
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                         "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", _cuda_include(nvcc),
                         "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + CXX_SOURCES]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
