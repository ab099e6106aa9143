"""Builds libppi_gpu.so (the CUDA evaluator behind include/ppi_gpu.h) in-tree.

nvcc compiles each translation unit of ppi-auto_gb300/csrc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel and links one
shared library into ppi-auto_gb300/_build/.  ``-fmad=false`` keeps every
multiply and add separately rounded, as the reference's host build does.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # ppi-auto_gb300/
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libppi_gpu.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-I", CSRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libppi_gpu.so")
    return exe


def _compile(src, ptxas_verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + NVCC_FLAGS
    if ptxas_verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, ptxas_verbose=False) -> str:
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), sources))
    if verbose or ptxas_verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + [o for o, _ in results] + ARCH + ["-cudart", "shared"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


# The benchmark's measurement library: per-opcode arithmetic throughput for
# the op-mix-aware roofline (not part of the evaluator library).
OPCOST_SRC = os.path.join(PKG, "bench_csrc", "opcost.cu")
OPCOST_LIB = os.path.join(OUT, "libppi_opcost.so")


def build_opcost() -> str:
    os.makedirs(OUT, exist_ok=True)
    tmp = OPCOST_LIB + ".tmp"
    cmd = [nvcc(), "-shared", OPCOST_SRC, "-o", tmp] + ARCH + NVCC_FLAGS + ["-cudart", "shared"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (OPCOST_SRC, r.stdout, r.stderr))
    os.replace(tmp, OPCOST_LIB)
    return OPCOST_LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
