"""Compile librbx.so (CUDA kernels for sm_103a + C ABI) in-tree with nvcc.

Usage: ``python -m openmm_rigidbody_plugin_gb300.build`` or ``build_library()`` from Python.
Translation units compile in parallel into ``_build/``; the shared library is written next to
this file. No cmake, no PyTorch extension machinery: the product is a plain C-ABI library.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librbx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["rbx_refined.cu", "rbx_kernels.cu", "rbx_forces.cu", "rbx_setup.cu", "rbx_plan.cu", "rbx_host.cpp",
           "rbx_batch.cpp"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librbx")
    return path


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-std=c++17", "-O3", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall"]
    if src.endswith(".cu"):
        # FP32 division and square root need not be IEEE-exact anywhere on the single/mixed path
        # (rotation increments and series; the float-float sums use explicit round-to-nearest
        # adds); FP64 code is unaffected by these flags.
        cmd += ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
        if src == "rbx_setup.cu":
            # the device body setup repeats the host's FP64 arithmetic exactly: no contraction
            cmd += ["-fmad=false"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++", "-Xcompiler", "-ffp-contract=off"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compilation of {src} failed:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "rbx.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build_library(force=False, verbose=False):
    """Build librbx.so if any source is newer than it; returns the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["--cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link of librbx.so failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
