"""Builds libsenk_gpu.so in-tree for sm_103a (nvcc, no cmake).

Every CUDA translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the host-only unit with g++. Host
code is built without floating-point contraction (``-ffp-contract=off``), so the
setup functions round exactly as the reference does on x86 and on Arm hosts. The
result lands in ``senk_gb300/_lib/libsenk_gpu.so``; objects in ``senk_gb300/_build``.
Rebuilds only what changed (sources or headers newer than the object).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsenk_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    # the build script itself too: a change of flags rebuilds everything
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h*")) + [os.path.abspath(__file__)]


def _stale(obj: str, src: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _compile(src: str, verbose: bool) -> str:
    name = os.path.splitext(os.path.basename(src))[0]
    obj = os.path.join(BUILD, name + ".o")
    if not _stale(obj, src, _headers()):
        return obj
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-Xptxas", "-warn-spills", *inc, "-c", src, "-o", obj]
    else:
        # no FMA contraction in host code: the setup (Ilu0, Ilup, ...) must round
        # as the reference does on every host (g++ contracts by default on Arm)
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I", cuda_inc, *inc, "-c", src,
               "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and verbose:
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> str:
    """Compile and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
