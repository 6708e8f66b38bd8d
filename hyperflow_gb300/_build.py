"""Builds the in-tree CUDA library ``hyperflow_gb300/libhyperflow_gb300.so`` for sm_103a.

Translation units compile in parallel; the shared object links them with the static
CUDA runtime, so loading the library needs no GPU (CUDA calls then report
"no device").  Host code is compiled with -ffp-contract=off so host-side setup
arithmetic (initial conditions, geometry) rounds like the reference on both x86 and Arm.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhyperflow_gb300.so")
HOSTMATH_LIB = os.path.join(PKG, "libhf_hostmath.so")

SOURCES = ["hf_cart.cu", "hf_api.cpp", "hf_uns.cu", "hf_noalloc.cu", "hf_batch.cu", "hf_learned.cu", "hf_diag.cu",
           "hf_render.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(PKG, "..", "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], obj: str = OBJ) -> str:
    out = os.path.join(obj, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    if os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(srcp), *(os.path.getmtime(os.path.join(CSRC, h))
                                      for h in os.listdir(CSRC) if h.endswith((".cuh", ".h", ".hpp")))):
        return out
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", srcp, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False, extra: list[str] | None = None, variant: str = "") -> str:
    """variant "checked": the library with -DHF_CHECKS (every geometry- or mesh-dependent global
    index range-checked into the error word), as libhyperflow_gb300_checked.so."""
    obj = os.path.join(OBJ, variant) if variant else OBJ
    lib_path = LIB if not variant else os.path.join(PKG, f"libhyperflow_gb300_{variant}.so")
    flags = list(extra or []) + (["-DHF_CHECKS"] if variant == "checked" else [])
    os.makedirs(obj, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, flags, obj), srcs))
    cmd = [nvcc(), *ARCH, "-shared", "-o", lib_path, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if variant:
        if verbose:
            print("built", lib_path)
        return lib_path
    # the kernels' arithmetic built for the host (CPU tests of the device math)
    hm = _compile("hf_hostmath.cu", extra or [])
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", HOSTMATH_LIB, hm], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
