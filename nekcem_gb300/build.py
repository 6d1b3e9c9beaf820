"""Builds the in-tree CUDA library ``nekcem_gb300/libnekcem_gb300.so`` for sm_103a.

The library is the product: the C ABI of ``include/nekcem_gpu.h`` with the
stage kernels.  Sources compile in parallel with nvcc (one -gencode, no
cmake); the plain-form kernels compile with ``--fmad=false`` so their
rounding follows the reference's unfused arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libnekcem_gb300.so")
OBJDIR = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "nekgpu_host.cpp": ["-Xcompiler", "-ffp-contract=off"],  # same rounding on x86 and Arm
    "nekgpu_plain.cu": ["--fmad=false"],
    "nekgpu_fused.cu": [],
    "nekgpu_mixed.cu": [],
    "nekgpu_util.cu": [],
    "nekgpu_noalloc.cu": [],
    "nekgpu_adjoint.cu": [],
    "nekgpu_adjoint_host.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "nekgpu_io.cpp": [],
    # --fmad=false for the device code; the host part evaluates the source's
    # time factor, which must round as the oracle's does
    "nekgpu_2d.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "nekgpu_curved.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(INCLUDE, "nekcem_gpu.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJDIR, src + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, x) for s, x in SOURCES.items()]
        objs = [f.result() for f in futs]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
