"""Build libmhdgb.so (and the C++ driver) for sm_103a, in-tree.

    python -m mhdturbulence_gb300.build          # or __graft_entry__.build()

Translation units are compiled in parallel with nvcc:
  csrc/stages.cu  -fmad=false   stage kernels + the bit-exact FP64 fused step
  csrc/fp64.cu                  FP64 fused steps (FMA contraction), several tile shapes
  csrc/mixed.cu                 FP32-mixed fused steps (fast FP32 div/sqrt), several tile shapes
  csrc/solver.cu                host side of the C ABI (include/mhdgb.h)
  csrc/ghost_noalloc.cu         allocation-free ghost fill on a caller-owned array
  csrc/output.cpp               writer of the reference's snapshot files (host code)
and linked into mhdturbulence_gb300/_build/libmhdgb.so (static CUDA runtime).
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
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libmhdgb.so")
DRIVER = os.path.join(OUT, "mhdgb_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the host code (grid generation, spacing tables) must round every operation
# separately, as the reference does; aarch64 g++ would otherwise fuse a*b+c into FMA.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include")]
UNITS = [
    ("stages.cu", ["-fmad=false"]),
    ("fp64.cu", []),
    ("mixed.cu", ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("solver.cu", []),
    ("ghost_noalloc.cu", []),
    ("output.cpp", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhdgb.so")


def _sources_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "mhdgb.h"),
                                                                  os.path.join(ROOT, "include", "mhdgb_ref_api.hpp")]
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(src, extra, verbose):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False, driver: bool = True) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        if not driver or os.path.exists(DRIVER):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libmhdgb.so failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if driver:
        src = os.path.join(CSRC, "mhdgb_run.cpp")
        if os.path.exists(src):
            r = subprocess.run([nvcc(), *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                                "-I" + os.path.join(ROOT, "include"), src,
                                "-o", DRIVER, "-L" + OUT, "-lmhdgb", "-Xlinker", "-rpath=$ORIGIN"],
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"build of mhdgb_run failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
