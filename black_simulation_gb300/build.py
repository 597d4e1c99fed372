"""Builds libbhk.so in-tree for sm_103a (nvcc cross-compiles; no GPU needed to build).

    python -m black_simulation_gb300.build            # or build() from Python

Translation units are compiled in parallel into _build/ and linked into
black_simulation_gb300/libbhk.so. bhk_steps.cu (the per-step mirrors) and bhk_eht.cu (the EHT
image, a sum over the integrator's steps) are compiled with --fmad=false so their FP64 results
track the reference's C++ to rounding.
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
OUT = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libbhk.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I" + os.path.join(ROOT, "include")]

UNITS = {
    "bhk_trace.cu": [],
    "bhk_api.cu": [],
    "bhk_steps.cu": ["--fmad=false"],
    "bhk_diag.cu": [],
    "bhk_static.cu": [],
    "bhk_surrogate.cu": [],
    "bhk_eht.cu": ["--fmad=false"],
}
EXTRA_UNITS: dict[str, list[str]] = {}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: libbhk needs the CUDA toolkit to build")
    return path


def _compile(src: str, flags: list[str], verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    units = dict(UNITS)
    units.update(EXTRA_UNITS)
    srcs = [os.path.join(CSRC, u) for u in units]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "bhk.h"))
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(d) for d in deps)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), units.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lcuda"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
