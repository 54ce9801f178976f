"""Build the sm_103a CUDA library ``libbcm_gb300.so`` in-tree.

Every translation unit is compiled for ``sm_103a`` only.  The FP64 kernels
are compiled with ``--fmad=false``: the reference's arithmetic is a sequence
of separately rounded multiplies and adds, and contracting them into FMAs
would change results in the last bit.  Output goes to
``bcm_cgli_gb300/_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbcm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra nvcc flags)
UNITS = [
    ("bcm_flux_fp64.cu", ["--fmad=false"]),
    # FP32 work of the split path: approximate division/sqrt (a few ulp) and
    # flush-to-zero are inside its error budget; the FP64 parts are unaffected.
    ("bcm_flux_split.cu", ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("bcm_rk.cu", ["--fmad=false"]),
    ("bcm_halo.cu", ["--fmad=false"]),
    ("bcm_capi.cu", ["--fmad=false"]),
    ("bcm_noalloc.cu", ["--fmad=false"]),
    ("bcm_lusgs.cu", ["--fmad=false"]),
    ("bcm_lusgs_split.cu", ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("bcm_output.cu", ["--fmad=false"]),
    ("bcm_ibm.cu", ["--fmad=false"]),
    ("bcm_tables.cpp", []),
    ("bcm_flags.cpp", []),
]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps() -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(os.path.dirname(HERE), "include", "bcm_gb300.h"))
    return hdrs


def _compile(src: str, flags: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _deps()):
        return obj
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xptxas", "-v" if verbose else "-O3", *flags, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-6000:]}")
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    srcs = [(os.path.join(CSRC, s), f) for s, f in UNITS]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda sf: _compile(sf[0], sf[1], verbose), srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
