"""In-tree build of libcoolpdlp_cuda.so (nvcc, sm_103a only).

Each .cu translation unit compiles in parallel into coolpdlp.jl_gb300/_build/,
then one shared library is linked into coolpdlp.jl_gb300/lib/.  Rebuilds are
incremental on source/header modification times.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

from . import _abi

PKG = _abi.PKG_ROOT
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build_library(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(_abi.LIB_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + [_abi.HEADER_PATH]
    hdr_time = _newest(headers)
    flags = NVCC_FLAGS + list(extra_flags or []) + os.environ.get("CPDLP_NVCC_EXTRA", "").split()
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not force and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time)):
            return obj
        cmd = [exe] + ARCH + flags + ["-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        os.replace(obj + ".tmp", obj)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(compile_one, sources))
    out = _abi.LIB_PATH
    if force or not os.path.exists(out) or os.path.getmtime(out) < _newest(objs):
        cmd = [exe] + ARCH + ["-shared", "-cudart", "static", "-o", out + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
