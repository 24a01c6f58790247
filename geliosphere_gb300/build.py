"""In-tree build of libgelio_cuda.so for sm_103a (nvcc, no cmake).

The translation units (four model kernels, the C-ABI host code, the
allocation-free entry point and the surrogate network) are compiled in parallel and linked into geliosphere_gb300/_lib/libgelio_cuda.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libgelio_cuda.so")

UNITS = ["api.cu", "k_fp.cu", "k_bp.cu", "k_solarprop.cu", "k_geliosphere.cu", "noalloc.cu", "mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 SDE steps: flush denormals, approximate division/sqrt where the
# kernels ask for them; the bit-exact parts use explicit _rn intrinsics.
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-ftz=true",
           "-prec-div=false", "-prec-sqrt=false", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _sources_newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "gelio.h"))
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = _headers()
    cmds = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ_DIR, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _sources_newer(obj, [src] + headers):
            cmds.append([nvcc(), *ARCH, *NVFLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return cmd

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, cmds))
    if force or cmds or _sources_newer(LIB, objs):
        link = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        run(link)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
