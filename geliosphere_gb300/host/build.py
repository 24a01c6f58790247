"""In-tree build of the host drop-in layer: libgelio_host.so and the
`geliosphere` executable (g++, no cmake), linked against libgelio_cuda.so."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
OUT = os.path.join(HERE, "_build")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgelio_host.so")
EXE = os.path.join(OUT, "geliosphere")

UNITS = ["ParamsCarrier.cpp", "FileUtils.cpp", "ResultsUtils.cpp", "Engine.cpp", "GpuModels.cpp", "Results.cpp",
         "Input.cpp", "Algorithms.cpp", "capi.cpp"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-result", "-I" + os.path.join(ROOT, "include")]


def _cxx() -> str:
    return os.environ.get("CXX", "g++")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    from geliosphere_gb300 import build as cuda_build
    cuda_lib = cuda_build.build()
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".hpp")]
    headers += [os.path.join(ROOT, "include", "gelio.h"), os.path.join(ROOT, "include", "gelio_host.h")]
    cmds, objs = [], []
    for u in UNITS + ["main.cpp"]:
        src = os.path.join(HERE, u)
        obj = os.path.join(OBJ, u.replace(".cpp", ".o"))
        if u != "main.cpp":
            objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmds.append([_cxx(), *CXXFLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stdout.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(run, cmds))
    libdir = os.path.dirname(cuda_lib)
    rpath = "-Wl,-rpath,$ORIGIN/../../_lib"
    if force or cmds or _newer(LIB, objs + [cuda_lib]):
        run([_cxx(), "-shared", "-o", LIB, *objs, "-L" + libdir, "-lgelio_cuda", rpath])
    main_obj = os.path.join(OBJ, "main.o")
    if force or cmds or _newer(EXE, [main_obj, LIB]):
        run([_cxx(), "-o", EXE, main_obj, "-L" + OUT, "-lgelio_host", "-L" + libdir, "-lgelio_cuda",
             "-Wl,-rpath,$ORIGIN", rpath])
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
