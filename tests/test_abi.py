"""The C-ABI library loads and exports every entry point that include/gelio.h
declares, with the struct layouts the header defines (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gelio.h")


def declared_functions(path):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gelio_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from geliosphere_gb300 import build
    build.build()
    from geliosphere_gb300 import abi
    return abi.load()


def test_exports_every_declared_symbol(lib):
    names = declared_functions(HEADER)
    assert len(names) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "geliosphere_gb300", "_lib", "libgelio_cuda.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (gelio_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_struct_layouts_match_header(tmp_path):
    from geliosphere_gb300 import abi
    prog = tmp_path / "sz.c"
    prog.write_text('#include <stdio.h>\n#include "gelio.h"\n'
                    'int main(){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gelio_sim_params), '
                    'sizeof(gelio_spectra), sizeof(gelio_exit_record), sizeof(gelio_run_opts), '
                    'sizeof(gelio_run_stats), sizeof(gelio_trajectory), sizeof(gelio_surrogate_opts));}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert sizes == [ctypes.sizeof(abi.SimParams), ctypes.sizeof(abi.Spectra), ctypes.sizeof(abi.ExitRecord),
                     ctypes.sizeof(abi.RunOpts), ctypes.sizeof(abi.RunStats), ctypes.sizeof(abi.Trajectory),
                     ctypes.sizeof(abi.SurrogateOpts)]


def test_status_strings_and_null_arguments(lib):
    from geliosphere_gb300 import abi
    assert lib.gelio_abi_version() == abi.GELIO_ABI_VERSION
    for code in (0, 1, 2, 3, 4, 5, 6, 7, 100, 101):
        assert lib.gelio_status_string(code)
    assert lib.gelio_create(None, 0) == abi.GELIO_ERR_INVALID_ARGUMENT
    assert lib.gelio_destroy(None) == abi.GELIO_ERR_INVALID_ARGUMENT
    assert lib.gelio_run(None, None, 0, None, None, None) == abi.GELIO_ERR_INVALID_ARGUMENT


def test_no_device_is_an_error_not_a_fallback(lib):
    from geliosphere_gb300 import abi
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    ctx = ctypes.c_void_p()
    assert lib.gelio_create(ctypes.byref(ctx), 0) == abi.GELIO_ERR_NO_DEVICE
    with pytest.raises(abi.GelioError):
        from geliosphere_gb300 import Engine
        Engine(0)


def test_host_library_exports_every_declared_symbol():
    from geliosphere_gb300 import host
    host.build()
    lib = host.load()
    names = declared_functions(os.path.join(ROOT, "include", "gelio_host.h"))
    assert len(names) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", host.LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (gelio_host_\w+)", out))
    missing = [n for n in names if n.startswith("gelio_host_") and n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)
