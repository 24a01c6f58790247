"""Host drop-in layer (C++): the reference application's command line,
settings, batch mode, GPU model entry points and spectrum writers over the
GB300 engine.  `build()` compiles libgelio_host.so and the `geliosphere`
executable in-tree; `load()` returns the ctypes handle with prototypes."""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_float, c_int32

from geliosphere_gb300 import abi

from .build import EXE, LIB, build  # noqa: F401

_LIB = None


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB):
        raise RuntimeError(f"host layer not built ({LIB} missing); run geliosphere_gb300.host.build()")
    abi.load()   # libgelio_cuda.so first (rpath also finds it)
    lib = ctypes.CDLL(LIB)
    protos = {
        "gelio_host_main": (c_int32, [c_int32, POINTER(c_char_p)]),
        "gelio_host_parse": (c_int32, [c_int32, POINTER(c_char_p)]),
        "gelio_host_reset": (None, []),
        "gelio_host_get_int": (c_int32, [c_char_p, c_int32]),
        "gelio_host_get_float": (c_float, [c_char_p, c_float]),
        "gelio_host_get_string": (c_int32, [c_char_p, c_char_p, c_char_p, c_int32]),
        "gelio_host_put_int": (None, [c_char_p, c_int32]),
        "gelio_host_put_float": (None, [c_char_p, c_float]),
        "gelio_host_put_string": (None, [c_char_p, c_char_p]),
        "gelio_host_load_settings": (c_int32, [c_char_p]),
        "gelio_host_resolve": (c_int32, [c_int32, POINTER(abi.SimParams)]),
        "gelio_host_batch_plan": (c_int32, [c_char_p, POINTER(abi.SimParams), POINTER(c_int32), c_int32,
                                            POINTER(c_int32)]),
        "gelio_host_write_spectra": (c_int32, [c_int32, POINTER(abi.Spectra), c_int32, c_char_p]),
        "gelio_host_log_line": (c_int32, [c_int32, POINTER(abi.ExitRecord), c_float, c_char_p, c_int32]),
        "gelio_host_carrington_rotation": (c_int32, [c_int32, c_int32]),
    }
    for name, (res, args) in protos.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def argv(args: list[str]):
    arr = (c_char_p * (len(args) + 1))()
    for i, a in enumerate(args):
        arr[i] = a.encode()
    arr[len(args)] = None
    return len(args), arr


def parse(args: list[str], program: str = "geliosphere") -> int:
    """gelio_host_parse of a command line; `program` is argv[0], whose
    directory is where month/year runs look for the measured-value tables."""
    n, arr = argv([program, *args])
    return load().gelio_host_parse(n, arr)


def resolve(model: int) -> abi.SimParams:
    """gelio_sim_params the GPU model would run from the current parameter map."""
    out = abi.SimParams()
    st = load().gelio_host_resolve(model, ctypes.byref(out))
    if st != 0:
        raise ValueError(f"gelio_host_resolve: status {st}")
    return out


def get_string(key: str, default: str = "") -> str:
    buf = ctypes.create_string_buffer(4096)
    load().gelio_host_get_string(key.encode(), default.encode(), buf, 4096)
    return buf.value.decode()


def batch_plan(csv_path: str, cap: int = 256):
    """(gelio_sim_params, 1-based CSV row) of every batch row that would run,
    resolved in the current directory as batch mode resolves it."""
    out = (abi.SimParams * cap)()
    rows = (c_int32 * cap)()
    n = c_int32()
    st = load().gelio_host_batch_plan(csv_path.encode(), out, rows, cap, ctypes.byref(n))
    if st != 0:
        raise ValueError(f"gelio_host_batch_plan: status {st}")
    return [(out[i], rows[i]) for i in range(min(n.value, cap))]
