"""TEST INFRASTRUCTURE: the reference's own 2D Geliosphere CUDA kernels on this GPU.

`make -C oracle ref_gpu` compiles the reference's CUDAKernel/src/
CosmicConstants.cu, CosmicUtils.cu and GeliosphereModel.cu (one translation
unit, oracle/ref_gpu_unit.cu) with the reference's CUDA flags
(CUDAKernel/CMakeLists.txt: --use_fast_math -Xptxas -O3) into
oracle/_ref/ref_geliosphere.cubin for sm_103a.  This module loads that cubin
through the CUDA driver API and drives it the way the reference's host code
does:

* GeliosphereGpuModel::setThreadBlockSize (GeliosphereGpuModel.cpp:48-93):
  compute capability 10.3 is not in its table, so 64 blocks x 64 threads
  (the kernels' own BLOCK_SIZE/THREAD_SIZE fallback, GeliosphereModel.cuh)
  and no shared-memory opt-in;
* setConstants / setGeliosphereModelConstants (CosmicConstants.cu:40-110)
  for a user-entered K0: the __constant__ values V, dt, K0, ratio, delta0,
  alphaM, polarity, rInit, thetainj, injectionMax, useUniformInjection are
  written from a gelio_sim_params (the same resolved values the engine's
  host layer derives from the command line);
* runGeliosphereSimulation (GeliosphereModel.cu:399-449): curandInitialization
  once, then per chunk of 4,096 particles nullCount, a device
  synchronisation, trajectoryPreSimulationGeliosphere, a synchronisation,
  trajectorySimulationGeliosphere (dynamic shared memory for 64 curand states
  and 64 float2), a synchronisation, the exit counter read from the symbol
  and the chunk's exit records copied to the host.  The reference reads the
  injection energies and weights of the exits from managed memory and prints
  each exit to log.dat with fprintf; here those two arrays are copied to the
  host per chunk and the rows are kept in memory (no text formatting).

The reference seeds curand with clock() (CosmicUtils.cu:47-50), so its runs
are not repeatable; comparisons with it are statistical.  Only bench.py and
tests/ use this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import time
from ctypes import byref, c_char_p, c_int, c_size_t, c_uint, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_geliosphere.cubin")

BLOCKS, THREADS = 64, 64                  # the cc 10.3 fallback shape of the reference
CHUNK = BLOCKS * THREADS
CURAND_STATE_BYTES = 48                   # sizeof(curandStateXORWOW)
RECORD = np.dtype([("Tkin", "<f4"), ("r", "<f4"), ("theta", "<f4"), ("id", "<i4")])   # trajectoryHistoryGeliosphere

# Itanium-mangled names of the reference kernels (C++ linkage)
K_NULL = b"_Z9nullCountv"
K_CURAND = b"_Z20curandInitializationP17curandStateXORWOW"
K_PRE = b"_Z34trajectoryPreSimulationGeliospherePfS_Pdi"
K_SIM = b"_Z31trajectorySimulationGeliosphereP28trajectoryHistoryGeliosphereiP17curandStateXORWOW"


def available() -> bool:
    return os.path.exists(CUBIN)


class CudaError(RuntimeError):
    pass


class _Driver:
    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        L = self.lib
        L.cuGetErrorString.argtypes = [c_int, ctypes.POINTER(c_char_p)]
        L.cuModuleLoad.argtypes = [ctypes.POINTER(c_void_p), c_char_p]
        L.cuModuleGetFunction.argtypes = [ctypes.POINTER(c_void_p), c_void_p, c_char_p]
        L.cuModuleGetGlobal_v2.argtypes = [ctypes.POINTER(c_uint64), ctypes.POINTER(c_size_t), c_void_p, c_char_p]
        L.cuModuleUnload.argtypes = [c_void_p]
        L.cuMemAlloc_v2.argtypes = [ctypes.POINTER(c_uint64), c_size_t]
        L.cuMemFree_v2.argtypes = [c_uint64]
        L.cuMemcpyHtoD_v2.argtypes = [c_uint64, c_void_p, c_size_t]
        L.cuMemcpyDtoH_v2.argtypes = [c_void_p, c_uint64, c_size_t]
        L.cuLaunchKernel.argtypes = [c_void_p, c_uint, c_uint, c_uint, c_uint, c_uint, c_uint, c_uint, c_void_p,
                                     ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p)]
        L.cuDevicePrimaryCtxRetain.argtypes = [ctypes.POINTER(c_void_p), c_int]
        L.cuDevicePrimaryCtxRelease_v2.argtypes = [c_int]
        L.cuCtxPushCurrent_v2.argtypes = [c_void_p]
        L.cuCtxPopCurrent_v2.argtypes = [ctypes.POINTER(c_void_p)]

    def check(self, rc, what):
        if rc != 0:
            s = c_char_p()
            self.lib.cuGetErrorString(rc, byref(s))
            raise CudaError(f"{what}: CUDA driver error {rc} ({(s.value or b'').decode()})")


class ReferenceGeliosphere:
    """The reference's 2D Geliosphere kernels loaded on one device.  Call
    run(sim, chunks) for each simulation; close() releases everything."""

    def __init__(self, device: int = 0):
        if not available():
            raise FileNotFoundError(f"{CUBIN} not built (make -C oracle ref_gpu needs the reference sources)")
        self.d = _Driver()
        L, chk = self.d.lib, self.d.check
        chk(L.cuInit(0), "cuInit")
        self.dev = device
        self.ctx = c_void_p()
        chk(L.cuDevicePrimaryCtxRetain(byref(self.ctx), device), "cuDevicePrimaryCtxRetain")
        chk(L.cuCtxPushCurrent_v2(self.ctx), "cuCtxPushCurrent")
        self.mod = c_void_p()
        chk(L.cuModuleLoad(byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for name in (K_NULL, K_CURAND, K_PRE, K_SIM):
            f = c_void_p()
            chk(L.cuModuleGetFunction(byref(f), self.mod, name), "cuModuleGetFunction " + name.decode())
            self.fn[name] = f
        # device buffers of GeliosphereGpuModel::prepareAndRunSimulation (GeliosphereGpuModel.cpp:16-21)
        self.buf = {}
        for key, nbytes in (("w", CHUNK * 8), ("pinj", CHUNK * 4), ("Tkininj", CHUNK * 4),
                            ("state", CHUNK * CURAND_STATE_BYTES), ("history", CHUNK * RECORD.itemsize)):
            p = c_uint64()
            chk(L.cuMemAlloc_v2(byref(p), nbytes), "cuMemAlloc " + key)
            self.buf[key] = p
        self._pop()

    # -- driver helpers ---------------------------------------------------
    def _push(self):
        self.d.check(self.d.lib.cuCtxPushCurrent_v2(self.ctx), "cuCtxPushCurrent")

    def _pop(self):
        c = c_void_p()
        self.d.check(self.d.lib.cuCtxPopCurrent_v2(byref(c)), "cuCtxPopCurrent")

    def _symbol(self, name: str):
        p, n = c_uint64(), c_size_t()
        self.d.check(self.d.lib.cuModuleGetGlobal_v2(byref(p), byref(n), self.mod, name.encode()),
                     "cuModuleGetGlobal " + name)
        return p, n.value

    def _put(self, name: str, value: np.ndarray):
        p, n = self._symbol(name)
        value = np.ascontiguousarray(value)
        assert value.nbytes == n, (name, value.nbytes, n)
        self.d.check(self.d.lib.cuMemcpyHtoD_v2(p, value.ctypes.data, n), "set " + name)

    def _launch(self, name, grid, block, shmem, args):
        # kernelParams: one pointer to each argument's value (the ctypes
        # objects in `args` stay alive for the call)
        ptrs = (c_void_p * len(args))(*[ctypes.addressof(a) for a in args]) if args else None
        self.d.check(self.d.lib.cuLaunchKernel(self.fn[name], grid, 1, 1, block, 1, 1, shmem, None,
                                               ptrs, None), "launch " + name.decode())

    def _sync(self):
        self.d.check(self.d.lib.cuCtxSynchronize(), "cuCtxSynchronize")

    def _get(self, dst: np.ndarray, src: c_uint64, nbytes: int):
        self.d.check(self.d.lib.cuMemcpyDtoH_v2(dst.ctypes.data, src, nbytes), "cuMemcpyDtoH")

    # -- the reference's run ----------------------------------------------
    def set_constants(self, sim):
        """setConstants + setGeliosphereModelConstants for a 2D Geliosphere
        simulation with a user-entered K0 (the value is applied as given)."""
        f32 = np.float32
        self._put("V", f32(sim.V))
        self._put("dt", f32(sim.dt))
        self._put("K0", f32(sim.K0))
        self._put("ratio", f32(sim.ratio))
        self._put("delta0", f32(sim.delta0))
        self._put("alphaM", f32(sim.tilt))
        self._put("polarity", f32(sim.polarity))
        self._put("rInit", f32(sim.r_injection))
        self._put("thetainj", f32(sim.theta_injection))
        self._put("injectionMax", f32(sim.injection_max))
        from geliosphere_gb300 import abi
        uniform = sim.injection == abi.GELIO_INJ_REFERENCE_UNIFORM
        if not uniform and sim.injection != abi.GELIO_INJ_SOLARPROP_GRID:
            raise ValueError("the reference kernel injects on its uniform grid or the SolarProp grid only")
        self._put("useUniformInjection", np.array([1 if uniform else 0], dtype=np.uint8))

    def run(self, sim, chunks: int):
        """`chunks` chunks of 4,096 particles of one simulation (particle ids
        0 .. 4096 chunks - 1, as the reference numbers them).  Returns
        (seconds, rows) with rows the reference log.dat columns (Tkininj,
        Tkin, r, w, thetainj, theta) of every exit, before %g formatting;
        seconds is the wall time of the chunk loop, from the first launch to
        the last record copied to the host."""
        self._push()
        try:
            self.set_constants(sim)
            b = self.buf
            self._launch(K_CURAND, BLOCKS, THREADS, 0, [b["state"]])
            self._sync()
            counter_ptr, _ = self._symbol("outputCounter")
            counter = np.zeros(1, np.int32)
            hist = np.empty(CHUNK, RECORD)
            tinj = np.empty(CHUNK, np.float32)
            w = np.empty(CHUNK, np.float64)
            shmem = THREADS * CURAND_STATE_BYTES + THREADS * 8
            parts = []
            t0 = time.perf_counter()
            for k in range(chunks):
                self._launch(K_NULL, 1, 1, 0, [])
                self._sync()
                self._launch(K_PRE, BLOCKS, THREADS, 0, [b["Tkininj"], b["pinj"], b["w"], c_int(k)])
                self._sync()
                self._launch(K_SIM, BLOCKS, THREADS, shmem, [b["history"], c_int(k), b["state"]])
                self._sync()
                self._get(counter, counter_ptr, 4)
                n = int(counter[0])
                if n:
                    if not 0 < n <= CHUNK:
                        raise CudaError(f"exit counter {n} outside the chunk")
                    self._get(hist, b["history"], n * RECORD.itemsize)
                    self._get(tinj, b["Tkininj"], CHUNK * 4)
                    self._get(w, b["w"], CHUNK * 8)
                    h = hist[:n].copy()
                    if h["id"].min() < 0 or h["id"].max() >= CHUNK:
                        raise CudaError("exit record with a particle id outside the chunk")
                    parts.append(np.stack([tinj[h["id"]].astype(np.float64), h["Tkin"].astype(np.float64),
                                           h["r"].astype(np.float64), w[h["id"]],
                                           np.full(n, np.float32(sim.theta_injection), np.float64),
                                           h["theta"].astype(np.float64)], 1))
            secs = time.perf_counter() - t0
        finally:
            self._pop()
        rows = np.concatenate(parts) if parts else np.zeros((0, 6))
        return secs, rows

    def close(self):
        if getattr(self, "mod", None) is None:
            return
        self._push()
        for p in self.buf.values():
            self.d.lib.cuMemFree_v2(p)
        self.d.lib.cuModuleUnload(self.mod)
        self.mod = None
        self._pop()
        self.d.lib.cuDevicePrimaryCtxRelease_v2(self.dev)
