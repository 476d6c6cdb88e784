"""ctypes wrapper of the CPU oracle (oracle/cpu_pm.cpp) -- TEST INFRASTRUCTURE.

The oracle restates the reference particle-mesh step (CosmosCuda.cuh,
tugrul512bit/CosmosSimulationWithCuda) on the host.  Only tests/, bench.py's
CPU-baseline leg and __graft_entry__.smoke() use it, always as the expected
result of a comparison or as the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libcpu_pm.so")
_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile oracle/libcpu_pm.so with oracle/Makefile (g++ -fopenmp)."""
    src = os.path.join(_HERE, "cpu_pm.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "libcpu_pm.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.opm_create.restype = ctypes.c_void_p
        L.opm_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.opm_destroy.argtypes = [ctypes.c_void_p]
        L.opm_set_threads.argtypes = [ctypes.c_int]
        L.opm_max_threads.restype = ctypes.c_int
        L.opm_deposit.argtypes = [ctypes.c_void_p, _f32p, _f32p, _f32p, ctypes.c_int64]
        L.opm_potential.argtypes = [ctypes.c_void_p]
        L.opm_gradient.argtypes = [ctypes.c_void_p]
        L.opm_integrate.argtypes = [ctypes.c_void_p, _f32p, _f32p, _f32p, _f32p, ctypes.c_int64]
        L.opm_step.argtypes = [ctypes.c_void_p, _f32p, _f32p, _f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int]
        for name in ("opm_get_density", "opm_get_potential", "opm_get_force",
                     "opm_set_density", "opm_set_potential", "opm_set_force"):
            getattr(L, name).argtypes = [ctypes.c_void_p, _f64p]
        L.opm_get_filters.argtypes = [ctypes.c_void_p, _f64p, _f64p]
        L.opm_integrate_f32_exact.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                              _f32p, _f32p, _f32p, _f32p, ctypes.c_int64]
        L.opm_sort_keys.argtypes = [_f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _u32p]
        L.opm_stable_sort_perm.argtypes = [_u32p, ctypes.c_int64, _u32p]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().opm_set_threads(int(n))


def max_threads() -> int:
    return int(lib().opm_max_threads())


class OraclePM:
    """The reference PM step on the CPU (fp64=True: FP64 oracle; False: FP32 port)."""

    def __init__(self, N: int, cic: bool, dt: float, gmult: float = 1.0, fp64: bool = True):
        self.N = int(N)
        self.cic = bool(cic)
        self.dt = float(dt)
        self.h = lib().opm_create(self.N, int(self.cic), self.dt, float(gmult), int(fp64))
        if not self.h:
            raise ValueError(f"oracle: unsupported lattice size {N}")

    def close(self):
        if self.h:
            lib().opm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stages ---------------------------------------------------------------
    def deposit(self, x, y, m):
        lib().opm_deposit(self.h, x, y, m, x.size)

    def potential(self):
        lib().opm_potential(self.h)

    def gradient(self):
        lib().opm_gradient(self.h)

    def integrate(self, x, y, xo, yo):
        lib().opm_integrate(self.h, x, y, xo, yo, x.size)

    def step(self, x, y, xo, yo, m, nsteps: int = 1):
        lib().opm_step(self.h, x, y, xo, yo, m, x.size, int(nsteps))

    # -- fields ---------------------------------------------------------------
    def density(self):
        out = np.empty((self.N, self.N), np.float64)
        lib().opm_get_density(self.h, out)
        return out

    def potential_field(self):
        out = np.empty((self.N, self.N), np.float64)
        lib().opm_get_potential(self.h, out)
        return out

    def force(self):
        out = np.empty((self.N, self.N, 2), np.float64)
        lib().opm_get_force(self.h, out)
        return out

    def set_density(self, a):
        lib().opm_set_density(self.h, np.ascontiguousarray(a, np.float64))

    def set_potential(self, a):
        lib().opm_set_potential(self.h, np.ascontiguousarray(a, np.float64))

    def set_force(self, a):
        lib().opm_set_force(self.h, np.ascontiguousarray(a, np.float64))

    def filters(self):
        f = np.empty((self.N, self.N, 2), np.float64)
        d = np.empty((self.N, self.N, 2), np.float64)
        lib().opm_get_filters(self.h, f, d)
        return f[..., 0] + 1j * f[..., 1], d[..., 0] + 1j * d[..., 1]


def integrate_f32_exact(force_xy, N, cic, dt, x, y, xo, yo):
    """FP32 gather + update in the exact operation order of the CUDA kernel."""
    lib().opm_integrate_f32_exact(np.ascontiguousarray(force_xy, np.float32), int(N), int(cic),
                                  float(dt), x, y, xo, yo, x.size)


def sort_keys(x, y, N: int, granularity: int):
    keys = np.empty(x.size, np.uint32)
    lib().opm_sort_keys(x, y, x.size, int(N), int(granularity), keys)
    return keys


def stable_sort_perm(keys):
    perm = np.empty(keys.size, np.uint32)
    lib().opm_stable_sort_perm(np.ascontiguousarray(keys, np.uint32), keys.size, perm)
    return perm
