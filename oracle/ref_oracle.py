"""ctypes wrapper of the reference-kernel runner -- TEST INFRASTRUCTURE.

RefGPU runs the reference's own CUDA kernels (compiled from CosmosCuda.cuh,
see oracle/ref_build.py) with cuFFT on the GPU, through the host sequence of
Universe<K>'s constructor and step (oracle/ref_runner.cpp).  It needs the PTX
built from the reference sources (oracle/_ref/*.ptx) and a GPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from oracle import ref_build

_lib = None
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def available(N: int, dt: float, g: float = 1.0) -> bool:
    return os.path.exists(ref_build.ptx_path(N, dt, g))


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build_runner()
        if not path or not os.path.exists(path):
            raise RuntimeError("reference runner not built (nvcc missing)")
        L = ctypes.CDLL(path)
        L.ref_create.restype = ctypes.c_void_p
        L.ref_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ref_destroy.argtypes = [ctypes.c_void_p]
        L.ref_error.restype = ctypes.c_char_p
        L.ref_set_state.argtypes = [ctypes.c_void_p] + [_f32p] * 5
        L.ref_get_state.argtypes = [ctypes.c_void_p] + [_f32p] * 4
        L.ref_get_fields.argtypes = [ctypes.c_void_p] + [_f32p] * 3
        L.ref_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_render.argtypes = [ctypes.c_void_p, _f32p, _f32p]
        L.ref_time_steps.restype = ctypes.c_float
        L.ref_time_steps.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib = L
    return _lib


class RefGPU:
    """The reference's step on the GPU for lattice N, time step dt (baked into the PTX)."""

    def __init__(self, N: int, cic: bool, dt: float, P: int, g: float = 1.0):
        path = ref_build.ptx_path(N, dt, g)
        if not os.path.exists(path):
            raise FileNotFoundError(f"reference PTX not built for N={N}, dt={dt}: {path}")
        self.N, self.P = N, P
        self.h = lib().ref_create(path.encode(), N, int(cic), P)
        if not self.h:
            raise RuntimeError("reference runner: " + lib().ref_error().decode())

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference runner: " + lib().ref_error().decode())

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, s):
        f = lambda a: np.ascontiguousarray(a, np.float32)
        self._check(lib().ref_set_state(self.h, f(s.x), f(s.y), f(s.x_old), f(s.y_old), f(s.m)))

    def step(self, n: int = 1):
        self._check(lib().ref_step(self.h, n))

    def state(self):
        out = [np.empty(self.P, np.float32) for _ in range(4)]
        self._check(lib().ref_get_state(self.h, *out))
        return out

    def fields(self):
        N = self.N
        d = np.empty((N, N), np.float32)
        p = np.empty((N, N), np.float32)
        f = np.empty((N, N, 2), np.float32)
        self._check(lib().ref_get_fields(self.h, d, p, f))
        return d, p, f

    def render(self, density):
        """One display frame of `density` through the reference's render chain."""
        frame = np.empty((self.N, self.N), np.float32)
        self._check(lib().ref_render(self.h, np.ascontiguousarray(density, np.float32), frame))
        return frame

    def time_steps(self, n: int) -> float:
        ms = lib().ref_time_steps(self.h, n)
        if ms < 0:
            raise RuntimeError("reference runner: " + lib().ref_error().decode())
        return float(ms)
