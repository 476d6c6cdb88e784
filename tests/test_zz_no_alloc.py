"""The tile sort that allocates no device memory (cosmos_tile_sort_noalloc).

Some callers cannot allocate device memory while they run -- a host that owns
a fixed amount of device memory, code inside an allocator callback, a real-time render
loop where cudaMalloc may stall.  This entry point sorts caller-owned device
positions using a fixed scratch array built into the library.  Its permutation
must equal the one of the allocating sort (cosmos_pm_sort) bit for bit, on
consecutive calls that reuse the shared scratch.  Kept in its own file, which
pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from oracle import pm_oracle

pytestmark = pytest.mark.gpu


class _Cuda:
    def __init__(self):
        for name in ("libcudart.so.13", "libcudart.so", "libcudart.so.12"):
            try:
                self.L = ctypes.CDLL(name)
                break
            except OSError:
                continue
        L = self.L
        L.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        L.cudaFree.argtypes = [ctypes.c_void_p]
        L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        L.cudaDeviceSynchronize.argtypes = []

    def upload(self, a):
        p = ctypes.c_void_p()
        assert self.L.cudaMalloc(ctypes.byref(p), a.nbytes) == 0
        assert self.L.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1) == 0
        return p

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        assert self.L.cudaMalloc(ctypes.byref(p), nbytes) == 0
        return p

    def download(self, p, out):
        assert self.L.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), p, out.nbytes, 2) == 0
        return out


def _positions(seed, P, N):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2, N + 2, P).astype(np.float32)
    y = rng.uniform(-2, N + 2, P).astype(np.float32)
    x[: P // 4] = x[0]  # ties: stability matters
    return x, y


def test_noalloc_sort_matches_allocating_sort_twice(cosmos_lib):
    L = cosmos_lib.load()
    cu = _Cuda()
    N, gran = 1024, 5
    for call, P in enumerate((700_000, 1 << 20)):  # second call: different data, full capacity
        x, y = _positions(100 + call, P, N)
        # existing entry point: sort of a handle's state (identity order first)
        with cosmos_lib.Simulation(N, P, cic=True, sort_interval=0, sort_granularity=gran) as s:
            s.set_particles(x, y)
            expect = s.sort()
        dx, dy = cu.upload(x), cu.upload(y)
        dperm = cu.alloc(P * 4)
        try:
            rc = L.cosmos_tile_sort_noalloc(dx, dy, P, N, gran, dperm, 0)
            assert rc == 0, L.cosmos_pm_last_error(None).decode()
            assert cu.L.cudaDeviceSynchronize() == 0
            got = cu.download(dperm, np.empty(P, np.uint32))
        finally:
            for p in (dx, dy, dperm):
                cu.L.cudaFree(p)
        np.testing.assert_array_equal(got, expect)
        np.testing.assert_array_equal(got, pm_oracle.stable_sort_perm(pm_oracle.sort_keys(x, y, N, gran)))


def test_noalloc_sorts_every_particle_of_a_ragged_count(cosmos_lib):
    """n % 4 != 0: the no-alloc sort orders all n particles (the handle's sort
    leaves the last n % 4 in place), checked against the oracle's stable sort."""
    L = cosmos_lib.load()
    cu = _Cuda()
    N, gran, P = 1024, 5, 700_003
    x, y = _positions(7, P, N)
    dx, dy = cu.upload(x), cu.upload(y)
    dperm = cu.alloc(P * 4)
    try:
        rc = L.cosmos_tile_sort_noalloc(dx, dy, P, N, gran, dperm, 0)
        assert rc == 0, L.cosmos_pm_last_error(None).decode()
        assert cu.L.cudaDeviceSynchronize() == 0
        got = cu.download(dperm, np.empty(P, np.uint32))
    finally:
        for p in (dx, dy, dperm):
            cu.L.cudaFree(p)
    np.testing.assert_array_equal(got, pm_oracle.stable_sort_perm(pm_oracle.sort_keys(x, y, N, gran)))


def test_noalloc_rejects_oversize(cosmos_lib):
    L = cosmos_lib.load()
    rc = L.cosmos_tile_sort_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), cosmos_lib.NOALLOC_MAX_PARTICLES + 1,
                                    1024, 5, ctypes.c_void_p(16), 0)
    assert rc == -4
    assert b"capacity" in L.cosmos_pm_last_error(None)
