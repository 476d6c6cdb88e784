"""ctypes binding of the cosmos_pm C ABI (include/cosmos_pm.h).

The CUDA library is built in-tree (cosmossimulationwithcuda_gb300/libcosmos_pm.so,
see build.py).  Loading fails loudly when it is missing: there is no CPU
fallback for any part of the step.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcosmos_pm.so")

COSMOS_OK = 0
ERRORS = {-1: "INVALID", -2: "CUDA", -3: "NOMEM", -4: "RANGE", -5: "TIMEOUT", -6: "STATE"}
DEPOSIT_NGP, DEPOSIT_CIC = 0, 1
FORCE_GRADIENT, FORCE_SPECTRAL, FORCE_SPECTRAL_TC_FP16, FORCE_SPECTRAL_TC_BF16 = 0, 1, 2, 3
FIELD_DENSITY, FIELD_POTENTIAL, FIELD_FORCE = 0, 1, 2
STAGE_DEPOSIT, STAGE_POTENTIAL, STAGE_FORCE, STAGE_INTEGRATE = 0, 1, 2, 3
TEST_FAIL_ALLOC, TEST_TC_SKIP_MMA, TEST_COPY_WAIT = 1, 2, 3

# Every function include/cosmos_pm.h declares (checked by the CPU test suite).
EXPORTS = (
    "cosmos_pm_default_config", "cosmos_pm_create", "cosmos_pm_destroy", "cosmos_pm_set_particles",
    "cosmos_pm_get_particles", "cosmos_pm_clear", "cosmos_pm_step", "cosmos_pm_synchronize",
    "cosmos_pm_get_positions_async", "cosmos_pm_poll", "cosmos_pm_wait", "cosmos_pm_run_stage",
    "cosmos_pm_get_field", "cosmos_pm_set_field", "cosmos_pm_sort", "cosmos_pm_tile_keys",
    "cosmos_pm_diagnostics", "cosmos_pm_set_profiling", "cosmos_pm_stage_times", "cosmos_pm_stream",
    "cosmos_pm_launches_per_step", "cosmos_pm_kernels_launched", "cosmos_pm_last_error", "cosmos_pm_version",
    "cosmos_tile_sort_noalloc", "cosmos_pm_render_frame", "cosmos_pm_get_frame_async",
    "cosmos_pm_host_alloc", "cosmos_pm_host_free", "cosmos_pm_autotune", "cosmos_pm_generate",
    "cosmos_pm_checkpoint_save", "cosmos_pm_checkpoint_load", "cosmos_pm_steps_taken", "cosmos_pm_test_hook",
    "cosmos_ensemble_default_config", "cosmos_ensemble_create", "cosmos_ensemble_destroy",
    "cosmos_ensemble_set_particles", "cosmos_ensemble_get_particles", "cosmos_ensemble_step",
    "cosmos_ensemble_synchronize", "cosmos_ensemble_get_field", "cosmos_ensemble_launches_per_step",
    "cosmos_ensemble_stream", "cosmos_ensemble_last_error", "cosmos_ensemble_test_barrier",
)
NOALLOC_MAX_PARTICLES = 1 << 20


class Config(ctypes.Structure):
    _fields_ = [
        ("lattice_n", ctypes.c_int32),
        ("deposit", ctypes.c_int32),
        ("dt", ctypes.c_float),
        ("gravity_multiplier", ctypes.c_float),
        ("num_particles", ctypes.c_int64),
        ("device", ctypes.c_int32),
        ("force_mode", ctypes.c_int32),
        ("sort_interval", ctypes.c_int32),
        ("sort_granularity", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("blur_r", ctypes.c_int32),
        ("item_size", ctypes.c_int32),
        ("fused_ctas_per_sm", ctypes.c_int32),
        ("fft_shape", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 3),
    ]


IC_UNIFORM, IC_EXP_DISK, IC_PLUMMER, IC_RING_DISK = 0, 1, 2, 3


class IcParams(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("black_hole", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("center_x", ctypes.c_float),
        ("center_y", ctypes.c_float),
        ("scale", ctypes.c_float),
        ("rmax", ctypes.c_float),
        ("mass", ctypes.c_float),
        ("mass_sigma", ctypes.c_float),
        ("bulk_vx", ctypes.c_float),
        ("bulk_vy", ctypes.c_float),
        ("spin", ctypes.c_float),
        ("dispersion", ctypes.c_float),
        ("g", ctypes.c_float),
        ("pad", ctypes.c_int32),
        ("total_particles", ctypes.c_int64),
        ("reserved", ctypes.c_int32 * 4),
    ]


class EnsembleConfig(ctypes.Structure):
    _fields_ = [
        ("num_sims", ctypes.c_int32),
        ("deposit", ctypes.c_int32),
        ("dt", ctypes.c_float),
        ("gravity_multiplier", ctypes.c_float),
        ("device", ctypes.c_int32),
        ("force_mode", ctypes.c_int32),
        ("sort_interval", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("persistent_step", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 7),
    ]


class CosmosError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cosmos_pm error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None
_f32p = ctypes.POINTER(ctypes.c_float)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


def load(path: str | None = None):
    """Load libcosmos_pm.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("COSMOS_PM_LIBRARY") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"cosmos_pm CUDA library not built ({path}); run build() first")
    L = ctypes.CDLL(path)
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    sig = {
        "cosmos_pm_default_config": (None, [ctypes.POINTER(Config)]),
        "cosmos_pm_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_vp)]),
        "cosmos_pm_destroy": (ctypes.c_int, [_vp]),
        "cosmos_pm_set_particles": (ctypes.c_int, [_vp, _f32p, _f32p, _f32p, _f32p, _f32p, i64, i64]),
        "cosmos_pm_get_particles": (ctypes.c_int, [_vp, _f32p, _f32p, _f32p, _f32p, _f32p, i64, i64]),
        "cosmos_pm_clear": (ctypes.c_int, [_vp]),
        "cosmos_pm_step": (ctypes.c_int, [_vp, i32]),
        "cosmos_pm_synchronize": (ctypes.c_int, [_vp]),
        "cosmos_pm_get_positions_async": (ctypes.c_int, [_vp, _f32p, _f32p, i32, ctypes.POINTER(ctypes.c_uint64)]),
        "cosmos_pm_poll": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.POINTER(i32)]),
        "cosmos_pm_wait": (ctypes.c_int, [_vp, ctypes.c_uint64]),
        "cosmos_pm_run_stage": (ctypes.c_int, [_vp, i32]),
        "cosmos_pm_get_field": (ctypes.c_int, [_vp, i32, _f32p]),
        "cosmos_pm_set_field": (ctypes.c_int, [_vp, i32, _f32p]),
        "cosmos_pm_sort": (ctypes.c_int, [_vp, _u32p]),
        "cosmos_pm_tile_keys": (ctypes.c_int, [_vp, _f32p, _f32p, i64, i32, _u32p]),
        "cosmos_pm_diagnostics": (ctypes.c_int, [_vp, _f64p, _f64p, _f64p, _f64p]),
        "cosmos_pm_set_profiling": (ctypes.c_int, [_vp, i32]),
        "cosmos_pm_stage_times": (ctypes.c_int, [_vp, _f32p, ctypes.POINTER(i32)]),
        "cosmos_pm_stream": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64)]),
        "cosmos_pm_launches_per_step": (ctypes.c_int, [_vp, ctypes.POINTER(i32)]),
        "cosmos_pm_kernels_launched": (ctypes.c_int, [_vp, ctypes.POINTER(i64)]),
        "cosmos_pm_last_error": (ctypes.c_char_p, [_vp]),
        "cosmos_pm_version": (ctypes.c_char_p, []),
        "cosmos_tile_sort_noalloc": (ctypes.c_int, [_vp, _vp, i64, i32, i32, _vp, ctypes.c_uint64]),
        "cosmos_pm_render_frame": (ctypes.c_int, [_vp, _f32p]),
        "cosmos_pm_get_frame_async": (ctypes.c_int, [_vp, _f32p, ctypes.POINTER(ctypes.c_uint64)]),
        "cosmos_pm_host_alloc": (ctypes.c_int, [i64, ctypes.POINTER(_vp)]),
        "cosmos_pm_host_free": (ctypes.c_int, [_vp]),
        "cosmos_pm_generate": (ctypes.c_int, [_vp, ctypes.POINTER(IcParams), i64, i64]),
        "cosmos_pm_checkpoint_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "cosmos_pm_checkpoint_load": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "cosmos_pm_steps_taken": (ctypes.c_int, [_vp, ctypes.POINTER(i64)]),
        "cosmos_pm_test_hook": (ctypes.c_int, [_vp, i32, i64]),
        "cosmos_pm_autotune": (ctypes.c_int, [ctypes.POINTER(Config), _f32p, _f32p, _f32p, _f32p, _f32p, i32,
                                              ctypes.c_char_p, ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_float)]),
        "cosmos_ensemble_default_config": (None, [ctypes.POINTER(EnsembleConfig)]),
        "cosmos_ensemble_create": (ctypes.c_int, [ctypes.POINTER(EnsembleConfig), ctypes.POINTER(i32),
                                                  ctypes.POINTER(i64), ctypes.POINTER(_vp)]),
        "cosmos_ensemble_destroy": (ctypes.c_int, [_vp]),
        "cosmos_ensemble_set_particles": (ctypes.c_int, [_vp, i32, _f32p, _f32p, _f32p, _f32p, _f32p, i64, i64]),
        "cosmos_ensemble_get_particles": (ctypes.c_int, [_vp, i32, _f32p, _f32p, _f32p, _f32p, _f32p, i64, i64]),
        "cosmos_ensemble_step": (ctypes.c_int, [_vp, i32]),
        "cosmos_ensemble_synchronize": (ctypes.c_int, [_vp]),
        "cosmos_ensemble_get_field": (ctypes.c_int, [_vp, i32, i32, _f32p]),
        "cosmos_ensemble_launches_per_step": (ctypes.c_int, [_vp, ctypes.POINTER(i32)]),
        "cosmos_ensemble_stream": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64)]),
        "cosmos_ensemble_last_error": (ctypes.c_char_p, [_vp]),
        "cosmos_ensemble_test_barrier": (ctypes.c_int, [_vp, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a, ctype=_f32p):
    if a is None:
        return None
    return a.ctypes.data_as(ctype)


def default_config(**kw) -> Config:
    c = Config()
    load().cosmos_pm_default_config(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def autotune(state, N: int, cic: bool = True, dt: float = 1e-3, gravity_multiplier: float = 1.0, device: int = 0,
             force_mode: int = FORCE_SPECTRAL, steps: int = 128, cache_path: str | None = None):
    """Fastest launch shapes for this state, measured on the device
    (cosmos_pm_autotune).  Returns ({sort_granularity, sort_interval,
    item_size, fused_ctas_per_sm, fft_shape}, ms_per_step)."""
    L = load()
    arrs = [np.ascontiguousarray(a, np.float32) for a in (state.x, state.y, state.x_old, state.y_old, state.m)]
    base = default_config(lattice_n=N, deposit=DEPOSIT_CIC if cic else DEPOSIT_NGP, dt=dt,
                          gravity_multiplier=gravity_multiplier, num_particles=arrs[0].size, device=device,
                          force_mode=force_mode)
    best = Config()
    ms = ctypes.c_float()
    rc = L.cosmos_pm_autotune(ctypes.byref(base), *[_ptr(a) for a in arrs], steps,
                              cache_path.encode() if cache_path else None, ctypes.byref(best), ctypes.byref(ms))
    if rc != COSMOS_OK:
        raise CosmosError(rc, L.cosmos_pm_last_error(None).decode())
    fields = ("sort_granularity", "sort_interval", "item_size", "fused_ctas_per_sm", "fft_shape")
    return {f: int(getattr(best, f)) for f in fields}, ms.value


class Simulation:
    """One particle-mesh simulation on one GPU, driven through the C ABI.

    Mirrors the reference Universe<K> (CosmosCuda.cuh:830-1428): construction
    builds the filter, set_particles uploads state (constructor / addGalaxy
    uploads), clear() parks every particle, step() enqueues steps."""

    def __init__(self, N: int, P: int, cic: bool = True, dt: float = 1e-3, gravity_multiplier: float = 1.0,
                 device: int = 0, force_mode: int = FORCE_GRADIENT, sort_interval: int = -1,
                 sort_granularity: int = -1, use_graph: bool = True, blur_r: int = 3, item_size: int = 0,
                 fused_ctas_per_sm: int = 0, fft_shape: int = 0):
        self.L = load()
        self.cfg = default_config(lattice_n=N, deposit=DEPOSIT_CIC if cic else DEPOSIT_NGP, dt=dt,
                                  gravity_multiplier=gravity_multiplier, num_particles=P, device=device,
                                  force_mode=force_mode, sort_interval=sort_interval,
                                  sort_granularity=sort_granularity, use_graph=int(use_graph), blur_r=blur_r,
                                  item_size=item_size, fused_ctas_per_sm=fused_ctas_per_sm, fft_shape=fft_shape)
        h = _vp()
        rc = self.L.cosmos_pm_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if rc != COSMOS_OK:
            raise CosmosError(rc, self.L.cosmos_pm_last_error(None).decode())
        self.h = h
        self.N, self.P, self.cic, self.dt = N, P, cic, dt

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.cosmos_pm_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != COSMOS_OK:
            raise CosmosError(rc, self.L.cosmos_pm_last_error(self.h).decode())

    # -- particle state -------------------------------------------------------
    def set_particles(self, x, y, x_old=None, y_old=None, m=None, offset: int = 0):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (x, y, x_old, y_old, m)]
        n = arrs[0].size
        self._check(self.L.cosmos_pm_set_particles(self.h, *[_ptr(a) for a in arrs], n, offset))

    def set_state(self, s):
        self.set_particles(s.x, s.y, s.x_old, s.y_old, s.m)

    def get_particles(self, count: int | None = None, offset: int = 0):
        count = self.P - offset if count is None else count
        out = [np.empty(count, np.float32) for _ in range(5)]
        self._check(self.L.cosmos_pm_get_particles(self.h, *[_ptr(a) for a in out], count, offset))
        return out

    def clear(self):
        self._check(self.L.cosmos_pm_clear(self.h))

    def save(self, path: str):
        self._check(self.L.cosmos_pm_checkpoint_save(self.h, path.encode()))

    def load(self, path: str):
        self._check(self.L.cosmos_pm_checkpoint_load(self.h, path.encode()))

    def steps_taken(self) -> int:
        n = ctypes.c_int64()
        self._check(self.L.cosmos_pm_steps_taken(self.h, ctypes.byref(n)))
        return n.value

    def test_hook(self, hook: int, value: int):
        self._check(self.L.cosmos_pm_test_hook(self.h, hook, value))

    def generate(self, kind: int, count: int, offset: int = 0, **params):
        """Seeded initial conditions on the device (cosmos_pm_generate); params
        are the fields of cosmos_ic_params (seed, center_x, scale, ...)."""
        ic = IcParams(kind=kind, g=1.0)
        for k, v in params.items():
            setattr(ic, k, int(v) if k in ("black_hole", "seed", "total_particles") else v)
        self._check(self.L.cosmos_pm_generate(self.h, ctypes.byref(ic), count, offset))

    # -- stepping -------------------------------------------------------------
    def step(self, n: int = 1):
        self._check(self.L.cosmos_pm_step(self.h, n))

    def synchronize(self):
        self._check(self.L.cosmos_pm_synchronize(self.h))

    def positions_async(self, hx, hy, ordered: bool = True) -> int:
        t = ctypes.c_uint64()
        self._check(self.L.cosmos_pm_get_positions_async(self.h, _ptr(hx), _ptr(hy), int(ordered), ctypes.byref(t)))
        return t.value

    def poll(self, ticket: int) -> bool:
        d = ctypes.c_int32()
        self._check(self.L.cosmos_pm_poll(self.h, ticket, ctypes.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int):
        self._check(self.L.cosmos_pm_wait(self.h, ticket))

    # -- stages and fields ----------------------------------------------------
    def render_frame(self):
        out = np.empty((self.N, self.N), np.float32)
        self._check(self.L.cosmos_pm_render_frame(self.h, _ptr(out)))
        return out

    def frame_async(self, host_frame) -> int:
        t = ctypes.c_uint64()
        self._check(self.L.cosmos_pm_get_frame_async(self.h, _ptr(host_frame), ctypes.byref(t)))
        return t.value

    def run_stage(self, stage: int):
        self._check(self.L.cosmos_pm_run_stage(self.h, stage))

    def get_field(self, field: int):
        shape = (self.N, self.N, 2) if field == FIELD_FORCE else (self.N, self.N)
        out = np.empty(shape, np.float32)
        self._check(self.L.cosmos_pm_get_field(self.h, field, _ptr(out)))
        return out

    def set_field(self, field: int, a):
        a = np.ascontiguousarray(a, np.float32)
        self._check(self.L.cosmos_pm_set_field(self.h, field, _ptr(a)))

    def sort(self):
        perm = np.empty(self.P, np.uint32)
        self._check(self.L.cosmos_pm_sort(self.h, _ptr(perm, _u32p)))
        return perm

    def tile_keys(self, x, y, granularity: int):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        keys = np.empty(x.size, np.uint32)
        self._check(self.L.cosmos_pm_tile_keys(self.h, _ptr(x), _ptr(y), x.size, granularity, _ptr(keys, _u32p)))
        return keys

    def diagnostics(self):
        v = [ctypes.c_double() for _ in range(4)]
        self._check(self.L.cosmos_pm_diagnostics(self.h, *[ctypes.byref(a) for a in v]))
        return tuple(a.value for a in v)

    def set_profiling(self, on: bool):
        self._check(self.L.cosmos_pm_set_profiling(self.h, int(on)))

    def stage_times(self):
        t = np.zeros(8, np.float32)
        n = ctypes.c_int32(8)
        self._check(self.L.cosmos_pm_stage_times(self.h, _ptr(t), ctypes.byref(n)))
        return t[: n.value]

    def stream(self) -> int:
        s = ctypes.c_uint64()
        self._check(self.L.cosmos_pm_stream(self.h, ctypes.byref(s)))
        return s.value

    def launches_per_step(self) -> int:
        n = ctypes.c_int32()
        self._check(self.L.cosmos_pm_launches_per_step(self.h, ctypes.byref(n)))
        return n.value

    def kernels_launched(self) -> int:
        """Kernels enqueued since creation (steps, sorts, prologue deposits, renders)."""
        n = ctypes.c_int64()
        self._check(self.L.cosmos_pm_kernels_launched(self.h, ctypes.byref(n)))
        return n.value


def version() -> str:
    return load().cosmos_pm_version().decode()


class Ensemble:
    """Many independent simulations stepped together (include/cosmos_ensemble.h).

    lattice_n[s], num_particles[s] per simulation (P_s a multiple of 4); one
    dt, deposit, gravity multiplier and force mode for all."""

    def __init__(self, lattice_n, num_particles, cic: bool = True, dt: float = 1e-3, gravity_multiplier: float = 1.0,
                 device: int = 0, force_mode: int = FORCE_SPECTRAL, sort_interval: int = 32, use_graph: bool = True,
                 persistent: bool = False):
        self.L = load()
        ns = np.ascontiguousarray(lattice_n, np.int32)
        ps = np.ascontiguousarray(num_particles, np.int64)
        if ns.shape != ps.shape or ns.ndim != 1:
            raise ValueError("lattice_n and num_particles must be 1-D of equal length")
        cfg = EnsembleConfig()
        self.L.cosmos_ensemble_default_config(ctypes.byref(cfg))
        cfg.num_sims = ns.size
        cfg.deposit = DEPOSIT_CIC if cic else DEPOSIT_NGP
        cfg.dt = dt
        cfg.gravity_multiplier = gravity_multiplier
        cfg.device = device
        cfg.force_mode = force_mode
        cfg.sort_interval = sort_interval
        cfg.use_graph = int(use_graph)
        cfg.persistent_step = int(persistent)
        self.cfg = cfg
        h = _vp()
        rc = self.L.cosmos_ensemble_create(ctypes.byref(cfg), ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                           ps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.byref(h))
        if rc != COSMOS_OK:
            raise CosmosError(rc, self.L.cosmos_ensemble_last_error(None).decode())
        self.h = h
        self.N = [int(n) for n in ns]
        self.P = [int(p) for p in ps]

    def close(self):
        if getattr(self, "h", None):
            self.L.cosmos_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != COSMOS_OK:
            raise CosmosError(rc, self.L.cosmos_ensemble_last_error(self.h).decode())

    def set_particles(self, sim: int, x, y, x_old=None, y_old=None, m=None, offset: int = 0):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (x, y, x_old, y_old, m)]
        self._check(self.L.cosmos_ensemble_set_particles(self.h, sim, *[_ptr(a) for a in arrs], arrs[0].size, offset))

    def set_state(self, sim: int, s):
        self.set_particles(sim, s.x, s.y, s.x_old, s.y_old, s.m)

    def get_particles(self, sim: int, count: int | None = None, offset: int = 0):
        count = self.P[sim] - offset if count is None else count
        out = [np.empty(count, np.float32) for _ in range(5)]
        self._check(self.L.cosmos_ensemble_get_particles(self.h, sim, *[_ptr(a) for a in out], count, offset))
        return out

    def step(self, n: int = 1):
        self._check(self.L.cosmos_ensemble_step(self.h, n))

    def synchronize(self):
        self._check(self.L.cosmos_ensemble_synchronize(self.h))

    def get_field(self, sim: int, field: int):
        N = self.N[sim]
        out = np.empty((N, N, 2) if field == FIELD_FORCE else (N, N), np.float32)
        self._check(self.L.cosmos_ensemble_get_field(self.h, sim, field, _ptr(out)))
        return out

    def test_barrier(self, value: int):
        """Test hook of the persistent step: one CTA skips its first grid-barrier arrival."""
        self._check(self.L.cosmos_ensemble_test_barrier(self.h, value))

    def launches_per_step(self) -> int:
        n = ctypes.c_int32()
        self._check(self.L.cosmos_ensemble_launches_per_step(self.h, ctypes.byref(n)))
        return n.value

    def stream(self) -> int:
        s = ctypes.c_uint64()
        self._check(self.L.cosmos_ensemble_stream(self.h, ctypes.byref(s)))
        return s.value


def test_hook(hook: int, value: int):
    """Library-wide test hook (cosmos_pm_test_hook with no handle)."""
    rc = load().cosmos_pm_test_hook(None, hook, value)
    if rc != COSMOS_OK:
        raise CosmosError(rc, load().cosmos_pm_last_error(None).decode())
