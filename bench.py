#!/usr/bin/env python3
"""Benchmark of the particle-mesh step on the 20M-particle / 2048^2 CIC disk.

One step = deposit -> FFT convolution -> force -> gather + update over all
20,000,000 particles (the drop-in headline workload: exponential disk of scale
length 200 cells at the lattice centre, circular velocities from the enclosed
mass plus 5% dispersion, lognormal(0, 0.3) masses, dt = 0.001).  Inputs are
seeded synthetic data of that shape.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line.  `value` is device-timed throughput (particle-steps/s)
with the state resident in HBM; `e2e` is the same metric through the C ABI
with host buffers: the state uploaded from page-locked host memory inside the
timed region and the step's output -- the display frame, as the reference's
worker delivers it -- read back to page-locked host memory every
--render-interval steps (2, the render cadence of the reference demo);
`e2e_positions` reads the positions back instead.  --impl reference times the
reference algorithm on the host cores (the CPU restatement of
CosmosCuda.cuh's step; the reference itself has no CPU step).  With N > 1
(torchrun) every rank runs an independent replica (the step is not sharded
across GPUs).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @20M, 2048²: plain FP32 vs TC split-FFT at ≤1e-5 rel force err"
UNIT = "particle-steps/s"
WORKLOAD = "disk-20M-2048-cic"


# ---- small cudart helper (events on the library's stream, pinned memory) ----------------
class CudaRT:
    def __init__(self):
        self.lib = None
        for name in ("libcudart.so.13", "libcudart.so", "libcudart.so.12"):
            try:
                self.lib = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if self.lib is None:
            raise RuntimeError("libcudart not found")
        L = self.lib
        L.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        L.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
        L.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
        L.cudaEventDestroy.argtypes = [ctypes.c_void_p]
        L.cudaHostRegister.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint]
        L.cudaHostUnregister.argtypes = [ctypes.c_void_p]
        L.cudaSetDevice.argtypes = [ctypes.c_int]
        L.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        L.cudaFree.argtypes = [ctypes.c_void_p]
        L.cudaMemsetAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]

    def event(self):
        e = ctypes.c_void_p()
        assert self.lib.cudaEventCreate(ctypes.byref(e)) == 0
        return e

    def record(self, e, stream):
        assert self.lib.cudaEventRecord(e, ctypes.c_void_p(stream)) == 0

    def elapsed_ms(self, a, b):
        assert self.lib.cudaEventSynchronize(b) == 0
        t = ctypes.c_float()
        assert self.lib.cudaEventElapsedTime(ctypes.byref(t), a, b) == 0
        return t.value

    def pin(self, arr):
        rc = self.lib.cudaHostRegister(ctypes.c_void_p(arr.ctypes.data), arr.nbytes, 0)
        if rc != 0:
            raise RuntimeError(f"cudaHostRegister failed ({rc})")

    def unpin(self, arr):
        self.lib.cudaHostUnregister(ctypes.c_void_p(arr.ctypes.data))

    def destroy(self, e):
        self.lib.cudaEventDestroy(e)


# Device time of at least this much per timed region: the re-sorts (every 32
# steps by default) fall inside it at their own cadence, and the clock sampler
# (one reading per 50 ms) sees the GPU under load.
MIN_TIMED_MS = 500.0


def timed_windows(rt, stream, run, steps: int, min_ms: float = MIN_TIMED_MS, max_windows: int = 5000):
    """Device times (ms) of back-to-back windows of exactly `steps` steps,
    each bracketed by CUDA events on the library's stream, until the windows
    add up to at least `min_ms`.  `run(k)` enqueues k steps.  The first window
    sizes the rest, which are enqueued without a host wait between them."""
    a, b = rt.event(), rt.event()
    rt.record(a, stream)
    run(steps)
    rt.record(b, stream)
    first = rt.elapsed_ms(a, b)
    rt.destroy(a)
    rt.destroy(b)
    more = 0 if first >= min_ms else int(min(max_windows - 1, math.ceil((min_ms - first) / max(first, 1e-3))))
    evs = [rt.event() for _ in range(more + 1)]
    rt.record(evs[0], stream)
    for i in range(more):
        run(steps)
        rt.record(evs[i + 1], stream)
    times = [first] + [rt.elapsed_ms(evs[i], evs[i + 1]) for i in range(more)]
    for e in evs:
        rt.destroy(e)
    return times


# ---- clocks sampled during the timed region ----------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout: float = 5.0):
        """Block until the sampler has produced its first line (it starts slowly)."""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.02)
        self.skip = len(self.lines)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[getattr(self, "skip", 0):]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_traffic(kernel: str, P: int):
    """DRAM bytes per launch of `kernel` from the committed ncu capture
    (profiles/traffic.json), scaled to P particles; None when not captured."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            rec = json.load(f)[kernel]
        return float(rec["dram_bytes_per_particle"]) * P
    except (OSError, KeyError, ValueError):
        return None


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---- CPU baseline: the reference algorithm restated on the host cores ---------------------
def cpu_baseline(state, N, cic, dt, seconds: float, min_steps: int = 2):
    from oracle import pm_oracle
    threads = os.cpu_count() or 1
    pm_oracle.set_threads(threads)
    o = pm_oracle.OraclePM(N, cic, dt, 1.0, fp64=False)
    s = state.copy()
    o.step(s.x, s.y, s.x_old, s.y_old, s.m, 1)  # warm-up (page-in, thread pool)
    n = 0
    t0 = time.perf_counter()
    while n < min_steps or (time.perf_counter() - t0) < seconds:
        o.step(s.x, s.y, s.x_old, s.y_old, s.m, 1)
        n += 1
    dt_s = time.perf_counter() - t0
    o.close()
    return {"value": state.count * n / dt_s, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} full steps of the {state.count}-particle {N}^2 {'CIC' if cic else 'NGP'} workload "
                      f"(FP32 restatement of the reference step, OpenMP over {threads} threads)"}


def _cic_sample(F, x, y, N):
    """Bilinear (CIC) sample of a force field at active particle positions, in
    the reference's gather weights (CosmosCuda.cuh:263-278)."""
    cx = np.trunc(x).astype(np.int64)
    cy = np.trunc(y).astype(np.int64)
    act = (cx >= 1) & (cx < N - 1) & (cy >= 1) & (cy < N - 1)
    cx, cy = cx[act], cy[act]
    fx = x[act].astype(np.float64) - cx
    fy = y[act].astype(np.float64) - cy
    Ff = F.reshape(N * N, 2).astype(np.float64)
    c = cx + cy * N
    return (Ff[c] * ((1 - fx) * (1 - fy))[:, None] + Ff[c + 1] * (fx * (1 - fy))[:, None]
            + Ff[c + N] * ((1 - fx) * fy)[:, None] + Ff[c + N + 1] * (fx * fy)[:, None])


def force_error_vs_fp64(state, N, cic, dt, F_gpu):
    """Relative L2 error of the GPU force against the FP64 oracle on the same
    positions: over the lattice, and sampled at the particles."""
    from oracle import pm_oracle
    pm_oracle.set_threads(os.cpu_count() or 1)
    o = pm_oracle.OraclePM(N, cic, dt, 1.0, fp64=True)
    o.deposit(state.x, state.y, state.m)
    o.potential()
    o.gradient()
    ref = o.force()
    o.close()
    lattice = float(np.linalg.norm(F_gpu - ref) / np.linalg.norm(ref))
    a = _cic_sample(F_gpu, state.x, state.y, N)
    b = _cic_sample(ref, state.x, state.y, N)
    particles = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return {"particles": particles, "lattice": lattice, "reference": "FP64 oracle (CPU) on the same positions"}


def force_error_series(sim, N, cic, dt, k: int):
    """Force error of k consecutive steps, each against FP64 on the GPU's own
    positions (fused_force_error per step): the first step's record, with the
    per-step series of all k under "series"."""
    errs = [fused_force_error(sim, N, cic, dt) for _ in range(max(1, k))]
    out = dict(errs[0])
    if len(errs) > 1:
        out["series"] = {"after_steps": [int(e["positions"].split(" steps")[0].split("after ")[-1]) for e in errs],
                         "particles": [e["particles"] for e in errs], "lattice": [e["lattice"] for e in errs],
                         "max_particles": max(e["particles"] for e in errs),
                         "max_lattice": max(e["lattice"] for e in errs)}
    return out


def fused_force_error(sim, N, cic, dt):
    """Force error of the path as it runs: the positions are read back after
    the steps taken so far, one more step is run, and the force field that step
    used (computed from the density the fused step kernel deposited for those
    positions) is compared with the FP64 oracle's force of the same positions."""
    from cosmossimulationwithcuda_gb300 import _lib, ics
    sim.synchronize()
    gx, gy, _, _, gm = sim.get_particles()
    sim.step(1)
    sim.synchronize()
    err = force_error_vs_fp64(ics.ParticleState(gx, gy, gx, gy, gm), N, cic, dt, sim.get_field(_lib.FIELD_FORCE))
    err["positions"] = (f"GPU positions after {sim.steps_taken() - 1} steps; the force of the next step, from the "
                        f"density the fused step kernel deposited")
    return err


IC_TEXT = {
    "disk-20M-2048-cic": "exponential disk, scale 200 cells, v_c from enclosed mass + 5% dispersion, "
                         "lognormal(0,0.3) masses",
    "uniform-1M-512-ngp": "uniform on the lattice, zero velocity, unit masses",
    "collide-100M-4096-cic": "two counter-rotating exponential disks (scale 300), approaching",
    "clumpy-1B-8192-cic": "uniform background + 32 Plummer clumps (a = 40 cells, 2% of the mass each), at rest",
}


def run_ensemble(args, ws, rank, local):
    """The 64-simulation ensemble: device-timed steps of all simulations,
    particle-steps/s summed over the simulations.  Both forms of the step are
    timed (one graph of per-pass kernels per step; one persistent cooperative
    launch per step) and the faster one is reported, the other beside it."""
    from cosmossimulationwithcuda_gb300 import _build, _lib, ics
    e = ics.ENSEMBLE
    Ns, Ps, states = ics.ensemble_workload()
    Ptot = int(sum(Ps))
    _build.build()
    rt = CudaRT()
    rt.lib.cudaSetDevice(local)
    mode = {"spectral": _lib.FORCE_SPECTRAL, "gradient": _lib.FORCE_GRADIENT, "tc-fp16": _lib.FORCE_SPECTRAL_TC_FP16,
            "tc-bf16": _lib.FORCE_SPECTRAL_TC_BF16}[args.force_mode]
    def timed_form(persistent: bool):
        """Device-timed steps of one form of the ensemble step: one graph of
        per-pass kernels per step, or one persistent cooperative launch."""
        ens = _lib.Ensemble(Ns, Ps, cic=e["cic"], dt=e["dt"], device=local, force_mode=mode,
                            sort_interval=args.sort_interval if args.sort_interval > 0 else 32, persistent=persistent)
        for i, st in enumerate(states):
            ens.set_state(i, st)
        ens.step(args.warmup)
        ens.synchronize()
        barrier(ws)
        win = timed_windows(rt, ens.stream(), ens.step, steps, min_ms=args.min_timed_ms)
        ens.synchronize()
        per = ens.launches_per_step()
        return ens, max_over_ranks(sum(win) / (steps * len(win)), ws), steps * len(win), per

    steps = args.steps
    forms = {}
    persistent_ok = mode == _lib.FORCE_SPECTRAL and all(128 <= n <= 1024 for n in Ns)
    clk = ClockSampler(local).__enter__()
    clk.wait_first()
    try:
        for persistent in ((False, True) if persistent_ok else (False,)):
            ens_f, ms_f, tsteps_f, per_f = timed_form(persistent)
            forms["persistent" if persistent else "graph"] = (ens_f, ms_f, tsteps_f, per_f)
    finally:
        clk.__exit__()
    best = min(forms, key=lambda k: forms[k][1])
    for k, v in forms.items():
        if k != best:
            v[0].close()
    ens, ms_step, timed_steps, per_step = forms[best]
    launches = per_step * timed_steps
    form_times = {k: {"ms_per_step": v[1], "launches_per_step": v[3], "value": Ptot / (v[1] / 1e3)}
                  for k, v in forms.items()}
    # whole-step algorithmic bytes: fused step 36 B/particle + 12 B/cell, density clear (memset) 4 B/cell;
    # force passes 37 B/cell (spectral:
    # FFT passes; gradient: 25 B/cell of FFT passes + 12 B/cell of stencil)
    cells = float(sum(n * n for n in Ns))
    algo = 36.0 * Ptot + (16.0 + 37.0) * cells
    peak, peak_kind = measured_peak_gbs()
    achieved = algo / (ms_step / 1e3) / 1e9
    # end to end: upload every simulation's state from page-locked memory, step, read positions back
    host = [st.copy() for st in states]
    pinned = [a for st in host for a in (st.x, st.y, st.x_old, st.y_old, st.m)]
    for a in pinned:
        rt.pin(a)
    e2e_steps = min(steps, 50)
    t0 = time.perf_counter()
    for i, st in enumerate(host):
        ens.set_state(i, st)
    ens.step(e2e_steps)
    outs = [ens.get_particles(i, count=None)[:2] for i in range(len(Ns))]
    t1 = time.perf_counter()
    for a in pinned:
        rt.unpin(a)
    ens.close()
    del outs
    cb = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # the reference algorithm on the host cores for the largest simulation (bounded sample)
        j = int(np.argmax(Ps))
        cb = cpu_baseline(states[j], Ns[j], e["cic"], e["dt"], args.cpu_seconds)
        cb["sample"] = "simulation %d of the ensemble (N=%d, P=%d): " % (j, Ns[j], Ps[j]) + cb["sample"]
    if rank != 0:
        return
    value = Ptot * ws / (ms_step / 1e3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps, "warmup": args.warmup,
            "timed_steps": timed_steps, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": e["name"], "sims": len(Ns), "particles_total": Ptot,
                       "lattices": {str(n): int(sum(1 for m in Ns if m == n)) for n in sorted(set(Ns))},
                       "p_min": int(min(Ps)), "p_max": int(max(Ps)), "deposit": "CIC", "dt": e["dt"],
                       "force_mode": args.force_mode, "ic": "alternating binary (2 Plummer, 1:0.6) / exponential disk",
                       "l2": f"particle state {20 * Ptot / 1e6:.0f} MB exceeds the 126 MB L2"},
            "roofline": {"bound": "hbm", "kernel": "whole ensemble step", "achieved": round(achieved, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": algo, "traffic": None},
            "cpu_baseline": cb,
            "e2e": {"value": Ptot * e2e_steps / (t1 - t0), "unit": UNIT,
                    "h2d_bytes_per_step": int(20 * Ptot / e2e_steps), "d2h_bytes_per_step": int(20 * Ptot / e2e_steps),
                    "note": f"all states uploaded from page-locked memory, {e2e_steps} steps, all particles read back"},
            "clocks": clk.summary(), "gpu_launches": launches, "step_forms": form_times, "step_form": best}
    print(json.dumps(line), flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws: int):
    """All ranks meet here (no-op for one rank)."""
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, ws: int) -> float:
    """The largest `value` of all ranks (the timed region's wall time: the job
    is as slow as its slowest replica)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--particles", type=int, default=None, help="override the particle count (testing)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="seconds of CPU baseline work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort-interval", type=int, default=-1)
    ap.add_argument("--force-mode", choices=["spectral", "gradient", "tc-fp16", "tc-bf16"], default="spectral",
                    help="spectral: force from the FFT (<=1e-5 vs FP64); gradient: the reference's FP32 stencil; "
                         "tc-fp16 / tc-bf16: spectral with the column FFTs on the tensor cores (split precision)")
    ap.add_argument("--no-force-check", action="store_true", help="skip the FP64 force-accuracy check")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip timing the reference's kernels")
    ap.add_argument("--ref-steps", type=int, default=200)
    ap.add_argument("--ref-arm-seconds", type=float, default=120.0,
                    help="--impl reference: at most this many seconds of timed host steps")
    ap.add_argument("--render-interval", type=int, default=2,
                    help="e2e: read the positions back every this many steps")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the launch shapes (sort tile edge and cadence, work-item size, fused-kernel CTAs "
                         "per SM, column-pass shape) with cosmos_pm_autotune on this state first")
    ap.add_argument("--no-tc-compare", action="store_true",
                    help="skip the tensor-core split-FFT comparison run of the headline metric")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end runs through host buffers")
    ap.add_argument("--min-timed-ms", type=float, default=MIN_TIMED_MS,
                    help="device time the timed windows add up to at least (0: one window of --steps)")
    ap.add_argument("--precision-steps", type=int, default=3,
                    help="steps whose force is compared with FP64 after the timed region, per force form")
    ap.add_argument("--workload", default=WORKLOAD,
                    help="the headline disk (default), another single-simulation workload "
                         "(uniform-1M-512-ngp, collide-100M-4096-cic, clumpy-1B-8192-cic) or "
                         "ensemble-64-mixed-cic")
    args = ap.parse_args()

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    from cosmossimulationwithcuda_gb300 import ics

    if args.workload == ics.ENSEMBLE["name"]:
        return run_ensemble(args, ws, rank, local)
    if args.workload not in ics.WORKLOADS:
        raise SystemExit(f"unknown workload {args.workload}")
    w = ics.WORKLOADS[args.workload]
    N, cic, dt = w["N"], w["cic"], w["dt"]
    P = args.particles or w["P"]
    state = ics.make_workload(args.workload, P)
    config = {"workload": args.workload, "particles": P, "lattice": N, "deposit": "CIC" if cic else "NGP", "dt": dt,
              "ic": IC_TEXT[args.workload],
              "l2": f"particle state ({20 * P / 1e6:.0f} MB at 20 B/particle) and lattice fields "
                    f"({70 * N * N / 2048 ** 2:.0f} MB) against the 126 MB L2"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference arm: W warm-up and K timed full steps of the workload on
        # the host cores (fewer timed steps when K of them would take longer
        # than --ref-arm-seconds; `steps` is the count actually timed)
        from oracle import pm_oracle
        threads = os.cpu_count() or 1
        pm_oracle.set_threads(threads)
        o = pm_oracle.OraclePM(N, cic, dt, 1.0, fp64=False)
        s = state.copy()
        t0 = time.perf_counter()
        nw = 0
        while nw < max(1, args.warmup) and (nw == 0 or time.perf_counter() - t0 < 30.0):
            o.step(s.x, s.y, s.x_old, s.y_old, s.m, 1)
            nw += 1
        t_step = (time.perf_counter() - t0) / nw
        k = int(max(1, min(args.steps, args.ref_arm_seconds // max(t_step, 1e-9))))
        t0 = time.perf_counter()
        o.step(s.x, s.y, s.x_old, s.y_old, s.m, k)
        el = time.perf_counter() - t0
        o.close()
        v = P * k / el
        cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
              "sample": f"{k} full steps of the {P}-particle {N}^2 {'CIC' if cic else 'NGP'} workload after {nw} "
                        f"warm-up steps (FP32 restatement of the reference step, OpenMP over {threads} threads)"}
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": k, "steps_requested": args.steps, "warmup": nw, "ms_per_step": el / k * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded)", "config": config, "cpu_baseline": cb,
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from cosmossimulationwithcuda_gb300 import _build, _lib
    _build.build()
    rt = CudaRT()
    rt.lib.cudaSetDevice(local)
    mode = {"spectral": _lib.FORCE_SPECTRAL, "gradient": _lib.FORCE_GRADIENT, "tc-fp16": _lib.FORCE_SPECTRAL_TC_FP16,
            "tc-bf16": _lib.FORCE_SPECTRAL_TC_BF16}[args.force_mode]
    shape = {"sort_interval": args.sort_interval, "sort_granularity": -1}
    if args.autotune:
        cache = os.environ.get("COSMOS_PM_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "cosmos_pm",
                                                                     "autotune.txt"))
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        t0 = time.perf_counter()
        chosen, tms = _lib.autotune(state, N, cic=cic, dt=dt, device=local, force_mode=mode, steps=256,
                                    cache_path=cache)
        shape = dict(chosen)
        if not shape["sort_interval"]:
            shape["sort_granularity"] = -1
        config["autotune"] = dict(chosen, ms_per_step=tms, search_s=round(time.perf_counter() - t0, 2), cache=cache)
    sim = _lib.Simulation(N, P, cic=cic, dt=dt, device=local, force_mode=mode, **shape)
    stream = sim.stream()
    sim.set_state(state)
    config["force_mode"] = args.force_mode

    # ---- FP64 energy / momentum before the run (outside the timed region) ----
    def conserved():
        sim.run_stage(_lib.STAGE_DEPOSIT)
        sim.run_stage(_lib.STAGE_POTENTIAL)
        ke, pe, px, py = sim.diagnostics()
        # force = +grad(phi) with phi = G * rho > 0: E = KE - sum(m phi)/2
        return {"kinetic": ke, "potential": -pe, "energy": ke - pe, "momentum": [px, py]}

    cons0 = conserved()

    # ---- device-timed throughput (state resident) ----
    clk = ClockSampler(local).__enter__()
    sim.step(args.warmup)
    sim.synchronize()
    clk.wait_first()
    barrier(ws)
    k0 = sim.kernels_launched()
    try:
        windows = timed_windows(rt, stream, sim.step, args.steps, min_ms=args.min_timed_ms)
        timed_launches = sim.kernels_launched() - k0  # the steps' kernels and the re-sorts among them
    finally:
        clk.__exit__()
    sim.synchronize()
    timed_steps = args.steps * len(windows)
    ms_per_step = max_over_ranks(sum(windows) / timed_steps, ws)
    value = P * ws / (ms_per_step / 1e3)
    config["timing"] = (f"{len(windows)} back-to-back windows of {args.steps} steps ({timed_steps} steps, "
                        f"{sum(windows):.1f} ms of device time, CUDA events on the library's stream); the re-sorts "
                        f"fall inside at their own cadence; value = particles x steps / device time")

    # ---- force accuracy of the timed path against FP64 ----
    # The force of the step after the timed region comes from the density the
    # fused step kernel deposited for the positions the timed steps produced;
    # the FP64 oracle computes the force of the same positions.
    force_err = None
    if rank == 0 and not args.no_force_check:
        force_err = force_error_series(sim, N, cic, dt, args.precision_steps)
    cons1 = conserved()
    mtot = float(np.sum(state.m, dtype=np.float64))
    # momentum scale ~ sum m|v| (the larger kinetic energy: runs may start at rest)
    pscale = float(np.sqrt(2.0 * mtot * max(cons0["kinetic"], cons1["kinetic"], 1e-300)))
    drift = {"steps": args.warmup + timed_steps + (max(1, args.precision_steps) if force_err else 0), "start": cons0, "end": cons1,
             "energy_rel": (cons1["energy"] - cons0["energy"]) / abs(cons0["energy"]) if cons0["energy"] else None,
             "momentum_rel": float(np.hypot(cons1["momentum"][0] - cons0["momentum"][0],
                                            cons1["momentum"][1] - cons0["momentum"][1]) / pscale),
             "note": "FP64 sums on the GPU over active particles; v = (x - xOld)/dt, phi sampled at the NGP cell"}

    # ---- per-stage times over the timed region's own steps ----
    # The fused kernel's time depends on how far the particles drifted since
    # the last sort, and so on the state's age.  The timed steps are therefore
    # replayed from the same initial state (same warm-up, same number of
    # steps) one step per graph launch with CUDA events between the stages,
    # and each stage's time is averaged over exactly the timed region's steps.
    sim.set_state(state)
    conserved()
    sim.step(args.warmup)
    sim.synchronize()
    sim.set_profiling(True)
    prof_steps = timed_steps
    names = ["prologue", "fft_conv", "force", "fused_step", "sort"]
    acc = np.zeros(len(names))
    sorts = 0
    for _ in range(prof_steps):
        sim.step(1)
        t = np.pad(sim.stage_times(), (0, len(names)))[:len(names)]
        acc += t
        sorts += int(t[4] > 0)
    sim.set_profiling(False)
    sim.synchronize()
    stage_ms = acc / prof_steps  # sort: amortised per step
    stages = {n: round(float(t), 5) for n, t in zip(names, stage_ms)}
    stages["sort_per_sort"] = round(float(acc[4] / max(sorts, 1)), 5)
    # algorithmic bytes per launch (per step for the FFT passes)
    algo = {
        # read x, y, xOld, yOld, m (20 B), write x, y, xOld, yOld (16 B); force window 8 B/cell,
        # density flush 4 B/cell (the clear of the density is the row pass's)
        "fused_step": 36.0 * P + 12.0 * N * N,
        # gradient mode: r2c rows 4+4+4 (the density read, the half spectrum written, the density
        # cleared), columns 4+1+4 (real K on a quarter: 1 B/cell), c2r rows 4+4;
        # spectral mode (force straight from the FFT): r2c 4+4+4, columns 4+1+8, c2r 8+8
        "fft_conv": (41.0 if args.force_mode != "gradient" else 29.0) * N * N,
        "force": 12.0 * N * N,
    }
    dom = max(algo, key=lambda k: stages.get(k, 0.0))
    peak, peak_kind = measured_peak_gbs()
    achieved = algo[dom] / (stages[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": algo[dom], "traffic": measured_traffic(dom, P)}

    # ---- end to end through the C ABI with host buffers ----
    # The state is uploaded from page-locked host memory inside the timed region
    # and every R steps the step's output goes back to page-locked host memory:
    # the display frame (N*N floats, what the reference's worker delivers) for
    # `e2e`, the positions (x, y) for `e2e_positions`.  Host buffers rotate
    # through a small ring; a buffer is reused only after its copy has landed.
    def e2e_run(frames: bool):
        host_state = state.copy()
        if frames:
            bufs = [(np.empty((N, N), np.float32),) for _ in range(4)]
        else:
            bufs = [(np.empty(P, np.float32), np.empty(P, np.float32)) for _ in range(2)]
        pinned = [host_state.x, host_state.y, host_state.x_old, host_state.y_old, host_state.m]
        pinned += [a for b in bufs for a in b]
        for a in pinned:
            rt.pin(a)
        try:
            sim.synchronize()
            # one job of the workload's own length (1000 steps for the headline disk), or --steps if longer
            steps_e = max(args.steps, int(w.get("steps", 0)))
            R = max(1, args.render_interval)
            tickets, nread = {}, 0
            t0 = time.perf_counter()
            sim.set_state(host_state)
            done = 0
            while done < steps_e:
                k = min(R, steps_e - done)
                if k > 1:
                    sim.step(k - 1)
                slot = nread % len(bufs)
                if slot in tickets:
                    sim.wait(tickets[slot])
                # like the reference's worker: the frame of the density at the start
                # of the interval's last step, copied while that step runs
                tickets[slot] = (sim.frame_async(bufs[slot][0]) if frames
                                 else sim.positions_async(bufs[slot][0], bufs[slot][1], ordered=False))
                nread += 1
                sim.step(1)
                done += k
            for t in tickets.values():
                sim.wait(t)
            sim.synchronize()
            t1 = time.perf_counter()
        finally:
            for a in pinned:
                rt.unpin(a)
        out_bytes = (4 * N * N) if frames else (8 * P)
        return {"value": P * steps_e / (t1 - t0), "unit": UNIT, "h2d_bytes_per_step": int(20 * P / steps_e),
                "d2h_bytes_per_step": int(out_bytes * nread / steps_e),
                "steps": steps_e,
                "note": (f"one job of {steps_e} steps: the state uploaded once from page-locked memory (bytes "
                         f"amortised over the steps); "
                         + (f"the display frame ({N}x{N} floats, the reference's output) read back every {R} steps"
                            if frames else f"x, y read back every {R} steps") + "; host link measured at ~192 GB/s")}

    e2e = e2e_pos = None
    if not args.no_e2e:
        try:
            e2e = e2e_run(frames=True)
        except Exception as exc:  # report, never hide
            e2e = {"value": None, "unit": UNIT, "error": str(exc)}
        try:
            e2e_pos = e2e_run(frames=False)
        except Exception as exc:
            e2e_pos = {"value": None, "unit": UNIT, "error": str(exc)}

    launches = timed_launches
    sim.close()

    # ---- the metric's second arm: the same step with the tensor-core split FFT ----
    # FP16 hi/lo split (tc_split_fft) and BF16 hi/lo split (tc_split_fft_bf16)
    def tc_run(force_mode, precision):
        try:
            with _lib.Simulation(N, P, cic=cic, dt=dt, device=local, force_mode=force_mode, **shape) as ts:
                ts.set_state(state)
                ts.step(args.warmup)
                ts.synchronize()
                tw = timed_windows(rt, ts.stream(), ts.step, args.steps, min_ms=args.min_timed_ms / 2)
                tsteps = args.steps * len(tw)
                tms = sum(tw) / tsteps
                terr = None if args.no_force_check else force_error_series(ts, N, cic, dt, args.precision_steps)
            return {"value": P / (tms / 1e3), "unit": UNIT, "ms_per_step": tms, "steps": tsteps,
                    "force_rel_err_vs_fp64": terr, "precision": precision,
                    "faster_than_plain": bool(tms < ms_per_step),
                    "note": "column FFTs (3 of the 5 length-N transforms per step) as tcgen05 GEMMs; timed like "
                            "the plain path (back-to-back windows, re-sorts inside)"}
        except Exception as exc:
            return {"unavailable": str(exc)}

    tc_arm = tc_arm_bf16 = None
    if rank == 0 and not args.no_tc_compare and mode == _lib.FORCE_SPECTRAL and N in (1024, 2048, 4096):
        tc_arm = tc_run(_lib.FORCE_SPECTRAL_TC_FP16, "FP16 hi/lo split operands, FP32 accumulate")
        tc_arm_bf16 = tc_run(_lib.FORCE_SPECTRAL_TC_BF16, "BF16 hi/lo split operands, FP32 accumulate")

    # ---- the reference's own step on the same GPU (its kernels + cuFFT) ----
    ref_gpu = None
    if rank == 0 and not args.no_reference_gpu:
        try:
            from oracle import ref_oracle
            if ref_oracle.available(N, dt):
                with ref_oracle.RefGPU(N, cic, dt, P) as ref:
                    ref.set_state(state)
                    ref.time_steps(3)
                    rms = ref.time_steps(args.ref_steps)
                ref_gpu = {"ms_per_step": rms, "value": P / (rms / 1e3), "unit": UNIT, "steps": args.ref_steps,
                           "source": "reference kernels (CosmosCuda.cuh) compiled for sm_103a + cuFFT, "
                                     "Universe<K> step sequence, same GPU and state"}
            else:
                ref_gpu = {"unavailable": "reference PTX not built for this lattice/time step"}
        except Exception as exc:
            ref_gpu = {"unavailable": str(exc)}
    cb = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(state, N, cic, dt, args.cpu_seconds)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "timed_steps": timed_steps, "windows": len(windows), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": config,
            "roofline": roofline, "cpu_baseline": cb, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": launches, "stages_ms": stages, "reference_gpu": ref_gpu,
            "force_rel_err_vs_fp64": force_err, "fp64_drift": drift, "tc_split_fft": tc_arm, "tc_split_fft_bf16": tc_arm_bf16,
            "e2e_positions": e2e_pos}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
