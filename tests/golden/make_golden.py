#!/usr/bin/env python3
"""Generate golden fixtures from the reference's own CUDA kernels.

Runs the reference step (CosmosCuda.cuh's kernels compiled for this GPU, with
cuFFT, through oracle/ref_runner.cpp) on small seeded inputs and stores the
inputs and outputs as tests/golden/<case>.npz:
  inputs      x, y, x_old, y_old, m                      (float32)
  after step 1: density, potential, force (the lattices of the first step) and
              x1, y1, x_old1, y_old1
  after `steps`: xk, yk, x_oldk, y_oldk
(cases of kind "icdisk": inputs from the counter-based generator, not stored;
outputs at sampled particles `idx`, plus the next step's density and force
at sampled `cells`), and the render chain's frames as tests/golden/render<N>.npz: a sequence of
seeded density lattices (render_density) rendered one after another (the
running min / max carry over), stored as the values at fixed sampled cells;
the SHA-256 of every full frame goes into the manifest.
Needs a GPU and the reference PTX (oracle/_ref, built by oracle/ref_build.py
where the reference sources are present).

  python tests/golden/make_golden.py [--out DIR]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_oracle  # noqa: E402

# name: (N, cic, dt, P, steps, kind, seed)
CASES = {
    "ngp64_uniform": (64, False, 0.01, 4099, 5, "uniform", 11),
    "cic64_disk": (64, True, 0.01, 4096, 5, "disk", 12),
    "cic128_disk": (128, True, 0.005, 8192, 10, "disk", 13),
    "ngp512_uniform": (512, False, 0.002, 16384, 10, "uniform_rest", 14),
    # the headline lattice and deposit (particles only: the lattices are 16-32 MB)
    "cic2048_disk": (2048, True, 0.001, 16384, 3, "disk", 15),
    # the headline lattice at a density where the sorted tiles of the disk's
    # inner region hold thousands of particles, so the tile-sorted step runs
    # its shared-window gathers and fixed-point deposits: 2^20 particles on an
    # exponential disk of scale 200 cells from the counter-based generator
    # (inputs regenerated bit for bit by oracle/ic_np.py, not stored); the
    # outputs are stored at sampled particles and cells
    "cic2048_disk1m": (2048, True, 0.001, 1 << 20, 3, "icdisk", 16),
}
SAMPLES = 65536


def make_ic_inputs(N, dt, P, seed):
    """Exponential disk of scale 200 cells at the lattice centre, circular speeds
    from the enclosed mass plus 5% dispersion, lognormal(0, 0.3) masses of mean
    ~1, from the platform-independent float32 generator."""
    from oracle import ic_np
    x, y, xo, yo, m = ic_np.generate(ic_np.EXP_DISK, P, seed=seed, N=N, dt=dt, center_x=N / 2.0, center_y=N / 2.0,
                                     scale=200.0, rmax=N / 2.0 - 8.0, mass=float(P), mass_sigma=0.3, spin=1.0,
                                     dispersion=0.05, g=1.0)
    return dict(x=x, y=y, x_old=xo, y_old=yo, m=m)


def sample_particles(P, seed):
    h = _splitmix64(np.arange(SAMPLES, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 32))
    return np.unique((h % np.uint64(P)).astype(np.int64))


def sample_cells(N, seed):
    """Cells of the central half of the lattice (where the disk's mass is)."""
    h = _splitmix64(np.arange(SAMPLES, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 33) + np.uint64(1))
    cx = N // 4 + (h % np.uint64(N // 2)).astype(np.int64)
    cy = N // 4 + ((h >> np.uint64(32)) % np.uint64(N // 2)).astype(np.int64)
    return np.unique(cx + cy * N)


def make_inputs(N, dt, P, kind, seed):
    rng = np.random.default_rng(seed)
    if kind in ("uniform", "uniform_rest"):
        x = rng.uniform(0.0, N, P)
        y = rng.uniform(0.0, N, P)
        if kind == "uniform":
            vx, vy = rng.normal(0.0, 2.0, (2, P))
            m = rng.lognormal(0.0, 0.3, P)
        else:
            vx = vy = np.zeros(P)
            m = np.ones(P)
        # a few particles parked outside the active window
        x[:5] = [-10.0, 0.5, N - 0.5, 1.0, N - 1.0]
    else:
        scale = N / 8.0
        r = np.minimum(rng.gamma(2.0, scale, P), N / 2 - 6)
        a = rng.uniform(0, 2 * np.pi, P)
        m = rng.lognormal(0.0, 0.3, P)
        order = np.argsort(r, kind="stable")
        menc = np.empty(P)
        menc[order] = np.cumsum(m[order]) - m[order]
        vc = np.sqrt(menc / np.maximum(r, 1e-3))
        x = N / 2 + r * np.cos(a)
        y = N / 2 + r * np.sin(a)
        vx = -vc * np.sin(a) * 0.05
        vy = vc * np.cos(a) * 0.05
    f = lambda v: np.ascontiguousarray(v, np.float32)
    x, y = f(x), f(y)
    return dict(x=x, y=y, x_old=f(x - vx * dt), y_old=f(y - vy * dt), m=f(m))


# render cases: name: (N, [(seed, scale) per frame]); the reference's blur grid
# covers the lattice only for N >= 1024
RENDER_CASES = {
    "render2048": (2048, [(21, 1e-4), (22, 3e-4), (23, 5e-5)]),
}
RENDER_DT = 0.001  # any reference PTX of this N will do; the render chain ignores dt
RENDER_SAMPLES = 8192


def _splitmix64(v: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014) on uint64 arrays."""
    with np.errstate(over="ignore"):
        z = v + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def render_density(N: int, seed: int, scale: float) -> np.ndarray:
    """Platform-independent seeded density lattice: a quarter of the cells hold
    a uniform value in [0, scale), the rest are empty."""
    h = _splitmix64(np.arange(N * N, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 40))
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
    occupied = (h & np.uint64(3)) == 0
    return np.where(occupied, u * scale, 0.0).astype(np.float32).reshape(N, N)


def render_sample_cells(N: int) -> np.ndarray:
    h = _splitmix64(np.arange(RENDER_SAMPLES, dtype=np.uint64) + np.uint64(7))
    return (h % np.uint64(N * N)).astype(np.int64)


class _S:
    def __init__(self, d):
        self.__dict__.update(d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    ap.add_argument("--render-only", action="store_true",
                    help="remake only the render fixtures; keep the step cases of the manifest")
    ap.add_argument("--only", default=None,
                    help="make only this step case; keep the other cases and the render fixtures of the manifest")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    manifest, kept_render = {}, None
    if args.render_only or args.only:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "manifest.json")) as f:
            old = json.load(f)
        manifest = old["cases"]
        kept_render = old.get("render", {}) if args.only else None
    for name, (N, cic, dt, P, steps, kind, seed) in CASES.items():
        if args.render_only:
            break
        if args.only and name != args.only:
            continue
        inp = make_ic_inputs(N, dt, P, seed) if kind == "icdisk" else make_inputs(N, dt, P, kind, seed)
        with ref_oracle.RefGPU(N, cic, dt, P) as ref:
            ref.set_state(_S(inp))
            ref.step(1)
            density, potential, force = ref.fields()
            x1, y1, xo1, yo1 = ref.state()
            ref.step(steps - 1)
            xk, yk, xok, yok = ref.state()
            if kind == "icdisk":  # the lattices of the next step: the density and force of (xk, yk)
                ref.step(1)
                dnext, _, fnext = ref.fields()
        if kind == "icdisk":
            idx, cells = sample_particles(P, seed), sample_cells(N, seed)
            pick = lambda a: a[idx]
            out = dict(idx=idx, x1=pick(x1), y1=pick(y1), x_old1=pick(xo1), y_old1=pick(yo1), xk=pick(xk),
                       yk=pick(yk), x_oldk=pick(xok), y_oldk=pick(yok), cells=cells,
                       density_next=dnext.reshape(-1)[cells], force_next=fnext.reshape(-1, 2)[cells])
        else:
            out = dict(inp, x1=x1, y1=y1, x_old1=xo1, y_old1=yo1, xk=xk, yk=yk, x_oldk=xok, y_oldk=yok)
        if N <= 128:
            out.update(density=density, potential=potential, force=force)
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **out)
        manifest[name] = dict(N=N, cic=cic, dt=dt, P=P, steps=steps, kind=kind, seed=seed, fields=N <= 128)
        print(name, "ok", flush=True)
    render = {} if kept_render is None else kept_render
    for name, (N, frames) in RENDER_CASES.items():
        if kept_render is not None:
            break
        cells = render_sample_cells(N)
        values, digests = [], []
        with ref_oracle.RefGPU(N, False, RENDER_DT, 4) as ref:
            for seed, scale in frames:
                frame = ref.render(render_density(N, seed, scale))
                values.append(frame.reshape(-1)[cells])
                digests.append(hashlib.sha256(frame.tobytes()).hexdigest())
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), cells=cells, values=np.stack(values))
        render[name] = dict(N=N, blur_r=3, frames=[[seed, scale] for seed, scale in frames], sha256=digests)
        print(name, "ok", flush=True)
    with open(os.path.join(args.out, "manifest.json"), "w") as f:
        json.dump({"source": "reference kernels (CosmosCuda.cuh) compiled for sm_103a + cuFFT, "
                             "run by oracle/ref_runner.cpp", "cases": manifest, "render": render}, f, indent=1)


if __name__ == "__main__":
    main()
