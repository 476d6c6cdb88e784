#!/usr/bin/env python3
"""Generate golden fixtures from the reference's own CUDA kernels.

Runs the reference step (CosmosCuda.cuh's kernels compiled for this GPU, with
cuFFT, through oracle/ref_runner.cpp) on small seeded inputs and stores the
inputs and outputs as tests/golden/<case>.npz:
  inputs      x, y, x_old, y_old, m                      (float32)
  after step 1: density, potential, force (the lattices of the first step) and
              x1, y1, x_old1, y_old1
  after `steps`: xk, yk, x_oldk, y_oldk
Needs a GPU and the reference PTX (oracle/_ref, built by oracle/ref_build.py
where the reference sources are present).

  python tests/golden/make_golden.py [--out DIR]
"""
from __future__ import annotations

import argparse
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
}


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


class _S:
    def __init__(self, d):
        self.__dict__.update(d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    manifest = {}
    for name, (N, cic, dt, P, steps, kind, seed) in CASES.items():
        inp = make_inputs(N, dt, P, kind, seed)
        with ref_oracle.RefGPU(N, cic, dt, P) as ref:
            ref.set_state(_S(inp))
            ref.step(1)
            density, potential, force = ref.fields()
            x1, y1, xo1, yo1 = ref.state()
            ref.step(steps - 1)
            xk, yk, xok, yok = ref.state()
        out = dict(inp, x1=x1, y1=y1, x_old1=xo1, y_old1=yo1, xk=xk, yk=yk, x_oldk=xok, y_oldk=yok)
        if N <= 128:
            out.update(density=density, potential=potential, force=force)
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **out)
        manifest[name] = dict(N=N, cic=cic, dt=dt, P=P, steps=steps, kind=kind, seed=seed, fields=N <= 128)
        print(name, "ok", flush=True)
    with open(os.path.join(args.out, "manifest.json"), "w") as f:
        json.dump({"source": "reference kernels (CosmosCuda.cuh) compiled for sm_103a + cuFFT, "
                             "run by oracle/ref_runner.cpp", "cases": manifest}, f, indent=1)


if __name__ == "__main__":
    main()
