"""Seeded initial conditions for the particle-mesh workloads.

The reference fills its particles with std::random_device seeded generators
(CosmosCuda.cuh:931-952 uniform fill, :1080-1116 addGalaxy ring disk), so its
initial conditions cannot be reproduced.  These generators are seeded
(numpy PCG64) and produce the FP32 state the reference stores,
(x, y, xOld, yOld, m) (CosmosCuda.cuh:857-861).  A velocity v is encoded the way
addGalaxy encodes it: xOld = x - v*dt (CosmosCuda.cuh:1099-1100).

Units: lattice cells for positions, cells per unit time for velocities, and
the solver's own gravity: the potential of a point mass m is m/r (the 1/r
Green's lattice of CosmosCuda.cuh:100-117) and the acceleration is its
gradient times the gravity multiplier, so a circular orbit of radius R around
an enclosed mass M has v^2 = g * M / R.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class ParticleState:
    x: np.ndarray
    y: np.ndarray
    x_old: np.ndarray
    y_old: np.ndarray
    m: np.ndarray

    @property
    def count(self) -> int:
        return int(self.x.size)

    def copy(self) -> "ParticleState":
        return ParticleState(self.x.copy(), self.y.copy(), self.x_old.copy(), self.y_old.copy(), self.m.copy())


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _state(x, y, vx, vy, m, dt) -> ParticleState:
    x = _f32(x)
    y = _f32(y)
    return ParticleState(x, y, _f32(x - vx * dt), _f32(y - vy * dt), _f32(m))


def uniform(P: int, N: int, dt: float, seed: int = 1, mass: float = 1.0) -> ParticleState:
    """Uniform positions in [0, N)^2, zero velocity, equal masses (the small plain workload)."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, N, P)
    y = rng.uniform(0.0, N, P)
    z = np.zeros(P)
    return _state(x, y, z, z, np.full(P, mass), dt)


def _enclosed_circular_speed(r: np.ndarray, m: np.ndarray, g: float) -> np.ndarray:
    """sqrt(g * M(<r) / r), with M(<r) the mass of the particles strictly inside r."""
    order = np.argsort(r, kind="stable")
    menc = np.empty_like(r)
    menc[order] = np.cumsum(m[order]) - m[order]
    return np.sqrt(g * menc / np.maximum(r, 1e-3))


def exponential_disk(P: int, N: int, dt: float, seed: int = 2, scale: float = 200.0,
                     center=None, dispersion: float = 0.05, g: float = 1.0,
                     rmax: float | None = None, bulk_velocity=(0.0, 0.0), spin: float = 1.0,
                     mass_sigma: float = 0.3) -> ParticleState:
    """Exponential disk: surface density ~ exp(-R/scale), circular velocities from
    the enclosed mass plus a Gaussian dispersion of `dispersion` * v_c per axis,
    masses lognormal(0, mass_sigma).  Radii beyond rmax (default: 8 cells inside
    the lattice edge) are redrawn."""
    rng = np.random.default_rng(seed)
    cx, cy = (N / 2.0, N / 2.0) if center is None else center
    if rmax is None:
        rmax = min(cx, cy, N - cx, N - cy) - 8.0
    r = rng.gamma(2.0, scale, P)
    bad = r >= rmax
    while bad.any():
        r[bad] = rng.gamma(2.0, scale, int(bad.sum()))
        bad = r >= rmax
    a = rng.uniform(0.0, 2.0 * np.pi, P)
    m = rng.lognormal(0.0, mass_sigma, P)
    vc = _enclosed_circular_speed(r, m, g)
    ca, sa = np.cos(a), np.sin(a)
    vx = -spin * vc * sa + dispersion * vc * rng.standard_normal(P) + bulk_velocity[0]
    vy = spin * vc * ca + dispersion * vc * rng.standard_normal(P) + bulk_velocity[1]
    return _state(cx + r * ca, cy + r * sa, vx, vy, m, dt)


def colliding_disks(P: int, N: int, dt: float, seed: int = 3, scale: float = 300.0,
                    separation: float = 1200.0, approach_per_step: float = 0.5) -> ParticleState:
    """Two counter-rotating exponential disks whose centres are `separation` cells
    apart along x and approach each other at `approach_per_step` cells per step."""
    h = P // 2
    vrel = approach_per_step / dt / 2.0
    c = N / 2.0
    rmax = min(separation / 2.0, c - separation / 2.0) - 8.0
    a = exponential_disk(h, N, dt, seed, scale, (c - separation / 2, c), rmax=rmax,
                         bulk_velocity=(vrel, 0.0), spin=1.0)
    b = exponential_disk(P - h, N, dt, seed + 1000, scale, (c + separation / 2, c), rmax=rmax,
                         bulk_velocity=(-vrel, 0.0), spin=-1.0)
    return ParticleState(*(np.concatenate([getattr(a, f), getattr(b, f)])
                           for f in ("x", "y", "x_old", "y_old", "m")))


def plummer(P: int, N: int, dt: float, center, a: float, total_mass: float, seed: int,
            bulk_velocity=(0.0, 0.0), g: float = 1.0, rmax: float | None = None) -> ParticleState:
    """Plummer sphere projected on the plane (surface density of a Plummer model),
    circular velocities from the enclosed particle mass, equal masses."""
    rng = np.random.default_rng(seed)
    cx, cy = center
    if rmax is None:
        rmax = 20.0 * a
    # projected Plummer: Sigma ~ (1 + R^2/a^2)^-2  ->  M(<R) / M = R^2 / (R^2 + a^2)
    u = rng.uniform(0.0, 1.0, P)
    u = np.minimum(u, rmax ** 2 / (rmax ** 2 + a ** 2))
    r = a * np.sqrt(u / (1.0 - u))
    th = rng.uniform(0.0, 2.0 * np.pi, P)
    m = np.full(P, total_mass / P)
    vc = _enclosed_circular_speed(r, m, g)
    vx = -vc * np.sin(th) + bulk_velocity[0]
    vy = vc * np.cos(th) + bulk_velocity[1]
    return _state(cx + r * np.cos(th), cy + r * np.sin(th), vx, vy, m, dt)


def binary_star(P: int, N: int, dt: float, seed: int = 4, separation: float | None = None,
                a: float | None = None, mass_ratio: float = 0.6, g: float = 1.0) -> ParticleState:
    """Two Plummer spheres with mass ratio 1 : mass_ratio on a circular mutual orbit."""
    if separation is None:
        separation = N / 4.0
    if a is None:
        a = N / 40.0
    p1 = int(round(P / (1.0 + mass_ratio)))
    p2 = P - p1
    m1, m2 = float(p1), float(p2)  # unit-mass particles
    c = N / 2.0
    d1 = separation * m2 / (m1 + m2)
    d2 = separation * m1 / (m1 + m2)
    # relative circular speed for a 1/r potential: v^2 = g (m1 + m2) / separation
    vrel = np.sqrt(g * (m1 + m2) / separation)
    v1 = vrel * m2 / (m1 + m2)
    v2 = vrel * m1 / (m1 + m2)
    rmax = min(separation / 2.0, c - separation / 2.0)
    s1 = plummer(p1, N, dt, (c - d1, c), a, m1, seed, (0.0, -v1), g, rmax=rmax)
    s2 = plummer(p2, N, dt, (c + d2, c), a * 0.8, m2, seed + 1, (0.0, v2), g, rmax=rmax)
    return ParticleState(*(np.concatenate([getattr(s1, f), getattr(s2, f)])
                           for f in ("x", "y", "x_old", "y_old", "m")))


def clumpy_uniform(P: int, N: int, dt: float, seed: int = 5, clumps: int = 32, clump_a: float = 40.0,
                   clump_fraction: float = 0.02) -> ParticleState:
    """Uniform background plus `clumps` Plummer clumps of scale radius clump_a,
    each holding clump_fraction of the mass, everything at rest."""
    rng = np.random.default_rng(seed)
    per = int(P * clump_fraction)
    nbg = P - per * clumps
    xs = [rng.uniform(8.0, N - 8.0, nbg)]
    ys = [rng.uniform(8.0, N - 8.0, nbg)]
    for k in range(clumps):
        c = rng.uniform(0.1 * N, 0.9 * N, 2)
        u = np.minimum(rng.uniform(0.0, 1.0, per), 0.999)
        r = clump_a * np.sqrt(u / (1.0 - u))
        r = np.minimum(r, 0.09 * N)
        th = rng.uniform(0.0, 2.0 * np.pi, per)
        xs.append(c[0] + r * np.cos(th))
        ys.append(c[1] + r * np.sin(th))
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    z = np.zeros(P)
    return _state(x, y, z, z, np.ones(P), dt)


def reference_ring_disk(n: int, N: int, dt: float, seed: int, cx: float = 0.5, cy: float = 0.5,
                        angular_velocity: float = 1.0, mass_per_particle: float = 1.0,
                        radius: float = 0.3, vx: float = 0.0, vy: float = 0.0,
                        black_hole: bool = False, total_particles: int | None = None) -> ParticleState:
    """The reference addGalaxy ring disk (CosmosCuda.cuh:1071-1116), seeded.

    Positions r = (0.1 + 0.9 u) * N * radius at a uniform angle; the orbit speed
    scaling sqrt(4.4e-6 * totalMass * r / radius^2) and the xOld encoding follow
    :1090-1101; with black_hole the last particle sits at the centre with mass
    n * mass_per_particle / 1000 (:1103-1110).  Masses are divided by
    total_particles like the reference (:1101)."""
    rng = np.random.default_rng(seed)
    total_particles = n if total_particles is None else total_particles
    w = angular_velocity / dt
    rad2 = (N * radius) ** 2
    total_mass = mass_per_particle * n + (n * mass_per_particle / 1000.0 if black_hole else 0.0)
    cvx, cvy = vx / dt, vy / dt
    r = (0.1 + 0.9 * rng.uniform(0.0, 1.0, n).astype(np.float32)) * (N * radius)
    a = 2.0 * np.pi * rng.uniform(0.0, 1.0, n)
    s = np.sqrt(0.0000044 * total_mass * r / rad2)
    x = r * np.cos(a) + cx * N
    y = r * np.sin(a) + cy * N
    vxx = x - cx * N
    vyy = y - cy * N
    xo = -dt * ((vyy * w) * s + cvx * N) + x
    yo = -dt * ((-vxx * w) * s + cvy * N) + y
    m = np.full(n, mass_per_particle / total_particles)
    if black_hole and n > 0:
        x[-1] = cx * N
        y[-1] = cy * N
        xo[-1] = x[-1] - cvx * N * dt
        yo[-1] = y[-1] - cvy * N * dt
        m[-1] = (n * mass_per_particle / 1000.0) / total_particles
    return ParticleState(_f32(x), _f32(y), _f32(xo), _f32(yo), _f32(m))


# Workloads (sizes and families of the benchmark configurations).
WORKLOADS = {
    "uniform-1M-512-ngp": dict(P=1 << 20, N=512, cic=False, dt=0.002, steps=10),
    "disk-20M-2048-cic": dict(P=20_000_000, N=2048, cic=True, dt=0.001, steps=1000),
    "collide-100M-4096-cic": dict(P=100_000_000, N=4096, cic=True, dt=0.001, steps=1),
    "clumpy-1B-8192-cic": dict(P=1_000_000_000, N=8192, cic=True, dt=0.0005, steps=100),
}


# The 64-simulation ensemble: N uniform over {256, 512, 1024}, P log-uniform
# over [1e4, 2e6] (rounded to a multiple of 4), initial conditions alternating
# between a binary (two Plummer spheres, 1 : 0.6, circular orbit) and an
# exponential disk; CIC, dt = 0.002.
ENSEMBLE = dict(name="ensemble-64-mixed-cic", sims=64, lattices=(256, 512, 1024), p_min=1e4, p_max=2e6,
                cic=True, dt=0.002, steps=200)


def ensemble_workload(seed: int = 4, sims: int | None = None, p_scale: float = 1.0):
    """(lattice sizes, particle counts, states) of the ensemble workload."""
    e = ENSEMBLE
    sims = e["sims"] if sims is None else sims
    rng = np.random.default_rng(seed)
    Ns = rng.choice(np.array(e["lattices"]), sims)
    Ps = np.exp(rng.uniform(np.log(e["p_min"]), np.log(e["p_max"]), sims)) * p_scale
    Ps = np.maximum((np.round(Ps / 4) * 4).astype(np.int64), 4)
    states = []
    for i, (N, P) in enumerate(zip(Ns, Ps)):
        N, P = int(N), int(P)
        if i % 2 == 0:
            states.append(binary_star(P, N, e["dt"], seed=1000 + i))
        else:
            states.append(exponential_disk(P, N, e["dt"], seed=1000 + i, scale=N / 10.0))
    return [int(n) for n in Ns], [int(p) for p in Ps], states


def make_workload(name: str, P: int | None = None, seed: int | None = None) -> ParticleState:
    w = WORKLOADS[name]
    P = w["P"] if P is None else P
    N, dt = w["N"], w["dt"]
    if name.startswith("uniform"):
        return uniform(P, N, dt, seed=1 if seed is None else seed)
    if name.startswith("disk"):
        return exponential_disk(P, N, dt, seed=2 if seed is None else seed, scale=200.0 * N / 2048)
    if name.startswith("collide"):
        return colliding_disks(P, N, dt, seed=3 if seed is None else seed)
    if name.startswith("clumpy"):
        return clumpy_uniform(P, N, dt, seed=5 if seed is None else seed)
    raise KeyError(name)
