"""Float32 restatement of the device initial-condition generator -- TEST INFRASTRUCTURE.

Restates cosmossimulationwithcuda_gb300/csrc/pm_ics.cu operation by operation
in numpy float32 (every multiply, add, divide and square root separately
rounded, as the kernel's _rn intrinsics are), so the GPU output must match it
bit for bit.  Counter-based draws: SplitMix64 (Steele, Lea, Flood, OOPSLA
2014) of seed + GOLDEN * (16 i + d + 1), i the particle identity.

Families mirror cosmos_ic_params (include/cosmos_pm.h); the RING_DISK
family is the reference's addGalaxy formula (CosmosCuda.cuh:1080-1110).
"""
from __future__ import annotations

import numpy as np

F = np.float32
U = np.uint64
GOLDEN = U(0x9E3779B97F4A7C15)
UNIFORM, EXP_DISK, PLUMMER, RING_DISK = 0, 1, 2, 3


def splitmix(z):
    z = np.asarray(z, np.uint64)
    z = (z ^ (z >> U(30))) * U(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> U(27))) * U(0x94D049BB133111EB)
    return z ^ (z >> U(31))


def draw(seed, i, d):
    return splitmix(U(seed) + GOLDEN * (U(16) * i + U(d + 1)))


def uniform_open(h):
    return ((h >> U(40)).astype(np.uint32) | np.uint32(1)).astype(F) * F(5.9604644775390625e-8)


def uniform_closed(h):
    return (h >> U(40)).astype(np.uint32).astype(F) * F(5.9604644775390625e-8)


def ln(u):
    u = np.asarray(u, F)
    bits = u.view(np.uint32)
    e = ((bits >> np.uint32(23)) & np.uint32(0xFF)).astype(np.int32) - np.int32(127)
    m = ((bits & np.uint32(0x7FFFFF)) | np.uint32(0x3F800000)).view(F)
    big = m > F(1.41421354)
    m = np.where(big, m * F(0.5), m)
    e = np.where(big, e + np.int32(1), e)
    s = (m - F(1.0)) / (m + F(1.0))
    s2 = s * s
    p = np.full_like(s, F(0.111111112))
    p = p * s2 + F(0.142857149)
    p = p * s2 + F(0.200000003)
    p = p * s2 + F(0.333333343)
    p = p * s2 + F(1.0)
    return (F(2.0) * s) * p + e.astype(F) * F(0.693147182)


def exp_(x):
    x = np.clip(np.asarray(x, F), F(-80.0), F(80.0))
    k = np.rint(x * F(1.44269502))
    r = (x - k * F(0.693145751953125)) - k * F(1.42860682e-6)
    p = np.full_like(r, F(2.48015876e-5))
    for c in (1.98412701e-4, 1.38888892e-3, 8.33333377e-3, 4.16666679e-2, 0.166666672, 0.5, 1.0, 1.0):
        p = p * r + F(c)
    scale = ((k.astype(np.int32) + np.int32(127)).astype(np.uint32) << np.uint32(23)).view(F)
    return p * scale


def sincos_turn(h24):
    h24 = np.asarray(h24, np.uint32)
    q = h24 >> np.uint32(22)
    f = h24 & np.uint32(0x3FFFFF)
    upper = f > np.uint32(0x200000)
    f = np.where(upper, np.uint32(0x400000) - f, f)
    th = f.astype(F) * F(3.74507039e-7)
    t2 = th * th
    ps = np.full_like(th, F(-2.50521079e-8))
    for c in (2.75573188e-6, -1.98412701e-4, 8.33333377e-3, -0.166666672, 1.0):
        ps = ps * t2 + F(c)
    s0 = th * ps
    pc = np.full_like(th, F(2.08767559e-9))
    for c in (-2.75573188e-7, 2.48015876e-5, -1.38888892e-3, 4.16666679e-2, -0.5):
        pc = pc * t2 + F(c)
    c0 = pc * t2 + F(1.0)
    s1 = np.where(upper, c0, s0)
    c1 = np.where(upper, s0, c0)
    sn = np.select([q == 0, q == 1, q == 2], [s1, c1, -s1], -c1)
    cs = np.select([q == 0, q == 1, q == 2], [c1, -s1, -c1], s1)
    return sn.astype(F), cs.astype(F)


def gauss(ha, hb):
    sn, cs = sincos_turn((hb >> U(40)).astype(np.uint32))
    return np.sqrt(F(-2.0) * ln(uniform_open(ha))) * cs


def generate(kind, count, first=0, seed=0, N=2048, dt=0.001, center_x=0.0, center_y=0.0, scale=1.0, rmax=0.0,
             mass=1.0, mass_sigma=0.0, bulk_vx=0.0, bulk_vy=0.0, spin=0.0, dispersion=0.0, g=1.0,
             black_hole=False, total_particles=0):
    """(x, y, x_old, y_old, m) float32 arrays of `count` particles with
    identities first .. first+count-1."""
    j = np.arange(count, dtype=np.int64)
    i = (np.int64(first) + j).astype(np.uint64)
    cx, cy, s, dt_f = F(center_x), F(center_y), F(scale), F(dt)
    mass_f = F(mass)
    m = np.full(count, mass_f / F(count), F)
    if kind == RING_DISK:
        Nf, n = F(N), F(count)
        w = F(spin) / dt_f
        R = Nf * s
        rad2 = R * R
        total = mass_f * n + ((n * mass_f) / F(1000.0) if black_hole else F(0.0))
        cvx, cvy = F(bulk_vx) / dt_f, F(bulk_vy) / dt_f
        cxn, cyn = cx * Nf, cy * Nf
        r = (F(0.1) + F(0.9) * uniform_closed(draw(seed, i, 0))) * R
        sn, cs = sincos_turn((draw(seed, i, 1) >> U(40)).astype(np.uint32))
        speed = np.sqrt(((F(4.4e-6) * total) * r) / rad2)
        px = r * cs + cxn
        py = r * sn + cyn
        vecx, vecy = px - cxn, py - cyn
        pxo = (-dt_f) * ((vecy * w) * speed + cvx * Nf) + px
        pyo = (-dt_f) * (((-vecx) * w) * speed + cvy * Nf) + py
        m = np.full(count, mass_f / F(total_particles), F)
        if black_hole and count > 0:
            px[-1], py[-1] = cxn, cyn
            pxo[-1] = px[-1] - (cvx * Nf) * dt_f
            pyo[-1] = py[-1] - (cvy * Nf) * dt_f
            m[-1] = ((n * mass_f) / F(1000.0)) / F(total_particles)
        return px, py, pxo, pyo, m
    if kind == UNIFORM:
        px = cx + (F(2.0) * uniform_closed(draw(seed, i, 0)) - F(1.0)) * s
        py = cy + (F(2.0) * uniform_closed(draw(seed, i, 1)) - F(1.0)) * s
        vx = F(dispersion) * gauss(draw(seed, i, 2), draw(seed, i, 3))
        vy = F(dispersion) * gauss(draw(seed, i, 4), draw(seed, i, 5))
    else:
        rmax_f = F(rmax)
        if kind == EXP_DISK:
            r = np.zeros(count, F)
            ok = np.zeros(count, bool)
            for t in range(6):
                u = uniform_open(draw(seed, i, 2 * t)) * uniform_open(draw(seed, i, 2 * t + 1))
                rt = (-s) * ln(u)
                take = ~ok
                r = np.where(take, rt, r)
                ok = ok | (take & ((rmax_f <= F(0)) | (rt < rmax_f)))
            r = np.where(ok, r, rmax_f * uniform_closed(draw(seed, i, 12)))
            q = r / s
            frac = F(1.0) - (F(1.0) + q) * exp_(-q)
            if rmax_f > F(0):
                qm = rmax_f / s
                frac = frac / (F(1.0) - (F(1.0) + qm) * exp_(np.full(1, -qm, F))[0])
        else:
            u = uniform_open(draw(seed, i, 0))
            umax = F(1.0)
            if rmax_f > F(0):
                rm2 = rmax_f * rmax_f
                umax = rm2 / (rm2 + s * s)
                u = np.where(u > umax, umax, u)
            r = s * np.sqrt(u / (F(1.0) - u))
            frac = u / umax
        sn, cs = sincos_turn((draw(seed, i, 13) >> U(40)).astype(np.uint32))
        px = cx + r * cs
        py = cy + r * sn
        rr = np.where(r > F(1e-3), r, F(1e-3))
        vc = np.sqrt(((F(g) * mass_f) * frac) / rr)
        vx = ((-F(spin)) * vc) * sn
        vy = (F(spin) * vc) * cs
        if F(dispersion) > F(0):
            sd = F(dispersion) * vc
            ha, hb = draw(seed, i, 14), draw(seed, i, 15)
            vx = vx + sd * gauss(ha, hb)
            vy = vy + sd * gauss(ha ^ GOLDEN, hb ^ GOLDEN)
    vx = vx + F(bulk_vx)
    vy = vy + F(bulk_vy)
    if F(mass_sigma) > F(0):
        h = draw(seed, i, 11)
        m = m * exp_(F(mass_sigma) * gauss(h, splitmix(h)))
    return (px.astype(F), py.astype(F), (px - vx * dt_f).astype(F), (py - vy * dt_f).astype(F), m.astype(F))
