"""CPU checks of the float32 initial-condition restatement (oracle/ic_np.py):
its series for ln, exp, sin and cos against numpy's functions, and the
sampled distributions against their analytic moments."""
import numpy as np

from oracle import ic_np

F = np.float32


def test_series_functions_accuracy():
    u = np.linspace(1e-6, 1.0, 200001, dtype=F)
    assert np.max(np.abs(ic_np.ln(u) - np.log(u.astype(np.float64)))) < 2e-6
    x = np.linspace(-30.0, 5.0, 200001, dtype=F)
    ex = np.exp(x.astype(np.float64))
    assert np.max(np.abs(ic_np.exp_(x) - ex) / ex) < 5e-7
    h = np.arange(0, 1 << 24, 97, dtype=np.uint32)
    sn, cs = ic_np.sincos_turn(h)
    a = 2.0 * np.pi * h.astype(np.float64) / (1 << 24)
    assert np.max(np.abs(sn - np.sin(a))) < 3e-7 and np.max(np.abs(cs - np.cos(a))) < 3e-7


def test_gaussian_moments():
    i = np.arange(1_000_000, dtype=np.uint64)
    z = ic_np.gauss(ic_np.draw(7, i, 0), ic_np.draw(7, i, 1)).astype(np.float64)
    assert abs(z.mean()) < 5e-3 and abs(z.std() - 1.0) < 5e-3


def test_family_distributions():
    n = 400_000
    x, y, xo, yo, m = ic_np.generate(ic_np.EXP_DISK, n, seed=3, center_x=1024, center_y=1024, scale=50.0, mass=n,
                                     spin=1.0, dt=0.001)
    r = np.hypot(x - 1024.0, y - 1024.0)
    assert abs(r.mean() / 100.0 - 1.0) < 0.01  # gamma(2) radius: mean 2 * scale
    assert np.allclose(m, 1.0)
    x, y, *_ = ic_np.generate(ic_np.PLUMMER, n, seed=4, center_x=500, center_y=500, scale=20.0, mass=n)
    r = np.hypot(x - 500.0, y - 500.0)
    assert abs(np.median(r) / 20.0 - 1.0) < 0.02  # projected Plummer: M(<a) = M / 2
    x, y, *_ = ic_np.generate(ic_np.UNIFORM, n, seed=5, center_x=100, center_y=100, scale=50.0)
    assert x.min() >= 50.0 and x.max() < 150.0 and abs(x.mean() - 100.0) < 0.2


def test_ring_disk_follows_the_reference_formula():
    """addGalaxy (CosmosCuda.cuh:1080-1110): radii in [0.1, 1] * N * radius,
    the black hole last, masses over the total particle count."""
    N, n, T = 256, 5000, 20000
    x, y, xo, yo, m = ic_np.generate(ic_np.RING_DISK, n, seed=1, N=N, dt=50.0, center_x=0.25, center_y=0.75,
                                     scale=0.2, mass=1.0, spin=0.005, bulk_vx=2.5e-5, black_hole=True,
                                     total_particles=T)
    r = np.hypot(x[:-1] - 64.0, y[:-1] - 192.0)
    assert r.min() >= 0.1 * N * 0.2 * 0.999 and r.max() <= N * 0.2 * 1.001
    assert x[-1] == F(64.0) and y[-1] == F(192.0)
    assert m[0] == F(1.0) / F(T) and m[-1] == F(F(n) * F(1.0) / F(1000.0)) / F(T)
