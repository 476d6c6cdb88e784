"""CPU tests of the oracle: the C++ restatement against the independent numpy
restatement, and known-answer tests derived from the mathematics of the
reference algorithm (the reference ships no tests or golden vectors)."""
import numpy as np
import pytest

from oracle import pm_np, pm_oracle
from tests.conftest import rel_l2


def _particles(rng, P, N, margin=0.0):
    x = rng.uniform(margin, N - margin, P).astype(np.float32)
    y = rng.uniform(margin, N - margin, P).astype(np.float32)
    xo = (x + rng.normal(0, 0.02, P)).astype(np.float32)
    yo = (y + rng.normal(0, 0.02, P)).astype(np.float32)
    m = rng.lognormal(0.0, 0.3, P).astype(np.float32)
    return x, y, xo, yo, m


@pytest.mark.parametrize("cic", [False, True])
@pytest.mark.parametrize("N", [16, 64])
def test_cpp_oracle_matches_numpy(rng, N, cic):
    x, y, xo, yo, m = _particles(rng, 4 * N * N // 4 + 3, N)  # P % 4 == 3: trailing particles frozen
    o = pm_oracle.OraclePM(N, cic, 0.01, 1.0, fp64=True)
    xs, ys, xos, yos = x.copy(), y.copy(), xo.copy(), yo.copy()
    o.step(xs, ys, xos, yos, m, 1)
    (xn, yn, xon, yon), (rho, phi, F) = pm_np.step(x, y, xo, yo, m, N, cic, 0.01)
    assert rel_l2(o.density(), rho) < 1e-14
    assert rel_l2(o.potential_field(), phi) < 1e-12
    assert rel_l2(o.force(), F) < 1e-12
    np.testing.assert_array_equal(xs, xn)
    np.testing.assert_array_equal(ys, yn)
    np.testing.assert_array_equal(xos, xon)
    # trailing P % 4 particles untouched (CosmosCuda.cuh:239-242)
    np.testing.assert_array_equal(xs[-3:], x[-3:])


def test_fp32_port_close_to_fp64(rng):
    N = 64
    x, y, xo, yo, m = _particles(rng, 8192, N)
    o64 = pm_oracle.OraclePM(N, True, 0.01, 1.0, fp64=True)
    o32 = pm_oracle.OraclePM(N, True, 0.01, 1.0, fp64=False)
    for o in (o64, o32):
        o.deposit(x, y, m)
        o.potential()
        o.gradient()
    assert rel_l2(o32.density(), o64.density()) < 1e-6
    assert rel_l2(o32.potential_field(), o64.potential_field()) < 1e-6
    assert rel_l2(o32.force(), o64.force()) < 1e-4


def test_green_filter_is_real_even():
    """G is real and even, so FFT(G) is real (the basis of the real filter K)."""
    N = 32
    o = pm_oracle.OraclePM(N, True, 0.01, 1.0, fp64=True)
    G, D = o.filters()
    assert np.abs(G.imag).max() < 1e-9 * np.abs(G.real).max()
    # CIC deconvolution spectrum after the phase shift: (-1)^(kx+ky) cos(pi kx/N) cos(pi ky/N)
    k = np.arange(N)
    ks = np.where(k <= N // 2, k, k - N)
    c = np.cos(np.pi * ks / N)
    sign = (-1.0) ** (k[None, :] + k[:, None])
    np.testing.assert_allclose(D.real, sign * c[None, :] * c[:, None], atol=1e-12)
    assert np.abs(D.imag).max() < 1e-12


def test_fft_delta_and_parseval():
    """Potential of one unit mass (NGP) = G shifted to its cell / 1.001."""
    N = 32
    o = pm_oracle.OraclePM(N, False, 0.01, 1.0, fp64=True)
    rho = np.zeros((N, N))
    rho[10, 7] = 1.0  # y = 10, x = 7
    o.set_density(rho)
    o.potential()
    phi = o.potential_field()
    G = pm_np.green_lattice(N)
    expect = np.roll(G, (10, 7), axis=(0, 1)) / 1.001
    np.testing.assert_allclose(phi, expect, rtol=1e-12, atol=1e-12)
    # Parseval on the density spectrum
    r = np.random.default_rng(1).random((N, N))
    assert abs(np.sum(r ** 2) - np.sum(np.abs(np.fft.fft2(r)) ** 2) / N ** 2) < 1e-9


def test_convolution_matches_direct_sum():
    """FFT convolution equals the O(N^4) circular sum of rho * G (NGP)."""
    N = 16
    rng = np.random.default_rng(7)
    rho = rng.random((N, N))
    o = pm_oracle.OraclePM(N, False, 0.01, 1.0, fp64=True)
    o.set_density(rho)
    o.potential()
    G = pm_np.green_lattice(N)
    direct = np.zeros((N, N))
    for y in range(N):
        for x in range(N):
            direct += rho[y, x] * np.roll(G, (y, x), axis=(0, 1))
    np.testing.assert_allclose(o.potential_field(), direct / 1.001, rtol=1e-11)


def test_uniform_density_zero_interior_force():
    N = 32
    o = pm_oracle.OraclePM(N, False, 0.01, 1.0, fp64=True)
    o.set_density(np.ones((N, N)))
    o.potential()
    o.gradient()
    F = o.force()
    assert np.abs(F[2:-2, 2:-2]).max() < 1e-9


def test_two_particles_equal_opposite():
    N = 64
    x = np.array([20.5, 40.5, -10, -10], np.float32)
    y = np.array([32.5, 32.5, -10, -10], np.float32)
    m = np.array([1.0, 1.0, 1.0, 1.0], np.float32)
    o = pm_oracle.OraclePM(N, False, 0.01, 1.0, fp64=True)
    o.deposit(x, y, m)
    o.potential()
    o.gradient()
    F = o.force()
    f1 = F[32, 20]
    f2 = F[32, 40]
    assert f1[0] > 0 and f2[0] < 0  # attraction along +grad(phi)
    np.testing.assert_allclose(f1[0], -f2[0], rtol=1e-9)
    assert abs(f1[1]) < 1e-9 and abs(f2[1]) < 1e-9


def test_momentum_conserved_without_wraps(rng):
    N = 64
    P = 4000
    x, y, xo, yo, m = _particles(rng, P, N, margin=16)
    o = pm_oracle.OraclePM(N, False, 1e-3, 1.0, fp64=True)
    xs, ys, xos, yos = x.copy(), y.copy(), xo.copy(), yo.copy()
    o.step(xs, ys, xos, yos, m, 1)
    # momentum change = dt * sum(m F) ~ 0 for the symmetric Green's lattice
    dp = np.sum(m.astype(np.float64) * ((xs - xos) - (x - xo)))
    scale = np.sum(m.astype(np.float64) * np.abs((xs - xos) - (x - xo)))
    assert abs(dp) < 0.05 * scale


def test_cell_index_truncation():
    """Cells use C truncation; particles outside [1, N-1)^2 are inactive."""
    N = 16
    x = np.array([0.99, 1.0, 14.999, 15.0, -0.5, 7.25, 7.25, 7.25], np.float32)
    y = np.array([5.0, 5.0, 5.0, 5.0, 5.0, 0.5, 14.5, 15.5], np.float32)
    m = np.ones(8, np.float32)
    o = pm_oracle.OraclePM(N, False, 0.01, 1.0, fp64=True)
    o.deposit(x, y, m)
    rho = o.density()
    assert rho[5, 1] == 1.0 and rho[5, 14] == 1.0 and rho[14, 7] == 1.0
    assert rho.sum() == 3.0


def test_sort_keys_and_stable_permutation(rng):
    N = 256
    P = 10000
    x = rng.uniform(-2, N + 2, P).astype(np.float32)
    y = rng.uniform(-2, N + 2, P).astype(np.float32)
    keys = pm_oracle.sort_keys(x, y, N, 5)
    cx = np.trunc(x).astype(np.int64)
    cy = np.trunc(y).astype(np.int64)
    act = (cx >= 1) & (cx < N - 1) & (cy >= 1) & (cy < N - 1)

    def spread(v):
        out = np.zeros_like(v)
        for b in range(16):
            out |= ((v >> b) & 1) << (2 * b)
        return out

    expect = np.where(act, spread(np.where(act, cx, 0) >> 5) | (spread(np.where(act, cy, 0) >> 5) << 1), 64)
    np.testing.assert_array_equal(keys, expect.astype(np.uint32))
    perm = pm_oracle.stable_sort_perm(keys)
    np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))
