"""Independent numpy FP64 restatement of the reference PM step -- TEST INFRASTRUCTURE.

A second, vectorised restatement of CosmosCuda.cuh's step (small N only),
written with numpy's pocketfft instead of the hand-written radix-2 FFT of
oracle/cpu_pm.cpp, so that the two oracles cross-check each other.  Used only
by tests.
"""
from __future__ import annotations

import numpy as np


def green_lattice(N: int) -> np.ndarray:
    """G(i, j): 1/r with minimum-image distances, 3.0 at r <= 0.5.

    CosmosCuda.cuh:100-117 (index = i + j*N, so axis 0 of the returned array
    is j (y) and axis 1 is i (x))."""
    i = np.arange(N)
    d = np.where(i <= N // 2, i, i - N).astype(np.float64)
    r = np.sqrt(d[None, :] ** 2 + d[:, None] ** 2)
    with np.errstate(divide="ignore"):
        g = np.where(r > 0.5, 1.0 / np.where(r > 0, r, 1.0), 3.0)
    return g


def mass_assignment_spectrum(N: int, cic: bool) -> np.ndarray:
    """FFT of the mass-assignment kernel at (N/2, N/2), with the CIC phase shift.

    CosmosCuda.cuh:384-414 (kernel), :1025 (FFT), :427-443 (phase, fx = fy = -0.5)."""
    d = np.zeros((N, N), np.complex128)
    h = N // 2
    if cic:
        d[h:h + 2, h:h + 2] = 0.25
    else:
        d[h, h] = 1.0
    D = np.fft.fft2(d)
    if cic:
        k = np.arange(N)
        ks = np.where(k <= h, k, k - N).astype(np.float64)
        ph = -2.0 * np.pi * (ks[None, :] * -0.5 / N + ks[:, None] * -0.5 / N)
        D = D * np.exp(1j * ph)
    return D


def deposit(x, y, m, N: int, cic: bool) -> np.ndarray:
    """CosmosCuda.cuh:493-592: NGP / CIC deposit of the first 4*floor(P/4) particles."""
    P = (x.size // 4) * 4
    x = x[:P].astype(np.float32)
    y = y[:P].astype(np.float32)
    m = m[:P].astype(np.float64)
    xi = np.trunc(x).astype(np.int64)
    yi = np.trunc(y).astype(np.int64)
    act = (xi >= 1) & (xi < N - 1) & (yi >= 1) & (yi < N - 1)
    xi, yi, m = xi[act], yi[act], m[act]
    fx = x[act].astype(np.float64) - xi
    fy = y[act].astype(np.float64) - yi
    rho = np.zeros(N * N, np.float64)
    if cic:
        np.add.at(rho, xi + yi * N, (1 - fx) * (1 - fy) * m)
        np.add.at(rho, xi + 1 + yi * N, fx * (1 - fy) * m)
        np.add.at(rho, xi + (yi + 1) * N, (1 - fx) * fy * m)
        np.add.at(rho, xi + 1 + (yi + 1) * N, fx * fy * m)
    else:
        np.add.at(rho, xi + yi * N, m)
    return rho.reshape(N, N)


def potential(rho: np.ndarray, cic: bool) -> np.ndarray:
    """CosmosCuda.cuh:1245 copy, :1266 FFT, :149-173 x filter, :120-148 / deconv,
    :1291 inverse FFT, :333-355 shift by N/2 and divide by N^2."""
    N = rho.shape[0]
    G = np.fft.fft2(green_lattice(N))
    D = mass_assignment_spectrum(N, cic)
    L = np.fft.fft2(rho.astype(np.complex128)) * G
    L = L * np.conj(D) / (np.abs(D) ** 2 + 0.001)
    lat = np.fft.ifft2(L) * (N * N)  # unnormalised inverse, like CUFFT_INVERSE
    return np.roll(lat.real, (N // 2, N // 2), axis=(0, 1)) / (N * N)


def gradient(phi: np.ndarray, gmult: float = 1.0) -> np.ndarray:
    """CosmosCuda.cuh:183-227: edge-clamped 4th-order central difference; (N, N, 2)."""
    N = phi.shape[0]

    def shifted(dy, dx):
        out = np.empty_like(phi)
        ys = np.arange(N) + dy
        xs = np.arange(N) + dx
        oky = (ys >= 0) & (ys < N)
        okx = (xs >= 0) & (xs < N)
        src = phi[np.clip(ys, 0, N - 1)][:, np.clip(xs, 0, N - 1)]
        mask = oky[:, None] & okx[None, :]
        out[:] = np.where(mask, src, phi)
        return out

    fx = (-shifted(0, 2) + 8 * shifted(0, 1) - 8 * shifted(0, -1) + shifted(0, -2)) / 12.0
    fy = (-shifted(2, 0) + 8 * shifted(1, 0) - 8 * shifted(-1, 0) + shifted(-2, 0)) / 12.0
    return np.stack([fx * gmult, fy * gmult], axis=-1)


def integrate(force, x, y, xo, yo, N: int, cic: bool, dt: float):
    """CosmosCuda.cuh:240-311 in FP64: returns new (x, y, xo, yo) as float32."""
    P = (x.size // 4) * 4
    x = x.copy(); y = y.copy(); xo = xo.copy(); yo = yo.copy()
    px = x[:P].astype(np.float64)
    py = y[:P].astype(np.float64)
    cx = np.trunc(x[:P]).astype(np.int64)
    cy = np.trunc(y[:P]).astype(np.int64)
    act = (cx >= 1) & (cx < N - 1) & (cy >= 1) & (cy < N - 1)
    idx = np.nonzero(act)[0]
    cx, cy = cx[idx], cy[idx]
    F = force.reshape(N * N, 2)
    c = cx + cy * N
    if cic:
        fx = px[idx] - cx
        fy = py[idx] - cy
        w = [(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy]
        cells = [c, c + 1, c + N, c + 1 + N]
        Fx = sum(F[cc, 0] * ww for cc, ww in zip(cells, w))
        Fy = sum(F[cc, 1] * ww for cc, ww in zip(cells, w))
    else:
        Fx, Fy = F[c, 0], F[c, 1]
    nx = 2 * px[idx] - xo[idx].astype(np.float64) + dt * Fx * dt
    ny = 2 * py[idx] - yo[idx].astype(np.float64) + dt * Fy * dt
    span = N - 4.0
    nx = np.where(nx < 2, nx + span, nx)
    ny = np.where(ny < 2, ny + span, ny)
    nx = np.where(nx > N - 2.0, nx - span, nx)
    ny = np.where(ny > N - 2.0, ny - span, ny)
    xo[idx] = x[idx]
    yo[idx] = y[idx]
    x[idx] = nx.astype(np.float32)
    y[idx] = ny.astype(np.float32)
    return x, y, xo, yo


def step(x, y, xo, yo, m, N: int, cic: bool, dt: float, gmult: float = 1.0):
    rho = deposit(x, y, m, N, cic)
    phi = potential(rho, cic)
    F = gradient(phi, gmult)
    return integrate(F, x, y, xo, yo, N, cic, dt), (rho, phi, F)


def blur_weights(R: int) -> np.ndarray:
    """Render blur kernel: 1/(r+1) for r < (R-1)/2, else 0 (CosmosCuda.cuh:954-966).

    Returned as [iy][ix] (row = y offset), float32 like the reference's table."""
    h = (R - 1) // 2
    d = np.arange(-h, h + 1, dtype=np.float64)
    r = np.sqrt(d[None, :] ** 2 + d[:, None] ** 2)
    return np.where(r < h, 1.0 / (r + 1.0), 0.0).astype(np.float32)


class Renderer:
    """Display frame of a density lattice (CosmosCuda.cuh:1249-1256).

    blur   k_calcBlurConvolution (:773-828): R x R weighted sum, zero outside
    minmax k_resetMinMax / k_calcMinMax (:630-743): the maximum starts at
           FLT_MIN and the block reduction pads its unused lanes with 0.0, so
           the frame extremes are min(min, 0) and max(max, 0, FLT_MIN)
    smooth k_initSmoothMinMax / k_smoothMinMax (:744-755): running extremes
           across frames, starting at (1e35, -1)
    scale  k_scaleWithMinMax (:756-772): 1.8 * ((v - lo) / (hi - lo))^0.25
    The blur is summed in FP64 here; the frame is compared with a tolerance."""

    def __init__(self, R: int = 3):
        self.R = R
        self.w = blur_weights(R).astype(np.float64)
        self.lo, self.hi = np.float32(1e35), np.float32(-1.0)

    def blur(self, rho: np.ndarray) -> np.ndarray:
        N = rho.shape[0]
        h = (self.R - 1) // 2
        p = np.zeros((N + 2 * h, N + 2 * h))
        p[h:h + N, h:h + N] = rho
        out = np.zeros((N, N))
        for iy in range(self.R):
            for ix in range(self.R):
                if self.w[iy, ix] != 0.0:
                    out += self.w[iy, ix] * p[iy:iy + N, ix:ix + N]
        return out

    def __call__(self, rho: np.ndarray) -> np.ndarray:
        b = self.blur(np.asarray(rho, np.float64))
        fmin = min(float(b.min()), 0.0)
        fmax = max(float(b.max()), 0.0, float(np.finfo(np.float32).tiny))
        self.lo = np.float32(min(float(self.lo), fmin))
        self.hi = np.float32(max(float(self.hi), fmax))
        lo, hi = float(self.lo), float(self.hi)
        return (1.8 * ((b - lo) / (hi - lo)) ** 0.25).astype(np.float32)
