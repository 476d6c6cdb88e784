"""Parity of the step at the headline's density: 20,000,000 particles on the
2048^2 CIC lattice, the exponential disk of scale 200 cells (the workload the
throughput is quoted on), through the path that is timed.

At this particle count the sorted state is cut into work items of 8192
particles (the most the fused kernel takes), almost every tile of the disk's
inner region holds far more than the window-free threshold, and the deposit
runs through the fused kernel's 32-bit fixed-point shared windows with the
scale 2^k < 2^31 / M_item.  Each check compares what that kernel produced
with the FP64 oracle (CPU) on the positions the GPU itself produced, so no
trajectory divergence enters the comparison:

  density after a step (the fused kernel's deposit of the new positions)
      against the FP64 deposit of those positions:        rel. L2 <= 1e-6
  force of the next step (computed from that density)
      against the FP64 force of the same positions:       rel. L2 <= 1e-5
      (over the lattice, and sampled at the particles with the CIC weights)
  positions after that step against one FP64 oracle step
      from the same positions:                             max |dx| <= 1e-3 cells
      (particles more than 3 cells inside the lattice edge)

Reference step under test: CosmosCuda.cuh:446-595 (deposit), :1245-1297
(FFT convolution), :174-229 (gradient), :231-312 (gather + update).
"""
import numpy as np
import pytest

from cosmossimulationwithcuda_gb300 import ics
from oracle import pm_oracle
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

WORKLOAD = "disk-20M-2048-cic"


def _cic_sample(F, x, y, N):
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


@pytest.fixture(scope="module")
def headline_state():
    return ics.make_workload(WORKLOAD)


@pytest.mark.parametrize("mode", ["spectral", "tc-fp16"])
def test_headline_fused_deposit_force_and_step_vs_fp64(cosmos_lib, headline_state, mode):
    w = ics.WORKLOADS[WORKLOAD]
    N, dt, st = w["N"], w["dt"], headline_state
    P = st.count
    fm = {"spectral": cosmos_lib.FORCE_SPECTRAL, "tc-fp16": cosmos_lib.FORCE_SPECTRAL_TC_FP16}[mode]
    pm_oracle.set_threads(pm_oracle.max_threads())
    with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=fm) as s:
        s.set_state(st)
        # step 1 sorts the state (tile order, 8192-particle items) and deposits
        # the new positions through the fused kernel's windows; step 2 runs
        # entirely on the fused kernel's density
        s.step(2)
        s.synchronize()
        x2, y2, xo2, yo2, m2 = s.get_particles()
        rho2 = s.get_field(cosmos_lib.FIELD_DENSITY)
        s.step(1)
        s.synchronize()
        F3 = s.get_field(cosmos_lib.FIELD_FORCE)  # the force step 3 used: from rho2
        x3, y3, xo3, yo3, _ = s.get_particles()
    np.testing.assert_array_equal(m2, st.m)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.deposit(x2, y2, m2)
    ref_rho = o.density()
    err_rho = rel_l2(rho2, ref_rho)
    assert err_rho <= 1e-6, f"fused-kernel density vs FP64 deposit: {err_rho:.3e}"
    np.testing.assert_array_equal(rho2 != 0, ref_rho != 0)
    o.potential()
    o.gradient()
    ref_F = o.force()
    err_F = rel_l2(F3, ref_F)
    assert err_F <= 1e-5, f"force from the fused-kernel density vs FP64: {err_F:.3e}"
    err_Fp = rel_l2(_cic_sample(F3, x2, y2, N), _cic_sample(ref_F, x2, y2, N))
    assert err_Fp <= 1e-5, f"force at the particles vs FP64: {err_Fp:.3e}"
    # one FP64 oracle step from the GPU's positions after step 2
    rx, ry, rxo, ryo = x2.copy(), y2.copy(), xo2.copy(), yo2.copy()
    o.integrate(rx, ry, rxo, ryo)
    o.close()
    keep = (x2 > 3) & (x2 < N - 3) & (y2 > 3) & (y2 < N - 3)
    assert np.abs(x3 - rx)[keep].max() <= 1e-3
    assert np.abs(y3 - ry)[keep].max() <= 1e-3
    assert np.abs(xo3 - rxo)[keep].max() <= 1e-3
