"""Edge cases of the step on the GPU, against the FP64 oracle.

- An empty state and a state of fewer than four particles: every stage runs,
  and the result equals the oracle's (the reference steps particles in groups
  of four, so a state of three particles never moves and deposits nothing).
- Heavy bodies (black holes) among a disk's particles: a particle heavier
  than 1/128 of its work item's mass deposits with global float atomics
  instead of the item's fixed-point window; the density the fused kernel
  deposits must still match the FP64 deposit (<= 1e-6 relative L2, also with
  the heavy bodies' cells left out) and the force of the next step the FP64
  force (<= 1e-5).
- The largest lattices of the benchmark configurations (4096^2 and 8192^2):
  the timed path's density and force against FP64, as at 2048^2 in
  test_gpu_headline.py.

Reference step under test: CosmosCuda.cuh:1209-1300 (deposit :446-595,
convolution :1245-1297, gradient :174-229, gather + update :231-312).
"""
import numpy as np
import pytest

from cosmossimulationwithcuda_gb300 import ics
from oracle import pm_oracle
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cic", [False, True])
@pytest.mark.parametrize("sort_interval", [0, 1])
def test_empty_state_runs_every_stage(cosmos_lib, cic, sort_interval):
    N = 64
    with cosmos_lib.Simulation(N, 0, cic=cic, dt=0.01, force_mode=cosmos_lib.FORCE_SPECTRAL,
                               sort_interval=sort_interval) as s:
        s.step(3)
        s.synchronize()
        assert s.steps_taken() == 3
        assert all(a.size == 0 for a in s.get_particles())
        assert not s.get_field(cosmos_lib.FIELD_DENSITY).any()
        assert not s.get_field(cosmos_lib.FIELD_FORCE).any()
        ke, pe, px, py = s.diagnostics()
        assert (ke, pe, px, py) == (0.0, 0.0, 0.0, 0.0)
        assert s.render_frame().shape == (N, N)


@pytest.mark.parametrize("P", [1, 3])
def test_fewer_than_four_particles_match_oracle(cosmos_lib, P):
    N, dt = 64, 0.01
    rng = np.random.default_rng(P)
    x = (rng.random(P) * 40 + 10).astype(np.float32)
    y = (rng.random(P) * 40 + 10).astype(np.float32)
    xo = (x - 0.01).astype(np.float32)
    yo = (y + 0.02).astype(np.float32)
    m = np.ones(P, np.float32)
    with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=cosmos_lib.FORCE_SPECTRAL) as s:
        s.set_particles(x, y, xo, yo, m)
        s.step(4)
        s.synchronize()
        gx, gy, gxo, gyo, gm = s.get_particles()
    rx, ry, rxo, ryo = x.copy(), y.copy(), xo.copy(), yo.copy()
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.step(rx, ry, rxo, ryo, m.copy(), 4)
    o.close()
    np.testing.assert_array_equal(gx, rx)
    np.testing.assert_array_equal(gy, ry)
    np.testing.assert_array_equal(gxo, rxo)
    np.testing.assert_array_equal(gyo, ryo)
    np.testing.assert_array_equal(gm, m)


def test_heavy_bodies_take_the_global_path(cosmos_lib):
    N, P, dt = 512, 300_000, 0.002
    st = ics.exponential_disk(P, N, dt, seed=41, scale=50.0)
    rng = np.random.default_rng(41)
    heavy = rng.choice(P, 12, replace=False)
    st.m[heavy] = np.float32(300.0) * st.m.mean()  # far above 1/128 of a 2048-particle item
    with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=cosmos_lib.FORCE_SPECTRAL, sort_interval=1) as s:
        s.set_state(st)
        s.step(2)
        s.synchronize()
        x2, y2, _, _, m2 = s.get_particles()
        rho2 = s.get_field(cosmos_lib.FIELD_DENSITY)
        s.step(1)
        s.synchronize()
        F3 = s.get_field(cosmos_lib.FIELD_FORCE)
    np.testing.assert_array_equal(m2, st.m)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.deposit(x2, y2, m2)
    ref = o.density()
    assert rel_l2(rho2, ref) <= 1e-6
    light = np.ones((N, N), bool)
    for i in heavy:
        cx, cy = int(x2[i]), int(y2[i])
        light[max(cy - 1, 0):cy + 3, max(cx - 1, 0):cx + 3] = False
    assert rel_l2(rho2[light], ref[light]) <= 1e-6
    o.potential()
    o.gradient()
    assert rel_l2(F3, o.force()) <= 1e-5
    o.close()


@pytest.mark.parametrize("N,P", [(4096, 2_000_000), (8192, 4_000_000)])
def test_largest_lattices_fused_density_and_force_vs_fp64(cosmos_lib, N, P):
    dt = 0.001
    st = ics.exponential_disk(P, N, dt, seed=43, scale=200.0 * N / 2048)
    pm_oracle.set_threads(pm_oracle.max_threads())
    with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=cosmos_lib.FORCE_SPECTRAL) as s:
        s.set_state(st)
        s.step(2)
        s.synchronize()
        x2, y2, _, _, m2 = s.get_particles()
        rho2 = s.get_field(cosmos_lib.FIELD_DENSITY)
        s.step(1)
        s.synchronize()
        F3 = s.get_field(cosmos_lib.FIELD_FORCE)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.deposit(x2, y2, m2)
    assert rel_l2(rho2, o.density()) <= 1e-6
    o.potential()
    o.gradient()
    assert rel_l2(F3, o.force()) <= 1e-5
    o.close()
