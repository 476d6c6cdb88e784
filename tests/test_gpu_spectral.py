"""Spectral force mode against the FP64 oracle (the reference's edge-clamped
stencil on the FP64 potential).

Tolerance: relative L2 force error <= 1e-5 over the lattice (the benchmark's
force-accuracy bar) and at the particles; edge cells (x or y in {0, 1, N-2,
N-1}, where the reference clamps the stencil) <= 1e-5 relative to the force
scale.  Trajectories: as in test_gpu_pm (max |dx| <= 1e-3 cells).
"""
import numpy as np
import pytest

from cosmossimulationwithcuda_gb300 import ics
from oracle import pm_oracle
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _spectral(lib, N, P, cic, dt=0.001, **kw):
    return lib.Simulation(N, P, cic=cic, dt=dt, force_mode=lib.FORCE_SPECTRAL, **kw)


def _oracle_force(rho, N, cic, g=1.0):
    o = pm_oracle.OraclePM(N, cic, 0.001, g, fp64=True)
    o.set_density(rho.astype(np.float64))
    o.potential()
    o.gradient()
    return o.force()


@pytest.mark.parametrize("N", [16, 64, 512, 2048])
@pytest.mark.parametrize("cic", [False, True])
def test_spectral_force_random_density(cosmos_lib, rng, N, cic):
    rho = (rng.random((N, N)) * 3.0).astype(np.float32)
    with _spectral(cosmos_lib, N, 4, cic, gravity_multiplier=1.25) as s:
        s.set_field(cosmos_lib.FIELD_DENSITY, rho)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        F = s.get_field(cosmos_lib.FIELD_FORCE)
    ref = _oracle_force(rho, N, cic, 1.25)
    assert rel_l2(F, ref) < 1e-5
    scale = np.sqrt(np.mean(ref ** 2))
    edges = [0, 1, N - 2, N - 1]
    assert np.abs(F[:, edges, 0] - ref[:, edges, 0]).max() < 1e-5 * scale * 10
    assert np.abs(F[edges, :, 1] - ref[edges, :, 1]).max() < 1e-5 * scale * 10


def test_spectral_force_disk_vs_gradient_mode(cosmos_lib):
    """Disk of 1M particles on 512^2: the spectral force is ~100x closer to FP64
    than the gradient of the FP32 potential (the reference algorithm)."""
    N, P, dt = 512, 1_000_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=5, scale=50.0)
    fields = {}
    for mode in (cosmos_lib.FORCE_GRADIENT, cosmos_lib.FORCE_SPECTRAL):
        with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=mode) as s:
            s.set_state(st)
            s.run_stage(cosmos_lib.STAGE_DEPOSIT)
            if mode == cosmos_lib.FORCE_GRADIENT:
                s.run_stage(cosmos_lib.STAGE_POTENTIAL)
            s.run_stage(cosmos_lib.STAGE_FORCE)
            fields[mode] = s.get_field(cosmos_lib.FIELD_FORCE)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.deposit(st.x, st.y, st.m)
    o.potential()
    o.gradient()
    ref = o.force()
    e_spec = rel_l2(fields[cosmos_lib.FORCE_SPECTRAL], ref)
    e_grad = rel_l2(fields[cosmos_lib.FORCE_GRADIENT], ref)
    assert e_spec < 1e-5
    assert e_spec < e_grad / 10


def test_spectral_uniform_1M_512_ngp_10_steps(cosmos_lib):
    """The small plain workload in spectral mode (edge cells populated)."""
    w = ics.WORKLOADS["uniform-1M-512-ngp"]
    st = ics.make_workload("uniform-1M-512-ngp")
    N, dt = w["N"], w["dt"]
    with _spectral(cosmos_lib, N, st.count, False, dt=dt) as s:
        s.set_state(st)
        s.step(10)
        s.synchronize()
        gx, gy, gxo, gyo, _ = s.get_particles()
    o = pm_oracle.OraclePM(N, False, dt, 1.0, fp64=True)
    ref = st.copy()
    o.step(ref.x, ref.y, ref.x_old, ref.y_old, ref.m, 10)
    keep = (st.x > 3) & (st.x < N - 3) & (st.y > 3) & (st.y < N - 3)
    assert np.abs(gx - ref.x)[keep].max() <= 1e-3
    assert np.abs(gy - ref.y)[keep].max() <= 1e-3


@pytest.mark.parametrize("sort_interval", [0, 4])
def test_spectral_disk_steps(cosmos_lib, sort_interval):
    N, P, dt = 256, 200_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=11, scale=25.0)
    with _spectral(cosmos_lib, N, P, True, dt=dt, sort_interval=sort_interval) as s:
        s.set_state(st)
        s.step(5)
        s.synchronize()
        gx, gy, *_ = s.get_particles()
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    ref = st.copy()
    o.step(ref.x, ref.y, ref.x_old, ref.y_old, ref.m, 5)
    keep = (st.x > 3) & (st.x < N - 3) & (st.y > 3) & (st.y < N - 3)
    assert np.abs(gx - ref.x)[keep].max() <= 1e-3
    assert np.abs(gy - ref.y)[keep].max() <= 1e-3
