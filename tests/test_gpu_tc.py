"""Tensor-core split-precision column FFTs (COSMOS_FORCE_SPECTRAL_TC_FP16 /
_BF16) against the FP64 oracle and the FP32 spectral mode.

Tolerances (relative L2 of the force over the lattice against FP64):
FP16 split <= 1e-5 (the benchmark's force-accuracy bar; the split carries
22 significant bits), BF16 split <= 1e-4 (16 bits).  Trajectories over 5 steps
within 1e-3 cells of the FP32 spectral mode.
"""
import numpy as np
import pytest

from cosmossimulationwithcuda_gb300 import ics
from oracle import pm_oracle
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"fp16": 1e-5, "bf16": 1e-4}


def _mode(lib, prec):
    return lib.FORCE_SPECTRAL_TC_FP16 if prec == "fp16" else lib.FORCE_SPECTRAL_TC_BF16


def _oracle_force(rho, N, cic, g=1.0):
    o = pm_oracle.OraclePM(N, cic, 0.001, g, fp64=True)
    o.set_density(rho.astype(np.float64))
    o.potential()
    o.gradient()
    F = o.force()
    o.close()
    return F


def _force(lib, N, mode, rho, cic=True, g=1.0):
    with lib.Simulation(N, 4, cic=cic, dt=0.001, force_mode=mode, gravity_multiplier=g) as s:
        s.set_field(lib.FIELD_DENSITY, rho)
        s.run_stage(lib.STAGE_FORCE)
        s.synchronize()
        return s.get_field(lib.FIELD_FORCE)


@pytest.mark.parametrize("N", [1024, 2048, 4096])
@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_tc_force_random_density(cosmos_lib, rng, N, prec):
    rho = (rng.random((N, N)) * 3.0).astype(np.float32)
    F = _force(cosmos_lib, N, _mode(cosmos_lib, prec), rho, g=1.25)
    ref = _oracle_force(rho, N, True, 1.25)
    err = rel_l2(F, ref)
    assert err < TOL[prec], err
    # the edge corrections still hold (x edges: Fx, y edges: Fy)
    scale = np.sqrt(np.mean(ref ** 2))
    edges = [0, 1, N - 2, N - 1]
    assert np.abs(F[:, edges, 0] - ref[:, edges, 0]).max() < 100 * TOL[prec] * scale
    assert np.abs(F[edges, :, 1] - ref[edges, :, 1]).max() < 100 * TOL[prec] * scale


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_tc_force_disk(cosmos_lib, prec):
    """A clustered density (an exponential disk of 2M particles on 2048^2):
    the FP16 range scale must hold over a large dynamic range."""
    N, P, dt = 2048, 2_000_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=8, scale=200.0)
    with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=_mode(cosmos_lib, prec)) as s:
        s.set_state(st)
        s.run_stage(cosmos_lib.STAGE_DEPOSIT)
        rho = s.get_field(cosmos_lib.FIELD_DENSITY)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        s.synchronize()
        F = s.get_field(cosmos_lib.FIELD_FORCE)
    ref = _oracle_force(rho, N, True)
    assert rel_l2(F, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_tc_steps_follow_fp32_spectral(cosmos_lib, prec):
    N, P, dt = 1024, 400_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=9, scale=100.0)
    out = {}
    for mode in (cosmos_lib.FORCE_SPECTRAL, _mode(cosmos_lib, prec)):
        with cosmos_lib.Simulation(N, P, cic=True, dt=dt, force_mode=mode) as s:
            s.set_state(st)
            s.step(5)
            s.synchronize()
            out[mode] = s.get_particles()
    a, b = out[cosmos_lib.FORCE_SPECTRAL], out[_mode(cosmos_lib, prec)]
    assert np.abs(a[0] - b[0]).max() <= 1e-3 and np.abs(a[1] - b[1]).max() <= 1e-3


def test_tc_rejects_unsupported_lattice(cosmos_lib):
    with pytest.raises(cosmos_lib.CosmosError):
        cosmos_lib.Simulation(512, 4, force_mode=cosmos_lib.FORCE_SPECTRAL_TC_FP16)
