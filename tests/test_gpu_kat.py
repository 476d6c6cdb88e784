"""Known-answer tests of the CUDA path, derived from the mathematics of the
particle-mesh step (the reference ships no tests or fixtures):

  * two equal masses feel equal and opposite forces along the line joining
    them, and none across it;
  * a uniform density gives no force (its potential is constant, so every
    difference of the reference's clamped stencil vanishes);
  * a step conserves total momentum when no particle wraps (the Green's
    lattice is even, so the pairwise forces cancel);
  * the force of one mass is the same wherever it sits (translation
    invariance of the periodic convolution), away from the clamped edges.

Each runs in the reference-faithful gradient mode and in the spectral mode
(FP32 passes), and the force tests also in the tensor-core split modes.
Tolerances are relative to the force scale of the case.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = ["gradient", "spectral", "tc-fp16", "tc-bf16"]


def _mode(lib, name):
    return {"gradient": lib.FORCE_GRADIENT, "spectral": lib.FORCE_SPECTRAL,
            "tc-fp16": lib.FORCE_SPECTRAL_TC_FP16, "tc-bf16": lib.FORCE_SPECTRAL_TC_BF16}[name]


def _force_of_particles(lib, N, mode, x, y, m, cic=False):
    """Force field of the density deposited from (x, y, m)."""
    P = x.size
    with lib.Simulation(N, P, cic=cic, dt=0.01, force_mode=_mode(lib, mode), use_graph=False) as s:
        s.set_particles(x, y, x, y, m)
        s.run_stage(lib.STAGE_DEPOSIT)
        if mode == "gradient":
            s.run_stage(lib.STAGE_POTENTIAL)
        s.run_stage(lib.STAGE_FORCE)
        s.synchronize()
        return s.get_field(lib.FIELD_FORCE).astype(np.float64)


def _tol(mode):
    # FP32 passes ~1e-6; the reference's FP32 differencing of the potential
    # (gradient mode) ~1e-5 at these sizes; 16-bit split tensor-core DFTs ~1e-5
    return {"gradient": 2e-5, "spectral": 2e-6, "tc-fp16": 2e-5, "tc-bf16": 5e-5}[mode]


@pytest.mark.parametrize("mode", MODES)
def test_two_masses_equal_and_opposite(cosmos_lib, mode):
    N = 1024  # the tensor-core modes start at 1024^2
    c = N // 2
    x = np.array([c - 3.5, c + 3.5, -10, -10], np.float32)  # NGP cells c - 4 and c + 3
    y = np.array([c + 0.5, c + 0.5, -10, -10], np.float32)
    m = np.array([1.0, 1.0, 0.0, 0.0], np.float32)
    F = _force_of_particles(cosmos_lib, N, mode, x, y, m)
    f1 = F[c, c - 4]
    f2 = F[c, c + 3]
    scale = np.abs(F).max()  # the errors of the passes scale with the whole field
    assert f1[0] > 0 and f2[0] < 0  # attraction: the force is +grad(phi)
    assert abs(f1[0]) > 0.01 * scale
    assert abs(f1[0] + f2[0]) < 10 * _tol(mode) * scale
    assert abs(f1[1]) < 10 * _tol(mode) * scale and abs(f2[1]) < 10 * _tol(mode) * scale


@pytest.mark.parametrize("mode", MODES)
def test_uniform_density_has_no_force(cosmos_lib, rng, mode):
    N = 1024
    with cosmos_lib.Simulation(N, 4, cic=True, dt=0.01, force_mode=_mode(cosmos_lib, mode), use_graph=False) as s:
        rho_r = (rng.random((N, N)) * 2.0).astype(np.float32)
        s.set_field(cosmos_lib.FIELD_DENSITY, rho_r)
        if mode == "gradient":
            s.run_stage(cosmos_lib.STAGE_POTENTIAL)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        scale = np.abs(s.get_field(cosmos_lib.FIELD_FORCE)).max()  # force scale of a unit-order density
        s.set_field(cosmos_lib.FIELD_DENSITY, np.ones((N, N), np.float32))
        if mode == "gradient":
            s.run_stage(cosmos_lib.STAGE_POTENTIAL)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        s.synchronize()
        F = s.get_field(cosmos_lib.FIELD_FORCE)
    assert np.abs(F).max() < 10 * _tol(mode) * scale


@pytest.mark.parametrize("mode", ["gradient", "spectral"])
@pytest.mark.parametrize("cic", [False, True])
def test_momentum_conserved_without_wraps(cosmos_lib, rng, mode, cic):
    N, P, dt = 256, 40_000, 0.05  # dt^2 F well above the float resolution of the positions
    x = rng.uniform(64, N - 64, P).astype(np.float32)
    y = rng.uniform(64, N - 64, P).astype(np.float32)
    m = rng.lognormal(0.0, 0.3, P).astype(np.float32)
    with cosmos_lib.Simulation(N, P, cic=cic, dt=dt, force_mode=_mode(cosmos_lib, mode)) as s:
        s.set_particles(x, y, x, y, m)
        s.step(1)
        s.synchronize()
        xs, ys, xos, yos, _ = s.get_particles()
    m64 = m.astype(np.float64)
    for a, ao in ((xs, xos), (ys, yos)):
        dv = a.astype(np.float64) - ao.astype(np.float64)  # = dt^2 F of the one step (started at rest)
        dp = np.sum(m64 * dv)
        assert np.abs(dv).max() > 1e-3
        assert abs(dp) < 1e-3 * np.sum(m64 * np.abs(dv))


@pytest.mark.parametrize("mode", ["gradient", "spectral"])
def test_force_of_one_mass_is_translation_invariant(cosmos_lib, mode):
    N = 512
    fields = []
    for (cx, cy) in ((200, 180), (300, 330)):
        x = np.array([cx + 0.5, -10, -10, -10], np.float32)
        y = np.array([cy + 0.5, -10, -10, -10], np.float32)
        m = np.array([1.0, 0.0, 0.0, 0.0], np.float32)
        F = _force_of_particles(cosmos_lib, N, mode, x, y, m)
        fields.append(F[cy - 60:cy + 60, cx - 60:cx + 60])
    scale = np.abs(fields[0]).max()
    assert np.abs(fields[0] - fields[1]).max() < 10 * _tol(mode) * scale
