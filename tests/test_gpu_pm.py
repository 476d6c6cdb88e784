"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances (relative L2 unless stated), against the FP64 oracle on identical
inputs:
  density  <= 1e-6   (FP32 atomics, order-dependent rounding)
  potential <= 2e-6  (FP32 FFT convolution)
  force (gradient mode) <= 3e-4 on lattices with 1e5-range potentials: the
      reference's own FP32 algorithm sits at ~1e-4 from FP64 because it
      differences an FP32 potential; on small cases <= 2e-5
  gather/update: bit-exact against the FP32 oracle given the same force field
  positions after k steps: max |dx| <= 1e-3 cells, particles within 3 cells of
      the lattice edge (wrap candidates) excluded
  cell keys and sort permutations: bit-exact
"""
import numpy as np
import pytest

from cosmossimulationwithcuda_gb300 import ics
from oracle import pm_oracle
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _sim(lib, N, P, cic, dt=0.01, **kw):
    return lib.Simulation(N, P, cic=cic, dt=dt, **kw)


def _random_state(rng, P, N, margin=0.0, vel=0.02):
    x = rng.uniform(margin, N - margin, P).astype(np.float32)
    y = rng.uniform(margin, N - margin, P).astype(np.float32)
    xo = (x + rng.normal(0, vel, P)).astype(np.float32)
    yo = (y + rng.normal(0, vel, P)).astype(np.float32)
    m = rng.lognormal(0.0, 0.3, P).astype(np.float32)
    return ics.ParticleState(x, y, xo, yo, m)


@pytest.mark.parametrize("N", [16, 64, 512, 2048])
@pytest.mark.parametrize("cic", [False, True])
def test_potential_matches_oracle(cosmos_lib, rng, N, cic):
    rho = rng.random((N, N)).astype(np.float32)
    rho[rng.random((N, N)) < 0.5] = 0
    with _sim(cosmos_lib, N, 4, cic) as s:
        s.set_field(cosmos_lib.FIELD_DENSITY, rho)
        s.run_stage(cosmos_lib.STAGE_POTENTIAL)
        phi = s.get_field(cosmos_lib.FIELD_POTENTIAL)
    o = pm_oracle.OraclePM(N, cic, 0.01, 1.0, fp64=True)
    o.set_density(rho.astype(np.float64))
    o.potential()
    assert rel_l2(phi, o.potential_field()) < 2e-6


@pytest.mark.parametrize("N", [16, 256])
def test_potential_single_mass_is_green(cosmos_lib, N):
    """One unit mass (NGP): phi = G shifted to the cell, / 1.001."""
    rho = np.zeros((N, N), np.float32)
    rho[N // 3, N // 5] = 1.0
    with _sim(cosmos_lib, N, 4, False) as s:
        s.set_field(cosmos_lib.FIELD_DENSITY, rho)
        s.run_stage(cosmos_lib.STAGE_POTENTIAL)
        phi = s.get_field(cosmos_lib.FIELD_POTENTIAL)
    from oracle import pm_np
    expect = np.roll(pm_np.green_lattice(N), (N // 3, N // 5), axis=(0, 1)) / 1.001
    np.testing.assert_allclose(phi, expect, rtol=0, atol=2e-6 * np.abs(expect).max())


@pytest.mark.parametrize("N", [64, 1024])
def test_gradient_matches_oracle(cosmos_lib, rng, N):
    phi = (rng.random((N, N)) * 100.0).astype(np.float32)
    with _sim(cosmos_lib, N, 4, True, gravity_multiplier=1.5) as s:
        s.set_field(cosmos_lib.FIELD_POTENTIAL, phi)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        F = s.get_field(cosmos_lib.FIELD_FORCE)
    o = pm_oracle.OraclePM(N, True, 0.01, 1.5, fp64=True)
    o.set_potential(phi.astype(np.float64))
    o.gradient()
    assert rel_l2(F, o.force()) < 1e-6


@pytest.mark.parametrize("cic", [False, True])
@pytest.mark.parametrize("N,P", [(64, 4099), (512, 1 << 18)])
def test_deposit_matches_oracle(cosmos_lib, rng, N, P, cic):
    st = _random_state(rng, P, N, margin=-1.0)  # includes inactive particles outside the window
    with _sim(cosmos_lib, N, P, cic) as s:
        s.set_state(st)
        s.run_stage(cosmos_lib.STAGE_DEPOSIT)
        rho = s.get_field(cosmos_lib.FIELD_DENSITY)
    o = pm_oracle.OraclePM(N, cic, 0.01, 1.0, fp64=True)
    o.deposit(st.x, st.y, st.m)
    ref = o.density()
    assert rel_l2(rho, ref) < 1e-6
    np.testing.assert_array_equal(rho != 0, ref != 0)


def test_deposit_ngp_integer_masses_exact(cosmos_lib, rng):
    """Equal unit masses under NGP: every cell is an integer count, so the
    order of the atomics cannot change the result."""
    N, P = 512, 1 << 20
    st = ics.uniform(P, N, 0.002, seed=3)
    with _sim(cosmos_lib, N, P, False, dt=0.002) as s:
        s.set_state(st)
        s.run_stage(cosmos_lib.STAGE_DEPOSIT)
        rho = s.get_field(cosmos_lib.FIELD_DENSITY)
    o = pm_oracle.OraclePM(N, False, 0.002, 1.0, fp64=True)
    o.deposit(st.x, st.y, st.m)
    np.testing.assert_array_equal(rho.astype(np.float64), o.density())


@pytest.mark.parametrize("cic", [False, True])
def test_integrate_bit_exact(cosmos_lib, rng, cic):
    N, P = 256, 100003
    st = _random_state(rng, P, N, margin=-1.5, vel=0.3)
    # include wrap cases near both edges
    st.x[:64] = np.linspace(1.0, 2.2, 64, dtype=np.float32)
    st.y[64:128] = np.linspace(N - 2.5, N - 1.01, 64, dtype=np.float32)
    F = (rng.standard_normal((N, N, 2)) * 50.0).astype(np.float32)
    dt = 0.01
    with _sim(cosmos_lib, N, P, cic, dt=dt) as s:
        s.set_state(st)
        s.set_field(cosmos_lib.FIELD_FORCE, F)
        s.run_stage(cosmos_lib.STAGE_INTEGRATE)
        gx, gy, gxo, gyo, _ = s.get_particles()
    x, y, xo, yo = st.x.copy(), st.y.copy(), st.x_old.copy(), st.y_old.copy()
    pm_oracle.integrate_f32_exact(F, N, cic, dt, x, y, xo, yo)
    np.testing.assert_array_equal(gx, x)
    np.testing.assert_array_equal(gy, y)
    np.testing.assert_array_equal(gxo, xo)
    np.testing.assert_array_equal(gyo, yo)
    # trailing P % 4 = 3 particles are never touched (CosmosCuda.cuh:239-242)
    np.testing.assert_array_equal(gx[-3:], st.x[-3:])


def _interior(st, N, margin=3.0):
    return (st.x > margin) & (st.x < N - margin) & (st.y > margin) & (st.y < N - margin)


def test_uniform_1M_512_ngp_10_steps(cosmos_lib):
    """The small plain workload: 2^20 particles, 512^2, NGP, dt 0.002, 10 steps."""
    w = ics.WORKLOADS["uniform-1M-512-ngp"]
    st = ics.make_workload("uniform-1M-512-ngp")
    N, dt = w["N"], w["dt"]
    with _sim(cosmos_lib, N, st.count, False, dt=dt) as s:
        s.set_state(st)
        s.step(10)
        s.synchronize()
        gx, gy, gxo, gyo, _ = s.get_particles()
    o = pm_oracle.OraclePM(N, False, dt, 1.0, fp64=True)
    ref = st.copy()
    o.step(ref.x, ref.y, ref.x_old, ref.y_old, ref.m, 10)
    keep = _interior(st, N)
    assert np.abs(gx - ref.x)[keep].max() <= 1e-3
    assert np.abs(gy - ref.y)[keep].max() <= 1e-3
    assert np.abs(gxo - ref.x_old)[keep].max() <= 1e-3


@pytest.mark.parametrize("sort_interval", [0, 3])
def test_disk_cic_steps(cosmos_lib, sort_interval):
    """Exponential disk, CIC, 5 steps: positions against the FP64 oracle,
    with and without the tile sort."""
    N, P, dt = 256, 200_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=11, scale=25.0)
    with _sim(cosmos_lib, N, P, True, dt=dt, sort_interval=sort_interval) as s:
        s.set_state(st)
        s.step(5)
        s.synchronize()
        gx, gy, gxo, gyo, gm = s.get_particles()
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    ref = st.copy()
    o.step(ref.x, ref.y, ref.x_old, ref.y_old, ref.m, 5)
    keep = _interior(st, N)
    np.testing.assert_array_equal(gm, st.m)
    assert np.abs(gx - ref.x)[keep].max() <= 1e-3
    assert np.abs(gy - ref.y)[keep].max() <= 1e-3


def test_force_field_error_vs_fp64_disk(cosmos_lib):
    """Force field of a disk (deposit -> potential -> gradient) against FP64."""
    N, P, dt = 512, 1_000_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=5, scale=50.0)
    with _sim(cosmos_lib, N, P, True, dt=dt) as s:
        s.set_state(st)
        for stage in (cosmos_lib.STAGE_DEPOSIT, cosmos_lib.STAGE_POTENTIAL, cosmos_lib.STAGE_FORCE):
            s.run_stage(stage)
        F = s.get_field(cosmos_lib.FIELD_FORCE)
        phi = s.get_field(cosmos_lib.FIELD_POTENTIAL)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o.deposit(st.x, st.y, st.m)
    o.potential()
    o.gradient()
    assert rel_l2(phi, o.potential_field()) < 2e-6
    # the gradient of an FP32 potential: the reference algorithm's own error floor
    assert rel_l2(F, o.force()) < 3e-4


def test_tile_keys_bit_exact(cosmos_lib, rng):
    N, P = 2048, 300_001
    x = rng.uniform(-3, N + 3, P).astype(np.float32)
    y = rng.uniform(-3, N + 3, P).astype(np.float32)
    x[:5] = [np.nan, np.inf, -np.inf, 1e30, 0.999999]
    with _sim(cosmos_lib, N, 4, True) as s:
        for g in (0, 3, 5, 8):
            np.testing.assert_array_equal(s.tile_keys(x, y, g), pm_oracle.sort_keys(x, y, N, g))


@pytest.mark.parametrize("P", [5, 4096, 1_000_003])
def test_sort_permutation_bit_exact(cosmos_lib, rng, P):
    N = 1024
    st = _random_state(rng, P, N, margin=-2.0)
    st.x[: P // 3] = st.x[0]  # heavy ties: stability matters
    with _sim(cosmos_lib, N, P, True, sort_interval=0, sort_granularity=5) as s:
        s.set_state(st)
        perm = s.sort()
        Pq = (P // 4) * 4
        keys = pm_oracle.sort_keys(st.x[:Pq], st.y[:Pq], N, 5)
        expect = pm_oracle.stable_sort_perm(keys)
        np.testing.assert_array_equal(perm[:Pq], expect)
        np.testing.assert_array_equal(perm[Pq:], np.arange(Pq, P, dtype=np.uint32))
        # identity-addressed reads see the original particles
        gx, gy, gxo, gyo, gm = s.get_particles()
        np.testing.assert_array_equal(gx, st.x)
        np.testing.assert_array_equal(gm, st.m)


def test_sorted_and_unsorted_steps_identical_ngp(cosmos_lib):
    """NGP with unit masses is order-independent, so sorting must not change
    a single bit of the trajectory; graph replay must match direct launches."""
    N, P, dt = 512, 1 << 18, 0.002
    st = ics.uniform(P, N, dt, seed=9)
    outs = []
    for kw in (dict(sort_interval=0, use_graph=False), dict(sort_interval=2, use_graph=True),
               dict(sort_interval=0, use_graph=True)):
        with _sim(cosmos_lib, N, P, False, dt=dt, **kw) as s:
            s.set_state(st)
            s.step(6)
            s.synchronize()
            outs.append(s.get_particles())
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("mode", ["spectral", "gradient"])
def test_step_batching_and_dependent_launches_identical_ngp(cosmos_lib, mode):
    """At 1024^2 the step's kernels launch as programmatic dependents and runs
    of steps without a sort go out as four-step graphs: step(13) must equal
    13 single steps and the direct (graph-free) launches bit for bit (NGP,
    unit masses: every density sum is exact, so the runs are deterministic)."""
    N, P, dt = 1024, 1 << 18, 0.002
    fm = cosmos_lib.FORCE_SPECTRAL if mode == "spectral" else cosmos_lib.FORCE_GRADIENT
    st = ics.uniform(P, N, dt, seed=4)
    outs = []
    for use_graph, batched in ((True, True), (True, False), (False, True)):
        with _sim(cosmos_lib, N, P, False, dt=dt, sort_interval=6, use_graph=use_graph, force_mode=fm) as s:
            s.set_state(st)
            if batched:
                s.step(13)
            else:
                for _ in range(13):
                    s.step(1)
            assert s.steps_taken() == 13
            s.synchronize()
            outs.append(list(s.get_particles()) + [s.get_field(cosmos_lib.FIELD_DENSITY)])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_kernel_launch_accounting(cosmos_lib):
    """kernels_launched counts every enqueued kernel: a plain step adds
    launches_per_step, a step that re-sorts adds the sort's kernels on top,
    a four-step graph adds four steps' worth."""
    N, P = 256, 40_000
    st = ics.uniform(P, N, 0.002, seed=2)
    with _sim(cosmos_lib, N, P, True, dt=0.002, sort_interval=8, force_mode=cosmos_lib.FORCE_SPECTRAL) as s:
        per = s.launches_per_step()
        assert per == 4  # row R2C, columns, row C2R (with the y-edge corrections), fused step
        s.set_state(st)
        k0 = s.kernels_launched()
        s.step(1)  # first-step deposit + sort + step
        k1 = s.kernels_launched()
        assert k1 - k0 > per + 1
        s.step(1)
        assert s.kernels_launched() - k1 == per
        k2 = s.kernels_launched()
        s.step(4)  # one four-step graph (no sort inside)
        assert s.kernels_launched() - k2 == 4 * per
        s.synchronize()


@pytest.mark.parametrize("cic", [False, True])
@pytest.mark.parametrize("sort_interval", [0, 1])
def test_fused_step_deposits_new_positions(cosmos_lib, cic, sort_interval):
    """After a step the density field holds the deposit of the NEW positions
    (the fused kernel's next-step deposit), in both the tile and global paths."""
    N, P, dt = 256, 300_000, 0.001
    st = ics.exponential_disk(P, N, dt, seed=21, scale=30.0)
    with _sim(cosmos_lib, N, P, cic, dt=dt, sort_interval=sort_interval) as s:
        s.set_state(st)
        s.step(3)
        s.synchronize()
        gx, gy, gxo, gyo, gm = s.get_particles()
        rho = s.get_field(cosmos_lib.FIELD_DENSITY)
    o = pm_oracle.OraclePM(N, cic, dt, 1.0, fp64=True)
    o.deposit(gx, gy, gm)
    assert rel_l2(rho, o.density()) < 1e-6


def test_fused_step_large_drift_fallbacks(cosmos_lib):
    """Fast particles leave their tile windows between sorts: the global
    fallbacks of the fused kernel must keep the trajectory exact."""
    N, P, dt = 256, 100_000, 0.01
    rng = np.random.default_rng(3)
    st = _random_state(rng, P, N, margin=20.0, vel=0.0)
    v = rng.normal(0.0, 300.0, (2, P))  # ~3 cells per step
    st.x_old[:] = st.x - (v[0] * dt).astype(np.float32)
    st.y_old[:] = st.y - (v[1] * dt).astype(np.float32)
    with _sim(cosmos_lib, N, P, True, dt=dt, sort_interval=1000) as s:
        s.set_state(st)
        s.step(6)
        s.synchronize()
        gx, gy, gxo, gyo, gm = s.get_particles()
        rho = s.get_field(cosmos_lib.FIELD_DENSITY)
    o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    ref = st.copy()
    o.step(ref.x, ref.y, ref.x_old, ref.y_old, ref.m, 6)
    keep = _interior(st, N, 25.0) & _interior(ref, N, 3.0)
    assert np.abs(gx - ref.x)[keep].max() <= 1e-3
    assert np.abs(gy - ref.y)[keep].max() <= 1e-3
    o2 = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
    o2.deposit(gx, gy, gm)
    assert rel_l2(rho, o2.density()) < 1e-6


def test_positions_async_ordered_and_internal(cosmos_lib, rng):
    N, P = 256, 50_000
    st = _random_state(rng, P, N)
    with _sim(cosmos_lib, N, P, True, dt=0.001, sort_interval=1) as s:
        s.set_state(st)
        s.step(3)
        hx = np.empty(P, np.float32)
        hy = np.empty(P, np.float32)
        t = s.positions_async(hx, hy, ordered=True)
        s.wait(t)
        assert s.poll(t)
        gx, gy, *_ = s.get_particles()
        np.testing.assert_array_equal(hx, gx)
        np.testing.assert_array_equal(hy, gy)
        ix = np.empty(P, np.float32)
        iy = np.empty(P, np.float32)
        t2 = s.positions_async(ix, iy, ordered=False)
        s.wait(t2)
        np.testing.assert_array_equal(np.sort(ix), np.sort(gx))


def test_set_particles_partial_after_sort(cosmos_lib, rng):
    N, P = 128, 10_000
    st = _random_state(rng, P, N)
    with _sim(cosmos_lib, N, P, True, sort_interval=0) as s:
        s.set_state(st)
        s.sort()
        new = _random_state(rng, 100, N)
        s.set_particles(new.x, new.y, new.x_old, new.y_old, new.m, offset=500)
        gx, gy, gxo, gyo, gm = s.get_particles()
        exp = st.x.copy()
        exp[500:600] = new.x
        np.testing.assert_array_equal(gx, exp)
        sub = s.get_particles(count=100, offset=500)
        np.testing.assert_array_equal(sub[4], new.m)


def test_clear_parks_particles(cosmos_lib, rng):
    N, P = 64, 1000
    with _sim(cosmos_lib, N, P, True) as s:
        s.set_state(_random_state(rng, P, N))
        s.clear()
        s.step(2)
        s.synchronize()
        gx, gy, gxo, gyo, _ = s.get_particles()
        assert np.all(gx == -10.0) and np.all(gyo == -10.0)
        s.run_stage(cosmos_lib.STAGE_DEPOSIT)
        assert np.all(s.get_field(cosmos_lib.FIELD_DENSITY) == 0)


def test_errors_are_status_codes(cosmos_lib):
    with pytest.raises(cosmos_lib.CosmosError) as e:
        cosmos_lib.Simulation(1000, 4)
    assert e.value.code == -1
    with _sim(cosmos_lib, 64, 100, True) as s:
        with pytest.raises(cosmos_lib.CosmosError) as e:
            s.set_particles(np.zeros(10, np.float32), np.zeros(10, np.float32), offset=95)
        assert e.value.code == -4
        with pytest.raises(cosmos_lib.CosmosError):
            s.run_stage(99)


def test_diagnostics_fp64(cosmos_lib, rng):
    N, P = 128, 8192
    dt = float(np.float32(0.01))  # the library stores dt as float
    st = _random_state(rng, P, N, margin=4, vel=0.05)
    with _sim(cosmos_lib, N, P, True, dt=dt) as s:
        s.set_state(st)
        ke, pe, px, py = s.diagnostics()
    vx = (st.x.astype(np.float64) - st.x_old) / dt
    vy = (st.y.astype(np.float64) - st.y_old) / dt
    m = st.m.astype(np.float64)
    assert np.abs(vx).max() * dt < (N - 4) / 2  # no wrapped particles in this state
    np.testing.assert_allclose(ke, 0.5 * np.sum(m * (vx ** 2 + vy ** 2)), rtol=1e-12)
    np.testing.assert_allclose(px, np.sum(m * vx), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(py, np.sum(m * vy), rtol=1e-9, atol=1e-9)


def test_diagnostics_unwraps_wrapped_particles(cosmos_lib):
    """A particle just wrapped keeps xOld on the far side; its velocity is the
    displacement modulo the wrap period N - 4."""
    N, dt = 64, float(np.float32(0.01))
    x = np.array([2.5, 30.0, 30.0, 30.0], np.float32)
    xo = np.array([2.5 + (N - 4) - 0.001, 30.0, 30.0, 30.0], np.float32)  # moved -0.001 across the edge
    y = np.full(4, 30.0, np.float32)
    m = np.ones(4, np.float32)
    with _sim(cosmos_lib, N, 4, True, dt=dt) as s:
        s.set_particles(x, y, xo, y, m)
        ke, pe, px, py = s.diagnostics()
    d = (np.float64(x[0]) - np.float64(xo[0])) + (N - 4)
    assert abs(px - d / dt) <= 1e-9 * abs(d / dt) + 1e-12
    assert abs(ke - 0.5 * (d / dt) ** 2) <= 1e-9 * ke


@pytest.mark.parametrize("use_graph", [True, False])
def test_stage_times_of_profiled_steps(cosmos_lib, use_graph):
    """Profiled steps (graph-launched with event nodes between the stages, or
    direct launches) report positive stage times and advance the state
    exactly like unprofiled steps (NGP, unit masses: bit-exact)."""
    N, P, dt = 1024, 1 << 18, 0.002
    st = ics.uniform(P, N, dt, seed=6)
    outs = []
    for profile in (True, False):
        with _sim(cosmos_lib, N, P, False, dt=dt, sort_interval=4, use_graph=use_graph,
                  force_mode=cosmos_lib.FORCE_SPECTRAL) as s:
            s.set_state(st)
            s.set_profiling(profile)
            sorts = 0
            for _ in range(6):
                s.step(1)
                if profile:
                    t = s.stage_times()
                    assert t[1] > 0 and t[3] > 0  # force passes, fused step
                    sorts += int(t[4] > 0)
            s.synchronize()
            if profile:
                assert sorts == 2  # steps 1 and 5
            outs.append(s.get_particles())
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
