"""Ensembles (include/cosmos_ensemble.h): many simulations of different N and
P stepped by one graph launch per step.

Each simulation must follow the step of a single cosmos_pm handle with the
same configuration on the tile path: positions after k steps within 1e-4
cells, the density within 1e-6 and the force within 1e-5 (relative L2) of the
single-simulation run with the spectral force; 1e-3, 1e-5 and 3e-4 with the
gradient force, whose FP32 potential differencing turns the reordered density
sums into ~1e-4 relative force noise.
(The two runs differ only in the order of float atomic additions.)"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

DT = 0.01


def _ics(N, P, kind, seed):
    from cosmossimulationwithcuda_gb300 import ics
    if P == 0:
        return None
    if kind == "disk":
        return ics.exponential_disk(P, N, DT, seed=seed, scale=N / 8)
    if kind == "binary":
        return ics.binary_star(P, N, DT, seed=seed)
    return ics.uniform(P, N, DT, seed=seed)


CASES = [  # (N, P, kind)
    (64, 4096, "disk"),
    (128, 8192, "uniform"),
    (64, 0, "disk"),
    (256, 20000, "disk"),
    (128, 4000, "binary"),
    (64, 2048, "uniform"),
]


def _run_pair(force_mode, steps, sort_interval=4, use_graph=True):
    from cosmossimulationwithcuda_gb300 import _lib
    Ns = [c[0] for c in CASES]
    Ps = [c[1] for c in CASES]
    states = [_ics(N, P, k, 100 + i) for i, (N, P, k) in enumerate(CASES)]
    with _lib.Ensemble(Ns, Ps, cic=True, dt=DT, force_mode=force_mode, sort_interval=sort_interval,
                       use_graph=use_graph) as ens:
        for i, st in enumerate(states):
            if st is not None:
                ens.set_state(i, st)
        ens.step(steps)
        ens.synchronize()
        got = [ens.get_particles(i) for i in range(len(CASES))]
        dens = [ens.get_field(i, _lib.FIELD_DENSITY) for i in range(len(CASES))]
        frc = [ens.get_field(i, _lib.FIELD_FORCE) for i in range(len(CASES))]
    want, wdens, wfrc = [], [], []
    for i, (N, P, _) in enumerate(CASES):
        with _lib.Simulation(N, max(P, 4), cic=True, dt=DT, force_mode=force_mode,
                             sort_interval=sort_interval) as s:
            if states[i] is not None:
                s.set_state(states[i])
            else:  # an empty simulation: one parked particle group
                s.clear()
            s.step(steps)
            s.synchronize()
            want.append(s.get_particles() if P else None)
            wdens.append(s.get_field(_lib.FIELD_DENSITY))
            wfrc.append(s.get_field(_lib.FIELD_FORCE))
    return got, want, dens, wdens, frc, wfrc


@pytest.mark.parametrize("force_mode", ["spectral", "gradient"])
def test_ensemble_matches_single_simulations(force_mode):
    from cosmossimulationwithcuda_gb300 import _lib
    fm = _lib.FORCE_SPECTRAL if force_mode == "spectral" else _lib.FORCE_GRADIENT
    got, want, dens, wdens, frc, wfrc = _run_pair(fm, steps=9)
    # the gradient mode differences an FP32 potential: reordered density sums
    # (1e-7) come out as ~1e-4 relative force noise, so its bound is looser
    tol, dtol, ftol = (1e-4, 1e-6, 1e-5) if force_mode == "spectral" else (1e-3, 1e-5, 3e-4)
    for i, (N, P, _) in enumerate(CASES):
        if P == 0:
            assert not dens[i].any() and not frc[i].any()
            continue
        for a, b in zip(got[i][:4], want[i][:4]):
            assert np.abs(a - b).max() <= tol, (i, np.abs(a - b).max())
        assert np.array_equal(got[i][4], want[i][4])  # masses untouched
        assert rel_l2(dens[i], wdens[i]) <= dtol, i
        assert rel_l2(frc[i], wfrc[i]) <= ftol, i


def test_ensemble_graph_and_direct_agree():
    from cosmossimulationwithcuda_gb300 import _lib
    a = _run_pair(_lib.FORCE_SPECTRAL, steps=5, use_graph=True)[0]
    b = _run_pair(_lib.FORCE_SPECTRAL, steps=5, use_graph=False)[0]
    for i, (N, P, _) in enumerate(CASES):
        if P:
            assert np.abs(a[i][0] - b[i][0]).max() <= 1e-4


def test_ensemble_identity_io_after_sort():
    """Particles are read and written by identity after the tile sort moved them."""
    from cosmossimulationwithcuda_gb300 import _lib, ics
    st = ics.exponential_disk(4096, 64, DT, seed=7, scale=8.0)
    with _lib.Ensemble([64, 64], [4096, 4096], dt=DT, sort_interval=2) as ens:
        ens.set_state(0, st)
        ens.set_state(1, st)
        ens.step(3)
        x, y, xo, yo, m = ens.get_particles(1)
        x0 = ens.get_particles(0)[0]
        assert np.array_equal(m, st.m.astype(np.float32))
        # rewrite identities [100, 200) of simulation 1 and read them back
        nx = np.full(100, 30.5, np.float32)
        ens.set_particles(1, nx, nx, nx, nx, None, offset=100)
        x2 = ens.get_particles(1)[0]
        assert np.array_equal(x2[100:200], nx)
        assert np.array_equal(x2[:100], x[:100]) and np.array_equal(x2[200:], x[200:])
        # simulation 0 is untouched by writes to simulation 1
        assert np.array_equal(ens.get_particles(0)[0], x0)
        ens.step(2)
        assert np.isfinite(ens.get_particles(1)[0]).all()


def test_ensemble_rejects_bad_configs():
    from cosmossimulationwithcuda_gb300 import _lib
    with pytest.raises(_lib.CosmosError):
        _lib.Ensemble([64], [4097])       # P not a multiple of 4
    with pytest.raises(_lib.CosmosError):
        _lib.Ensemble([100], [4096])      # N not a power of two
    with _lib.Ensemble([64, 128], [8, 8]) as ens:
        with pytest.raises(_lib.CosmosError):
            ens.get_particles(2, 1)       # no simulation 2
        with pytest.raises(_lib.CosmosError):
            ens.get_particles(0, 9)       # beyond P_0
        assert ens.launches_per_step() == 2 * 4


@pytest.mark.parametrize("persistent", [False, True])
def test_ensemble_members_match_fp64_oracle(persistent):
    """Members of an ensemble at the batched form's lattice sizes (256^2,
    512^2, 1024^2) against the FP64 oracle on each member's own GPU
    positions: the fused kernel's deposit <= 1e-6, the force the next step
    uses (computed from that deposit) <= 1e-5, and the positions after that
    step within 1e-3 cells of one FP64 oracle step (CosmosCuda.cuh:1209-1300)."""
    from cosmossimulationwithcuda_gb300 import _lib, ics
    from oracle import pm_oracle
    dt = 0.002
    members = [(256, 40_000, "binary", 31), (512, 400_000, "disk", 32), (1024, 1_200_000, "disk", 33),
               (512, 60_000, "binary", 34)]
    states = []
    for N, P, kind, seed in members:
        if kind == "binary":
            states.append(ics.binary_star(P, N, dt, seed=seed))
        else:
            states.append(ics.exponential_disk(P, N, dt, seed=seed, scale=N / 10.0))
    Ns = [m[0] for m in members]
    Ps = [m[1] for m in members]
    with _lib.Ensemble(Ns, Ps, cic=True, dt=dt, force_mode=_lib.FORCE_SPECTRAL, sort_interval=8,
                       persistent=persistent) as ens:
        for i, st in enumerate(states):
            ens.set_state(i, st)
        ens.step(5)
        ens.synchronize()
        before = [ens.get_particles(i) for i in range(len(members))]
        dens = [ens.get_field(i, _lib.FIELD_DENSITY) for i in range(len(members))]
        ens.step(1)
        ens.synchronize()
        after = [ens.get_particles(i) for i in range(len(members))]
        frc = [ens.get_field(i, _lib.FIELD_FORCE) for i in range(len(members))]
    pm_oracle.set_threads(pm_oracle.max_threads())
    for i, (N, P, _, _) in enumerate(members):
        x, y, xo, yo, m = before[i]
        o = pm_oracle.OraclePM(N, True, dt, 1.0, fp64=True)
        o.deposit(x, y, m)
        assert rel_l2(dens[i], o.density()) <= 1e-6, (i, rel_l2(dens[i], o.density()))
        o.potential()
        o.gradient()
        assert rel_l2(frc[i], o.force()) <= 1e-5, (i, rel_l2(frc[i], o.force()))
        rx, ry, rxo, ryo = x.copy(), y.copy(), xo.copy(), yo.copy()
        o.integrate(rx, ry, rxo, ryo)
        o.close()
        keep = (x > 3) & (x < N - 3) & (y > 3) & (y < N - 3)
        assert np.abs(after[i][0] - rx)[keep].max() <= 1e-3, i
        assert np.abs(after[i][1] - ry)[keep].max() <= 1e-3, i


PERSISTENT_CASES = [(128, 20000, "uniform"), (256, 40000, "uniform"), (512, 100000, "uniform"), (1024, 200000, "uniform"),
                    (256, 0, "uniform"), (512, 8000, "uniform")]


def _unit_mass_states(dt):
    from cosmossimulationwithcuda_gb300 import ics
    return [ics.uniform(P, N, dt, seed=200 + i) if P else None for i, (N, P, _) in enumerate(PERSISTENT_CASES)]


def _run_ensemble(persistent, steps, dt, cic=False, use_graph=True):
    from cosmossimulationwithcuda_gb300 import _lib
    states = _unit_mass_states(dt)
    with _lib.Ensemble([c[0] for c in PERSISTENT_CASES], [c[1] for c in PERSISTENT_CASES], cic=cic, dt=dt,
                       force_mode=_lib.FORCE_SPECTRAL, sort_interval=4, use_graph=use_graph,
                       persistent=persistent) as ens:
        if persistent:
            assert ens.launches_per_step() == 1
        for i, st in enumerate(states):
            if st is not None:
                ens.set_state(i, st)
        ens.step(steps)
        ens.synchronize()
        return ([ens.get_particles(i) for i in range(len(PERSISTENT_CASES))],
                [ens.get_field(i, _lib.FIELD_DENSITY) for i in range(len(PERSISTENT_CASES))])


@pytest.mark.parametrize("use_graph", [True, False])
def test_persistent_step_equals_graph_step_ngp(use_graph):
    """The one-launch persistent step runs the same bodies as the per-pass
    kernels: NGP with unit masses (every density sum exact) gives the same
    bits, including across re-sorts (sort every 4 steps, 9 steps)."""
    a_p, a_d = _run_ensemble(False, 9, 0.002)
    b_p, b_d = _run_ensemble(True, 9, 0.002, use_graph=use_graph)
    for i in range(len(PERSISTENT_CASES)):
        for x, y in zip(a_p[i], b_p[i]):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(a_d[i], b_d[i])


def test_persistent_step_cic_close_to_graph_step():
    a_p, a_d = _run_ensemble(False, 6, 0.002, cic=True)
    b_p, b_d = _run_ensemble(True, 6, 0.002, cic=True)
    for i, (N, P, _) in enumerate(PERSISTENT_CASES):
        if P:
            assert np.abs(a_p[i][0] - b_p[i][0]).max() <= 1e-4
            assert rel_l2(b_d[i], a_d[i]) <= 1e-6


def test_persistent_barrier_timeout_is_reported_and_recovers():
    """A grid barrier of the persistent step that never completes (one CTA
    skips its arrival) runs out after its bounded wait: every CTA returns, the
    status reaches cosmos_ensemble_synchronize as COSMOS_ERR_TIMEOUT, and the
    handle steps on normally once the hook is cleared."""
    from cosmossimulationwithcuda_gb300 import _lib
    dt = 0.002
    states = _unit_mass_states(dt)
    want = _run_ensemble(True, 2, dt)[0]
    with _lib.Ensemble([c[0] for c in PERSISTENT_CASES], [c[1] for c in PERSISTENT_CASES], cic=False, dt=dt,
                       force_mode=_lib.FORCE_SPECTRAL, sort_interval=4, persistent=True) as ens:
        for i, st in enumerate(states):
            if st is not None:
                ens.set_state(i, st)
        ens.test_barrier(1)
        with pytest.raises(_lib.CosmosError) as err:
            ens.step(1)
            ens.synchronize()
        assert err.value.code == -5  # COSMOS_ERR_TIMEOUT
        ens.test_barrier(0)
        for i, st in enumerate(states):  # the step that gave up is incomplete: start again
            if st is not None:
                ens.set_state(i, st)
        ens.step(2)
        ens.synchronize()
        got = [ens.get_particles(i) for i in range(len(PERSISTENT_CASES))]
    for i in range(len(PERSISTENT_CASES)):
        for x, y in zip(got[i], want[i]):
            np.testing.assert_array_equal(x, y)


def test_persistent_step_rejects_unsupported_configs():
    from cosmossimulationwithcuda_gb300 import _lib
    with pytest.raises(_lib.CosmosError):
        _lib.Ensemble([2048], [4096], persistent=True)  # lattice above 1024
    with pytest.raises(_lib.CosmosError):
        _lib.Ensemble([256], [4096], force_mode=_lib.FORCE_GRADIENT, persistent=True)
