"""Seeded initial conditions on the device (cosmos_pm_generate) against the
float32 restatement (oracle/ic_np.py): bit for bit, every family."""
import numpy as np
import pytest

from oracle import ic_np

pytestmark = pytest.mark.gpu

N, DT = 1024, 0.002

CASES = {
    "uniform": dict(kind=ic_np.UNIFORM, seed=11, center_x=512.0, center_y=400.0, scale=300.0, mass=2.0,
                    dispersion=3.0, bulk_vx=0.5),
    "exp_disk": dict(kind=ic_np.EXP_DISK, seed=12, center_x=512.0, center_y=512.0, scale=60.0, rmax=400.0,
                     mass=1e5, mass_sigma=0.3, spin=1.0, dispersion=0.05),
    "plummer": dict(kind=ic_np.PLUMMER, seed=13, center_x=300.0, center_y=700.0, scale=25.0, rmax=200.0,
                    mass=5e4, spin=-1.0, dispersion=0.1, bulk_vy=-2.0, g=1.5),
    "ring_disk": dict(kind=ic_np.RING_DISK, seed=14, center_x=0.25, center_y=0.75, scale=0.2, mass=1.0,
                      spin=0.005, bulk_vx=2.5e-5, bulk_vy=-5e-5, black_hole=True, total_particles=300_000),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_generate_bit_exact(cosmos_lib, name):
    p = dict(CASES[name])
    kind = p.pop("kind")
    P, count, offset = 300_000, 200_003, 50_000
    with cosmos_lib.Simulation(N, P, cic=True, dt=DT) as s:
        s.generate(kind, count, offset, **p)
        got = s.get_particles(count, offset)
    want = ic_np.generate(kind, count, first=offset, N=N, dt=DT, **p)
    for a, b, f in zip(got, want, ("x", "y", "x_old", "y_old", "m")):
        assert np.array_equal(a, b), (name, f, int(np.sum(a != b)))


def test_generate_split_calls_and_after_sort(cosmos_lib):
    """Positions depend only on (seed, identity): two calls equal one, also
    when the particles have been re-sorted internally in between."""
    p = dict(seed=21, center_x=512.0, center_y=512.0, scale=80.0, mass=1.0, spin=1.0)
    P = 100_000
    with cosmos_lib.Simulation(N, P, cic=True, dt=DT, sort_interval=1) as s:
        s.generate(cosmos_lib.IC_EXP_DISK, P, 0, **p)
        one = s.get_particles()
        s.step(2)  # sorts: internal order differs from identity order now
        s.generate(cosmos_lib.IC_EXP_DISK, 40_000, 0, **p)
        s.generate(cosmos_lib.IC_EXP_DISK, 60_000, 40_000, **p)
        two = s.get_particles()
    assert np.array_equal(one[0], two[0]) and np.array_equal(one[1], two[1])
    assert np.array_equal(one[2], two[2])


def test_generate_rejects_bad_arguments(cosmos_lib):
    with cosmos_lib.Simulation(64, 100, dt=DT) as s:
        with pytest.raises(cosmos_lib.CosmosError):
            s.generate(7, 10)
        with pytest.raises(cosmos_lib.CosmosError):
            s.generate(cosmos_lib.IC_EXP_DISK, 10, 95, scale=5.0)  # beyond P
        with pytest.raises(cosmos_lib.CosmosError):
            s.generate(cosmos_lib.IC_RING_DISK, 10, scale=0.2)      # total_particles missing
