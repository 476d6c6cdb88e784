"""cosmos_pm_autotune: the sort granularity / cadence search and its cache."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_caches(tmp_path):
    from cosmossimulationwithcuda_gb300 import _lib, ics
    N, P = 256, 200_000
    st = ics.exponential_disk(P, N, 0.002, seed=9, scale=N / 10)
    cache = str(tmp_path / "tune.txt")
    g, itv, ms = _lib.autotune(st, N, dt=0.002, steps=16, cache_path=cache)
    assert g in (4, 5, 6) and itv in (8, 16, 24, 32, 48, 64, 0) and ms > 0
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and lines[0].startswith(f"N={N} ")
    # a hit returns the stored choice and leaves the file alone
    g2, itv2, ms2 = _lib.autotune(st, N, dt=0.002, steps=16, cache_path=cache)
    assert (g2, itv2) == (g, itv) and abs(ms2 - ms) <= 1e-3 * ms + 1e-6
    assert open(cache).read().splitlines() == lines
    # the chosen configuration runs the same step
    with _lib.Simulation(N, P, dt=0.002, force_mode=_lib.FORCE_SPECTRAL, sort_granularity=g if itv else -1,
                         sort_interval=itv) as a, \
            _lib.Simulation(N, P, dt=0.002, force_mode=_lib.FORCE_SPECTRAL) as b:
        a.set_state(st)
        b.set_state(st)
        a.step(5)
        b.step(5)
        xa, xb = a.get_particles()[0], b.get_particles()[0]
    assert np.abs(xa - xb).max() <= 1e-4


def test_autotune_rejects_bad_arguments():
    from cosmossimulationwithcuda_gb300 import _lib, ics
    st = ics.uniform(1024, 64, 0.01, seed=1)
    with pytest.raises(_lib.CosmosError):
        _lib.autotune(st, 64, dt=0.01, steps=0)
    with pytest.raises(_lib.CosmosError):
        _lib.autotune(st, 100, dt=0.01, steps=4)  # N not a power of two
