"""Checkpoint / resume and failure detection, all without a GPU fault:
allocation failures are injected on the host side of the library, and the
tensor-core column pass is made to wait on a completion signal that nothing
sends, so its bounded wait runs out and the host reads the status."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _uniform_ngp(lib, N=128, P=20000, seed=3):
    """NGP with unit masses: every density sum is an exact integer, so runs are
    reproducible bit for bit whatever the order of the atomic additions."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(4, N - 4, P).astype(np.float32)
    y = rng.uniform(4, N - 4, P).astype(np.float32)
    vx, vy = rng.normal(0.0, 0.02, (2, P)).astype(np.float32)
    return x, y, (x - vx).astype(np.float32), (y - vy).astype(np.float32), np.ones(P, np.float32)


@pytest.mark.parametrize("mode", ["gradient", "spectral"])
def test_checkpoint_resume_bit_exact(cosmos_lib, tmp_path, mode):
    N, P, k = 128, 20000, 6
    fm = cosmos_lib.FORCE_SPECTRAL if mode == "spectral" else cosmos_lib.FORCE_GRADIENT
    st = _uniform_ngp(cosmos_lib, N, P)
    path = str(tmp_path / "state.ckpt")
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.01, force_mode=fm) as a:
        a.set_particles(*st)
        a.step(2 * k)
        want = a.get_particles()
        assert a.steps_taken() == 2 * k
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.01, force_mode=fm) as b:
        b.set_particles(*st)
        b.step(k)
        b.save(path)
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.01, force_mode=fm) as c:
        c.load(path)
        assert c.steps_taken() == k
        c.step(k)
        got = c.get_particles()
        assert c.steps_taken() == 2 * k
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_checkpoint_rejects_bad_files(cosmos_lib, tmp_path):
    N, P = 64, 4000
    st = _uniform_ngp(cosmos_lib, N, P)
    path = str(tmp_path / "s.ckpt")
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.01) as s:
        s.set_particles(*st)
        s.save(path)
        s.load(path)  # round trip
    raw = open(path, "rb").read()
    with cosmos_lib.Simulation(2 * N, P, cic=False, dt=0.01) as other:
        with pytest.raises(cosmos_lib.CosmosError):
            other.load(path)  # different lattice
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.02) as other:
        with pytest.raises(cosmos_lib.CosmosError):
            other.load(path)  # different time step
    with cosmos_lib.Simulation(N, P, cic=False, dt=0.01) as s:
        trunc = str(tmp_path / "t.ckpt")
        open(trunc, "wb").write(raw[:-7])
        with pytest.raises(cosmos_lib.CosmosError):
            s.load(trunc)
        bad = bytearray(raw)
        bad[-5] ^= 0x40
        flip = str(tmp_path / "f.ckpt")
        open(flip, "wb").write(bytes(bad))
        with pytest.raises(cosmos_lib.CosmosError):
            s.load(flip)  # checksum
        with pytest.raises(cosmos_lib.CosmosError):
            s.load(str(tmp_path / "missing.ckpt"))


def test_injected_allocation_failures_leave_no_leak(cosmos_lib):
    """Every device allocation of create() can fail; the handle is not created,
    everything allocated before is released, and the next create works."""
    import ctypes
    rt = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue

    def used():
        if rt is None:
            return 0
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total))
        return total.value - free.value
    with cosmos_lib.Simulation(256, 100_000, force_mode=cosmos_lib.FORCE_SPECTRAL):
        pass
    base = used()
    failures = 0
    for n in range(1, 40):
        cosmos_lib.test_hook(cosmos_lib.TEST_FAIL_ALLOC, n)
        try:
            with cosmos_lib.Simulation(256, 100_000, force_mode=cosmos_lib.FORCE_SPECTRAL):
                pass
        except cosmos_lib.CosmosError as e:
            assert e.code == -3  # COSMOS_ERR_NOMEM
            failures += 1
        finally:
            cosmos_lib.test_hook(cosmos_lib.TEST_FAIL_ALLOC, 0)
    assert failures >= 20
    assert used() <= base + (64 << 20)  # nothing of the failed creates is left behind
    with cosmos_lib.Simulation(256, 100_000, force_mode=cosmos_lib.FORCE_SPECTRAL) as s:
        s.step(1)
        s.synchronize()


def test_tc_wait_timeout_is_reported_and_recovers(cosmos_lib, rng):
    N = 1024
    rho = (rng.random((N, N)) * 3.0).astype(np.float32)
    with cosmos_lib.Simulation(N, 4, cic=True, dt=0.001, force_mode=cosmos_lib.FORCE_SPECTRAL) as ref:
        ref.set_field(cosmos_lib.FIELD_DENSITY, rho)
        ref.run_stage(cosmos_lib.STAGE_FORCE)
        want = ref.get_field(cosmos_lib.FIELD_FORCE)
    with cosmos_lib.Simulation(N, 4, cic=True, dt=0.001, force_mode=cosmos_lib.FORCE_SPECTRAL_TC_FP16,
                               use_graph=False) as s:
        s.set_field(cosmos_lib.FIELD_DENSITY, rho)
        s.test_hook(cosmos_lib.TEST_TC_SKIP_MMA, 1)
        with pytest.raises(cosmos_lib.CosmosError) as err:
            s.run_stage(cosmos_lib.STAGE_FORCE)
            s.synchronize()
        assert err.value.code == -5  # COSMOS_ERR_TIMEOUT
        s.test_hook(cosmos_lib.TEST_TC_SKIP_MMA, 0)
        s.set_field(cosmos_lib.FIELD_DENSITY, rho)
        s.run_stage(cosmos_lib.STAGE_FORCE)
        s.synchronize()  # the status was cleared and the context is usable
        got = s.get_field(cosmos_lib.FIELD_FORCE)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


def test_copy_wait_timeout_is_reported_and_recovers(cosmos_lib):
    """The fused step kernel's bounded copy waits: announced bytes that never
    arrive make them run out; the status reaches cosmos_pm_synchronize as
    COSMOS_ERR_TIMEOUT, and after the hook is cleared the handle steps on
    exactly like a fresh one from the same state (NGP, unit masses)."""
    from cosmossimulationwithcuda_gb300 import ics
    N, P, dt = 256, 200_000, 0.002
    st = ics.uniform(P, N, dt, seed=8)
    with cosmos_lib.Simulation(N, P, cic=False, dt=dt, sort_interval=1) as ref:
        ref.set_state(st)
        ref.step(2)
        ref.synchronize()
        want = ref.get_particles()
    with cosmos_lib.Simulation(N, P, cic=False, dt=dt, sort_interval=1) as s:
        s.set_state(st)
        s.test_hook(cosmos_lib.TEST_COPY_WAIT, 1)
        with pytest.raises(cosmos_lib.CosmosError) as err:
            s.step(1)
            s.synchronize()
        assert err.value.code == -5  # COSMOS_ERR_TIMEOUT
        s.test_hook(cosmos_lib.TEST_COPY_WAIT, 0)
        s.set_state(st)  # the step that gave up is incomplete: start again
        s.step(2)
        s.synchronize()  # the status was cleared and the context is usable
        got = s.get_particles()
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
