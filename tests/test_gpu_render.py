"""Display frames: the reference's render chain (CosmosCuda.cuh:1249-1256) on the GPU.

Checked against the numpy restatement (oracle/pm_np.py Renderer, FP64 blur;
frame values within 2e-5 absolute, on a 0..1.8 scale) and, bit for bit,
against the reference's own render kernels through the golden digests
(tests/golden/render2048.npz, manifest "render")."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pm_np
from tests.golden.make_golden import render_density

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 2e-5


def _sim(N, P=16, **kw):
    from cosmossimulationwithcuda_gb300 import _lib
    return _lib.Simulation(N, P, cic=True, dt=0.01, **kw)


@pytest.mark.parametrize("N,R", [(16, 3), (64, 3), (64, 5), (128, 7), (256, 3)])
def test_render_matches_oracle_sequence(N, R):
    """Three frames in a row: the running extremes grow with the second and
    hold through the third (smaller) one."""
    from cosmossimulationwithcuda_gb300 import _lib
    ren = pm_np.Renderer(R)
    with _sim(N, blur_r=R) as s:
        for seed, scale in [(1, 1e-4), (2, 5e-4), (3, 2e-5)]:
            rho = render_density(N, seed, scale)
            s.set_field(_lib.FIELD_DENSITY, rho)
            got = s.render_frame()
            want = ren(rho)
            assert np.abs(got - want).max() <= TOL


def test_render_blur_r1_is_blank():
    """BLUR_R = 1 leaves no nonzero weight (r < 0 never holds): a blank frame."""
    from cosmossimulationwithcuda_gb300 import _lib
    with _sim(32, blur_r=1) as s:
        s.set_field(_lib.FIELD_DENSITY, render_density(32, 5, 1e-3))
        assert not s.render_frame().any()


def test_render_invalid_blur_rejected():
    from cosmossimulationwithcuda_gb300 import _lib
    for r in (2, 17, -1):
        with pytest.raises(_lib.CosmosError):
            _sim(32, blur_r=r)


def test_render_bit_exact_vs_reference_kernels():
    """The reference's own render kernels (built with fast math) made these
    frames; ours must match them bit for bit."""
    from cosmossimulationwithcuda_gb300 import _lib
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        cases = json.load(f).get("render", {})
    assert cases, "render golden cases missing"
    for name, c in cases.items():
        g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        N = c["N"]
        with _sim(N, blur_r=c["blur_r"]) as s:
            for k, (seed, scale) in enumerate(c["frames"]):
                s.set_field(_lib.FIELD_DENSITY, render_density(N, seed, scale))
                frame = s.render_frame()
                assert np.array_equal(frame.reshape(-1)[g["cells"]], g["values"][k]), (name, k)
                assert hashlib.sha256(frame.tobytes()).hexdigest() == c["sha256"][k], (name, k)


def test_render_of_particles_uses_current_density():
    """After set_particles the density is stale: the frame deposits the current
    positions first, and after steps it shows the density the last step left."""
    from cosmossimulationwithcuda_gb300 import _lib, ics
    N, P = 64, 4096
    st = ics.exponential_disk(P, N, dt=0.01, seed=3, scale=N / 8)
    ren = pm_np.Renderer(3)
    with _lib.Simulation(N, P, cic=True, dt=0.01) as s:
        s.set_state(st)
        f0 = s.render_frame()
        rho0 = pm_np.deposit(st.x.astype(np.float64), st.y.astype(np.float64), st.m.astype(np.float64), N, True)
        assert np.abs(f0 - ren(rho0)).max() <= 1e-4
        s.step(3)
        f1 = s.render_frame()
        assert np.abs(f1 - ren(s.get_field(_lib.FIELD_DENSITY))).max() <= TOL


def test_frame_async_matches_sync():
    """An asynchronous frame equals the synchronous frame rendered right after
    it from the same density (the running extremes do not move in between),
    with the copy of the asynchronous one still in flight."""
    from cosmossimulationwithcuda_gb300 import _lib, ics
    N, P = 128, 8192
    st = ics.exponential_disk(P, N, dt=0.01, seed=4, scale=N / 8)
    with _lib.Simulation(N, P, cic=True, dt=0.01) as s:
        s.set_state(st)
        for _ in range(3):
            s.step(2)
            buf = np.empty((N, N), np.float32)
            t = s.frame_async(buf)
            sync = s.render_frame()
            s.wait(t)
            assert np.array_equal(buf, sync)
            assert sync.max() > 0
