"""Golden fixtures from the reference's own CUDA kernels (tests/golden/*.npz,
made by tests/golden/make_golden.py on the GPU: CosmosCuda.cuh's kernels
compiled for sm_103a, cuFFT, the Universe<K> launch sequence).

CPU tests pin the FP64 oracle to the reference; GPU tests check the CUDA path
against the same fixtures.  Tolerances (relative L2 over the lattice, absolute
cells for positions):
  density <= 1e-6, potential <= 1e-6, force <= 2e-5 (lattices of step 1; the
  reference is FP32 with float atomics and cuFFT)
  positions after step 1: max |dx| <= 1e-4 cells, every particle
  positions after k steps: max |dx| <= 1e-3 cells for particles starting more
  than 3 cells from the lattice edge (FP32 position rounding can flip an ulp
  where dt^2 F is close to half an ulp; NGP forces jump between cells)
"""
import json
import os

import numpy as np
import pytest

from oracle import pm_oracle
from tests.conftest import rel_l2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)["cases"]


CASES = _cases()


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def _interior(d, N):
    return (d["x"] > 3) & (d["x"] < N - 3) & (d["y"] > 3) & (d["y"] < N - 3)


def check_against_golden(name, c, d, fields, s1, sk):
    N = c["N"]
    if c["fields"]:
        rho, phi, F = fields
        assert rel_l2(rho, d["density"]) < 1e-6
        assert rel_l2(phi, d["potential"]) < 1e-6
        assert rel_l2(F, d["force"]) < 2e-5
    x1, y1, xo1, yo1 = s1
    assert np.abs(x1 - d["x1"]).max() <= 1e-4
    assert np.abs(y1 - d["y1"]).max() <= 1e-4
    assert np.abs(xo1 - d["x_old1"]).max() <= 1e-4
    xk, yk, xok, yok = sk
    keep = _interior(d, N)
    assert np.abs(xk - d["xk"])[keep].max() <= 1e-3
    assert np.abs(yk - d["yk"])[keep].max() <= 1e-3
    assert np.abs(xok - d["x_oldk"])[keep].max() <= 1e-3


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_kernels(name):
    c = CASES[name]
    d = _load(name)
    o = pm_oracle.OraclePM(c["N"], c["cic"], c["dt"], 1.0, fp64=True)
    x, y, xo, yo, m = [d[k].copy() for k in ("x", "y", "x_old", "y_old", "m")]
    o.step(x, y, xo, yo, m, 1)
    fields = (o.density(), o.potential_field(), o.force())
    s1 = (x.copy(), y.copy(), xo.copy(), yo.copy())
    o.step(x, y, xo, yo, m, c["steps"] - 1)
    check_against_golden(name, c, d, fields, s1, (x, y, xo, yo))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_path_matches_reference_kernels(cosmos_lib, name):
    c = CASES[name]
    d = _load(name)
    N, P = c["N"], d["x"].size
    args = (d["x"], d["y"], d["x_old"], d["y_old"], d["m"])
    fields = None
    if c["fields"]:
        with cosmos_lib.Simulation(N, P, cic=c["cic"], dt=c["dt"]) as s:
            s.set_particles(*args)
            for stage in (cosmos_lib.STAGE_DEPOSIT, cosmos_lib.STAGE_POTENTIAL, cosmos_lib.STAGE_FORCE):
                s.run_stage(stage)
            fields = (s.get_field(cosmos_lib.FIELD_DENSITY), s.get_field(cosmos_lib.FIELD_POTENTIAL),
                      s.get_field(cosmos_lib.FIELD_FORCE))
    for sort_interval in (0, 2):
        with cosmos_lib.Simulation(N, P, cic=c["cic"], dt=c["dt"], sort_interval=sort_interval) as s:
            s.set_particles(*args)
            s.step(1)
            s.synchronize()
            s1 = s.get_particles()[:4]
            s.step(c["steps"] - 1)
            s.synchronize()
            sk = s.get_particles()[:4]
        check_against_golden(name, c, d, fields, s1, sk)


def _render_cases():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f).get("render", {})


@pytest.mark.parametrize("name", sorted(_render_cases()))
def test_render_oracle_vs_reference_frames(name):
    """The numpy render chain (oracle/pm_np.py Renderer) against the frames the
    reference's own render kernels made, at the sampled cells."""
    from oracle import pm_np
    from tests.golden.make_golden import render_density
    c = _render_cases()[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    ren = pm_np.Renderer(c["blur_r"])
    N = c["N"]
    for k, (seed, scale) in enumerate(c["frames"]):
        frame = ren(render_density(N, seed, scale))
        assert np.abs(frame.reshape(-1)[g["cells"]] - g["values"][k]).max() <= 2e-5
