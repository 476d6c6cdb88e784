"""Golden fixtures from the reference's own CUDA kernels (tests/golden/*.npz,
made by tests/golden/make_golden.py on the GPU: CosmosCuda.cuh's kernels
compiled for sm_103a, cuFFT, the Universe<K> launch sequence).

CPU tests pin the FP64 oracle to the reference; GPU tests check the CUDA path
against the same fixtures.  Tolerances (relative L2 over the lattice, absolute
cells for positions):
  density <= 1e-6, potential <= 1e-6, force <= 2e-5 (lattices of step 1; the
  reference is FP32 with float atomics and cuFFT)
  positions after step 1: max |dx| <= 1e-4 cells (or one float32 ulp of the
  coordinate, 1.2e-4 cells above 1024), every particle
  positions after k steps: max |dx| <= 1e-3 cells for particles starting more
  than 3 cells from the lattice edge (FP32 position rounding can flip an ulp
  where dt^2 F is close to half an ulp; NGP forces jump between cells)
  1M-particle 2048^2 case: the density (<= 1e-5) and force (<= 1e-4: the
  reference differences an FP32 potential, ~1e-4 from FP64) of the positions
  after k steps, at sampled cells (lattices of two slightly different
  trajectories: the reference's and the one under test; measured for the FP64
  oracle: 1.2e-6 and 4.2e-5)
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


def _inputs(c, d):
    """(x, y, x_old, y_old, m) of a case: stored, or (kind "icdisk")
    regenerated bit for bit by the counter-based generator."""
    if c["kind"] == "icdisk":
        from tests.golden.make_golden import make_ic_inputs
        inp = make_ic_inputs(c["N"], c["dt"], c["P"], c["seed"])
    else:
        inp = d
    return tuple(np.ascontiguousarray(inp[k], np.float32) for k in ("x", "y", "x_old", "y_old", "m"))


def _interior(x, y, N):
    return (x > 3) & (x < N - 3) & (y > 3) & (y < N - 3)


def check_against_golden(name, c, d, inputs, fields, s1, sk, nxt=None):
    """fields: (density, potential, force) of step 1 (cases with "fields");
    s1 / sk: positions after step 1 / after `steps`; nxt (kind "icdisk"):
    (density, force) of the positions after `steps`."""
    N = c["N"]
    if c["fields"]:
        rho, phi, F = fields
        assert rel_l2(rho, d["density"]) < 1e-6
        assert rel_l2(phi, d["potential"]) < 1e-6
        assert rel_l2(F, d["force"]) < 2e-5
    idx = d["idx"] if "idx" in d else slice(None)
    x1, y1, xo1, yo1 = (np.asarray(a)[idx] for a in s1)
    for got, key in ((x1, "x1"), (y1, "y1"), (xo1, "x_old1")):
        # 1e-4 cells, or one float32 ulp of the coordinate (1.2e-4 above 1024)
        tol = np.maximum(1e-4, np.spacing(np.abs(d[key])))
        assert np.all(np.abs(got - d[key]) <= tol), float(np.abs(got - d[key]).max())
    xk, yk, xok, yok = (np.asarray(a)[idx] for a in sk)
    keep = _interior(inputs[0][idx], inputs[1][idx], N)
    assert np.abs(xk - d["xk"])[keep].max() <= 1e-3
    assert np.abs(yk - d["yk"])[keep].max() <= 1e-3
    assert np.abs(xok - d["x_oldk"])[keep].max() <= 1e-3
    if nxt is not None:
        rho, F = nxt
        cells = d["cells"]
        assert rel_l2(np.asarray(rho).reshape(-1)[cells], d["density_next"]) < 1e-5
        assert rel_l2(np.asarray(F).reshape(-1, 2)[cells], d["force_next"]) < 1e-4


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_kernels(name):
    c = CASES[name]
    d = _load(name)
    o = pm_oracle.OraclePM(c["N"], c["cic"], c["dt"], 1.0, fp64=True)
    inputs = _inputs(c, d)
    x, y, xo, yo, m = [a.copy() for a in inputs]
    o.step(x, y, xo, yo, m, 1)
    fields = (o.density(), o.potential_field(), o.force())
    s1 = (x.copy(), y.copy(), xo.copy(), yo.copy())
    o.step(x, y, xo, yo, m, c["steps"] - 1)
    nxt = None
    if "cells" in d:
        o.deposit(x, y, m)
        o.potential()
        o.gradient()
        nxt = (o.density(), o.force())
    check_against_golden(name, c, d, inputs, fields, s1, (x, y, xo, yo), nxt)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_path_matches_reference_kernels(cosmos_lib, name):
    c = CASES[name]
    d = _load(name)
    args = _inputs(c, d)
    N, P = c["N"], args[0].size
    fields = None
    if c["fields"]:
        with cosmos_lib.Simulation(N, P, cic=c["cic"], dt=c["dt"]) as s:
            s.set_particles(*args)
            for stage in (cosmos_lib.STAGE_DEPOSIT, cosmos_lib.STAGE_POTENTIAL, cosmos_lib.STAGE_FORCE):
                s.run_stage(stage)
            fields = (s.get_field(cosmos_lib.FIELD_DENSITY), s.get_field(cosmos_lib.FIELD_POTENTIAL),
                      s.get_field(cosmos_lib.FIELD_FORCE))
    # sort_interval 2: tile order, shared-window gathers and fixed-point
    # deposits wherever a tile holds enough particles; spectral mode beside the
    # reference's gradient
    modes = [(0, cosmos_lib.FORCE_GRADIENT), (2, cosmos_lib.FORCE_GRADIENT)]
    if "cells" in d:
        modes.append((2, cosmos_lib.FORCE_SPECTRAL))
    for sort_interval, fm in modes:
        with cosmos_lib.Simulation(N, P, cic=c["cic"], dt=c["dt"], sort_interval=sort_interval, force_mode=fm) as s:
            s.set_particles(*args)
            s.step(1)
            s.synchronize()
            s1 = s.get_particles()[:4]
            s.step(c["steps"] - 1)
            s.synchronize()
            sk = s.get_particles()[:4]
            nxt = None
            if "cells" in d:  # the fused kernel's deposit of sk, and the next step's force from it
                rho = s.get_field(cosmos_lib.FIELD_DENSITY)
                s.step(1)
                s.synchronize()
                nxt = (rho, s.get_field(cosmos_lib.FIELD_FORCE))
        check_against_golden(name, c, d, args, fields, s1, sk, nxt)


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
