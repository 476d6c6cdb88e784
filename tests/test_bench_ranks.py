"""The bench's multi-rank host logic on CPU (gloo, world_size 2): every rank
meets at the barrier, the timed region is the slowest rank's, and under
torchrun the reference arm prints one line from rank 0 while the other rank
exits without work.  Replicas only: no data-path collective."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, values, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    bench.barrier(ws)
    out[rank] = bench.max_over_ranks(values[rank], ws)
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo():
    import torch.multiprocessing as mp
    ws, port = 2, _free_port()
    values = [3.25, 7.5]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(ws, port, values, out), nprocs=ws, join=True)
        got = dict(out)
    assert got == {0: 7.5, 1: 7.5}


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    bench.barrier(1)


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "3", "--cpu-seconds", "0.2", "--particles", "40000",
           "--workload", "uniform-1M-512-ngp"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_line_carries_the_contract_keys():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3", "--cpu-seconds", "0.2",
           "--particles", "40000", "--workload", "uniform-1M-512-ngp"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "uniform-1M-512-ngp"
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
