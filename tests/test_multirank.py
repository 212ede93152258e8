"""The bench's multi-rank logic on CPU: two gloo ranks.

Every rank runs an independent replica (no data-path collective); the ranks
meet only at barriers and at the max-over-ranks reduction of the timed
region, and rank 0 alone prints the JSON line.  These tests run that logic
with world_size 2 on the gloo backend, without a GPU.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_body(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        bench.barrier(ws)
        ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
        ms_max = bench.max_over_ranks(ms, ws, "cpu")
        value = bench.job_value(ws, 1_000_000, 4, ms_max)
        bench.barrier(ws)
        out.put((rank, ms_max, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_body, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ms_max, value in got:
        assert ms_max == 15.0  # every rank sees the slowest rank's time
        # 2 replicas x 1 M points x 4 steps in 15 ms
        assert value == pytest.approx(2 * 1_000_000 * 4 / 0.015 / 1e6)


def test_job_value_single_rank_is_points_over_time():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_value(1, 100_000_000, 10, 85.0) == pytest.approx(100e6 * 10 / 0.085 / 1e6)


def test_reference_arm_under_torchrun_two_ranks():
    """bench.py --impl reference launched like the multi-GPU driver: rank 0
    alone runs the CPU baseline and prints one JSON line; rank 1 exits 0.
    The arm loads no GPU code: only the oracle's libraries are mapped, and its
    config object is the one our arm prints for the same workload."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--points", "30000"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["value"] > 0
    assert line["libraries_loaded"] and all(p.startswith("oracle/") for p in line["libraries_loaded"])
    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import oracle as O

    spec, W, Ov, B, _, _ = bench.workload(2, 30000, O.synth_config)
    xyz, bb = O.synth_cloud(spec, O.synth_config(2)[5])
    p = O.params(bb, spec.n, W, Ov, B)
    assert line["config"] == bench.workload_config(2, spec, W, Ov, B, p.ncells, p.ngrid)
