"""bench.py's multi-rank path on the CPU: two gloo ranks (127.0.0.1).

The GPU arm runs one replica per GPU and reports the whole job: the
slowest rank's time over all ranks' lattice updates.  Here the same
helpers run over gloo, and the reference arm -- which rank 0 alone runs on
the host cores, the other ranks exiting without work -- runs under
torch.distributed.run with two processes."""
import json
import os
import socket
import subprocess
import sys

import pytest

import cases

ROOT = cases.ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_max(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.max_over_ranks(1.5 + rank, world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_takes_the_slowest_rank_over_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_max, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 2.5, 1: 2.5}


def test_whole_job_throughput_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.whole_job_mlups(256 ** 3, 400, 1, 0.8) == pytest.approx(256 ** 3 * 400 / 0.8 / 1e6)
    assert bench.whole_job_mlups(256 ** 3, 400, 4, 0.8) == pytest.approx(
        4 * bench.whole_job_mlups(256 ** 3, 400, 1, 0.8))


def test_reference_arm_under_two_ranks_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS=str(max(1, (os.cpu_count() or 2) // 2)))
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "MLUPS"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["metric"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
