"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks (replicas, no
data-path collective; only the timing reduction crosses ranks)."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        w, r, local = bench.dist_env()
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        slow = bench.slowest_rank_ms(ms, w)
        dist.barrier()
        q.put((r, w, local, slow, bench.whole_job_vps(w, 32, 100, slow)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ws, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(ws))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert [g[2] for g in got] == [0, 1]
    # every rank reports the slowest rank's 15 ms; the job moved 2 x 32 x 100 vectors
    assert all(g[3] == 15.0 for g in got)
    assert all(abs(g[4] - 2 * 32 * 100 / 0.015) < 1e-6 for g in got)


def test_single_rank_needs_no_process_group():
    assert bench.slowest_rank_ms(7.5, 1) == 7.5
    assert bench.whole_job_vps(1, 32, 10, 5.0) == 32 * 10 / 0.005


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun only rank 0 runs the reference arm; rank 1 prints nothing
    and exits 0 (no grammar is built)."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", GMR_CACHE_DIR="/nonexistent")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
