"""The N > 1 path of bench.py on CPU: replicas (one process per GPU, no data
exchange on the fit path) whose job time is the slowest rank's, and the
reference arm running on rank 0 only.  Two gloo ranks on 127.0.0.1."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    ms = bench._max_over_ranks(10.0 + rank, ws, "cpu")  # rank 1 is the slow replica
    q.put((rank, ms, bench._replica_rate(1000, 3, ws, ms / 1e3)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank_and_rate_is_whole_job():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [11.0, 11.0]           # both ranks see the max
    assert all(abs(o[2] - 2 * 1000 * 3 / 0.011) < 1e-6 for o in out)  # total units over the slowest time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench._max_over_ranks(7.5, 1, "cpu") == 7.5
    assert bench._replica_rate(10, 2, 1, 0.5) == 40.0


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
