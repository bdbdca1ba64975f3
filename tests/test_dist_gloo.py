"""The N > 1 path of bench.py on the CPU: world_size 2 over gloo on 127.0.0.1.  The bench
runs one replica per GPU (no data-path collective); the host side reduces the timings:
the time is the maximum over ranks and the units the sum, every rank passes the same
barrier, and only rank 0 runs the reference arm."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    env_ws, env_rank, env_local = bench.dist_env()
    dist = bench.dist_init(env_ws)
    bench.dist_barrier(dist)
    t = bench.dist_max(dist, 1.5 + rank)        # per-rank elapsed time
    units = bench.dist_sum(dist, 100.0 * (rank + 1))  # units each replica processed
    bench.dist_barrier(dist)
    ran_reference = []

    class Args:
        warmup, steps = 3, 1

    if env_rank != 0:  # the reference arm: ranks other than 0 exit at once
        bench.run_reference(Args(), env_ws, env_rank)
        ran_reference.append("returned")
    Path(out_dir, f"rank{rank}.txt").write_text(f"{env_ws} {env_rank} {env_local} {t} {units} {ran_reference}")
    dist.destroy_process_group()


def test_two_replicas_reduce_timings(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = (tmp_path / "rank0.txt").read_text().split(" ", 5)
    r1 = (tmp_path / "rank1.txt").read_text().split(" ", 5)
    for r, rank in ((r0, 0), (r1, 1)):
        assert r[0] == "2" and r[1] == str(rank) and r[2] == str(rank)
        assert float(r[3]) == 2.5 and float(r[4]) == 300.0
    assert "returned" in r1[5] and "returned" not in r0[5]


def test_single_process_has_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.dist_init(1) is None
    assert bench.dist_max(None, 3.0) == 3.0 and bench.dist_sum(None, 3.0) == 3.0
