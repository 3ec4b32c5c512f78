"""The multi-rank bench path on CPU: each rank of a 2-rank gloo group runs
the same replica workload; the job time is the slowest rank's and the rate
counts every rank's units (weak scaling, no data-path collective)."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as td

    import bench

    td.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    job = bench.max_over_ranks(ms, "cpu")
    out[rank] = (job, bench.whole_job_rate(1e6, world, job))
    td.destroy_process_group()


def test_two_replicas_max_time_and_whole_job_rate():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0][0] == out[1][0] == pytest.approx(15.0)
    # 1e6 units per rank, 2 ranks, 15 ms -> 133.3 M units/s
    assert out[0][1] == pytest.approx(2e6 / 15e-3 / 1e6)
