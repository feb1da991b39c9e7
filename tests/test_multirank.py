"""The replica path of bench.py with two ranks on the CPU (gloo): the barrier,
the max-over-ranks time and the whole-job rate; the reference arm runs on
rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        bench.barrier(world)
        local_ms = 100.0 + 50.0 * rank  # rank 1 is the slower one
        max_ms = bench.reduce_max(local_ms, world, "gloo")
        rate = bench.replica_rate(1000, world, max_ms)
        # the reference arm prints from rank 0 only: other ranks return at once
        if rank != 0:
            assert bench.run_reference(None, world, rank) is None
        bench.barrier(world)
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as fh:
            fh.write(f"{max_ms} {rate}\n")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_rate(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in range(2):
        max_ms, rate = map(float, open(tmp_path / f"rank{r}.txt").read().split())
        assert max_ms == 150.0
        assert rate == pytest.approx(2 * 1000 / 0.150)
