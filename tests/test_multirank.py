"""The multi-rank host path of bench.py on CPU (gloo, world size 2): every rank times its own
batch, the reported step time is the slowest rank's, and ranks draw different queries (weak
scaling over independent replicas, no data-path collective)."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from gpu_nurbs_gb300 import synth
    assert bench.dist_env()[:2] == (rank, world)
    ts = [1.0 + rank, 2.0 + rank, 3.0 + rank]          # rank 1 is slower by 1 ms per step
    ms = bench.mean_step_ms_over_ranks(ts, world, "cpu")
    uv, _ = synth.query_params(64, 1000 + rank, "large")   # the seed bench.py gives this rank
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), ms=ms, uv=uv)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_report_the_slowest_and_draw_distinct_queries(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = (np.load(tmp_path / f"r{k}.npz") for k in (0, 1))
    assert float(r0["ms"]) == float(r1["ms"]) == pytest.approx(3.0)   # mean of rank 1's steps
    assert not np.array_equal(r0["uv"], r1["uv"])
