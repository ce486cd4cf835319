"""Host side of the multi-GPU bench path, on CPU: two gloo ranks.  The path
shards over views (replicas with disjoint poses, no collective on the data
path); the only exchange is the timing reduction, the slowest rank's time."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "webgpu-3dgs_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # each rank reports its own time; every rank gets the slowest
    out[rank] = bench.max_over_ranks(10.0 + 5.0 * rank, world, device="cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_ranks_render_disjoint_poses_and_rank0_is_the_single_gpu_workload():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "webgpu-3dgs_gb300"))
    import bench
    c0, c1 = bench.workload_cameras(64, 0), bench.workload_cameras(64, 1)
    assert all(not np.array_equal(a, b) for a, b in zip(c0, c1))
    single = bench.workload_cameras(64)
    assert all(np.array_equal(a, b) for a, b in zip(c0, single))
