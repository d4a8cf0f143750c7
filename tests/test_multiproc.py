"""Multi-process path on CPU: world_size-2 gloo ranks each step their own replica of a scene (the
solver does not shard: replicas only, no collective on the data path), and the bench's whole-job
aggregation (cell-steps of all ranks / slowest rank's time) is computed through torch.distributed."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import time

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle
    from em_lab_gb300 import configs

    oracle.set_threads(1)
    sc = configs.random_scene(size=(20, 18, 16), pml=3, seed=4)
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    dist.barrier()
    t0 = time.perf_counter()
    o.step(25)
    el = time.perf_counter() - t0 + 0.01 * rank  # ranks finish at different times
    cells = float(np.prod(sc.grid.size)) * 25
    value, max_el = bench.replica_throughput(cells, el, dist, "cpu")
    f = o.read_components()
    out[rank] = (value, max_el, el, cells, [float(np.abs(c).sum()) for c in f])
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of this multi-threaded process
    out = mgr.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    v0, m0, e0, c0, s0 = out[0]
    v1, m1, e1, c1, s1 = out[1]
    assert s0 == s1  # replicas of one scene are identical across processes
    assert m0 == m1 == max(e0, e1)
    assert v0 == v1 == pytest.approx((c0 + c1) / max(e0, e1) / 1e6)
