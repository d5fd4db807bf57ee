"""Replicas on two CPU ranks (gloo): frames are sharded without overlap, every
frame is processed exactly once, and the job's throughput is the total frame
count over the slowest rank's time. The per-frame work is the CPU oracle on
tiny frames (the GPU path has no collective to test)."""
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


def _worker(rank, world, port, result_q):
    import time
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__))))
    import oracle
    from helpers import oracle_spec
    from us_lab4a_gb300 import replicas, workloads
    frames = workloads.mixed(num_frames=6, small=True, storage="f32")
    mine = replicas.shard(len(frames), rank, world)
    t0 = time.perf_counter()
    sums = {}
    for i in mine:
        fr = frames[i]
        v, _, _ = oracle.process(oracle_spec(oracle, fr.spec, nthreads=1), fr.make_rf_numpy(), fr.grid_xyz,
                                 dtype=np.float32)
        sums[i] = float(v.sum())
    secs = time.perf_counter() - t0
    stats = {"rank": rank, "frames": len(mine), "seconds": secs, "sums": sums}
    allstats = replicas.gather_stats(stats)
    slowest = replicas.max_over_ranks(secs)
    if rank == 0:
        result_q.put((allstats, slowest, replicas.aggregate(allstats)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    allstats, slowest, agg = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seen = [i for s in allstats for i in s["sums"]]
    assert sorted(seen) == list(range(6))          # every frame once
    assert len(set(seen)) == len(seen)             # no overlap
    assert slowest == max(s["seconds"] for s in allstats)
    assert agg["frames"] == 6 and agg["frames_per_s"] == pytest.approx(6 / slowest)


def test_shard_covers_all_items():
    from us_lab4a_gb300 import replicas
    for world in (1, 2, 3, 8):
        got = sorted(i for r in range(world) for i in replicas.shard(17, r, world))
        assert got == list(range(17))
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)
