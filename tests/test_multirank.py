"""Host-side sharding over ranks, run as two gloo ranks on CPU.

Each rank checks its contiguous chunk of a state batch with the oracle (the
stand-in for its GPU on this CPU-only test) and the chunks are gathered in
rank order; the result must equal the single-process answer.
"""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from puzzletunneldiscovery_gb300 import workloads as W
from puzzletunneldiscovery_gb300.shard import shard_range


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from puzzletunneldiscovery_gb300.shard import gather, shard_range
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    Ve, Fe, Vr, Fr = W.interlocking_tori(1.0, 0.25, 16, 8)
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    q = W.uniform_states(1001, -2.0, 2.0, ow.scene_scale, seed=3)
    lo, hi = shard_range(len(q), rank, world)
    local = torch.from_numpy(ow.is_valid(q[lo:hi]).astype(np.uint8))
    full = gather(local, world)
    if rank == 0:
        np.save(out_path, full.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_shard_ranges_cover_batch():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c and a <= b


def test_two_gloo_ranks_match_single_process(tmp_path, oracle_mod):
    out = str(tmp_path / "gathered.npy")
    port = _free_port()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    Ve, Fe, Vr, Fr = W.interlocking_tori(1.0, 0.25, 16, 8)
    ow = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    q = W.uniform_states(1001, -2.0, 2.0, ow.scene_scale, seed=3)
    assert (np.load(out).astype(bool) == ow.is_valid(q)).all()


def _bench_rank(rank, world, port, out_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, units = bench.max_time_sum_units(100.0 + 50.0 * rank, 1000 * (rank + 1), world, torch.device("cpu"))
    if rank == 0:
        np.save(out_path, np.array([ms, units]))
    dist.barrier()
    dist.destroy_process_group()


def test_bench_reduces_over_ranks(tmp_path):
    """bench.py's whole-job figures at N > 1: the slowest rank's time, all ranks' units."""
    out = str(tmp_path / "agg.npy")
    mp.spawn(_bench_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    ms, units = np.load(out)
    assert ms == 150.0 and units == 3000.0
