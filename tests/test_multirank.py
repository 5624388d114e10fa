"""Sharding of a batch of atmospheres over ranks (gloo, world size 2, CPU):
each rank synthesises its contiguous slice with the oracle, the slices are
gathered in rank order and must equal the serial synthesis of the whole
batch; the step time used for throughput is the slowest rank's."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pyrh_gb300.shard import rank_seed, shard_bounds


def test_shard_bounds_cover_each_atmosphere_once():
    for natm in (1, 5, 6, 7, 16384):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                a, b = shard_bounds(natm, r, world)
                seen.extend(range(a, b))
                assert (b - a) in (natm // world, natm // world + 1)
            assert seen == list(range(natm))
    assert rank_seed(1000, 3) == 1003
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from conftest import batch_member, load_golden
    from oracle import oracle as O
    from pyrh_gb300.shard import gather_shards, max_over_ranks, shard_bounds
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = load_golden("lte_batch")
    natm = b["T"].shape[0]
    a, e = shard_bounds(natm, rank, world)
    local = [O.lte_synth(batch_member(b, i), md_float=False) for i in range(a, e)]
    parts = gather_shards(local, dist)
    slowest = max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        full = [s for part in parts for s in part]
        np.savez(os.path.join(out_dir, "gathered.npz"), *full, slowest=slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_equal_serial_batch(golden, tmp_path):
    from conftest import batch_member
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    g = np.load(tmp_path / "gathered.npz")
    b = golden("lte_batch")
    natm = b["T"].shape[0]
    assert float(g["slowest"]) == 2.0
    for i in range(natm):
        np.testing.assert_array_equal(g[f"arr_{i}"], O.lte_synth(batch_member(b, i), md_float=False))
