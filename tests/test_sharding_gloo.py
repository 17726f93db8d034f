"""Multi-rank host logic on CPU (gloo, world size 2): the Morton-ordered target
shards partition the targets, each is compact in space, and the transfer
computed shard by shard (each rank with the whole source cloud, no data-path
collective) and put back in the caller's order by `assemble` equals the
single-rank transfer.  The per-rank transfer here is the CPU oracle (no GPU);
on GPUs each rank runs the same shard, through the same two functions
(`target_shard`, `assemble`), with the library."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from datatransferkit_gb300 import synthetic as syn
from datatransferkit_gb300.sharding import assemble, morton_codes, slice_bounds, target_shard


def test_slice_bounds_partition():
    for n in (0, 1, 7, 100, 8_000_000):
        for world in (1, 2, 3, 8):
            spans = [slice_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        slice_bounds(10, 2, 2)


def test_morton_shards_partition_and_are_compact():
    tgt = syn.uniform_points(50_000, 3)
    for world in (1, 2, 3, 8):
        shards = [target_shard(tgt, r, world) for r in range(world)]
        allidx = np.concatenate(shards)
        assert len(allidx) == len(tgt) and np.array_equal(np.sort(allidx), np.arange(len(tgt)))
        assert all(np.all(np.diff(s) > 0) for s in shards)  # caller order within a shard
        sizes = [len(s) for s in shards]
        assert max(sizes) - min(sizes) <= 1
        if world > 1:
            # a run of the Morton curve: each shard's box is far smaller than the cloud's
            vol = [np.prod(tgt[s].max(0) - tgt[s].min(0)) for s in shards]
            assert np.mean(vol) < 0.75
    # one rank: the whole set in its own order
    assert np.array_equal(target_shard(tgt, 0, 1), np.arange(len(tgt)))
    # ties in the code are cut by index, so duplicates still partition
    dup = np.repeat(tgt[:10], 100, axis=0)
    parts = [target_shard(dup, r, 4) for r in range(4)]
    assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(len(dup)))
    codes = morton_codes(np.array([[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5]], float))
    assert codes[0] == 0 and codes[1] == (1 << 63) - 1 and codes[0] < codes[2] < codes[1]


def test_assemble_checks_its_shards():
    with pytest.raises(ValueError):
        assemble([np.ones(2), np.ones(2)], [np.array([0, 1]), np.array([1, 2])], 3)
    with pytest.raises(ValueError):
        assemble([np.ones(2)], [np.array([0, 1])], 3)
    out = assemble([np.array([1.0, 3.0]), np.array([2.0])], [np.array([0, 2]), np.array([1])], 3)
    assert out.tolist() == [1.0, 2.0, 3.0]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import cpu
    src = syn.uniform_points(4000, 1)
    tgt = syn.uniform_points(1001, 2)
    vals = syn.smooth_field(src)
    shard = target_shard(tgt, rank, world)
    y = cpu.mls_transfer(src, tgt[shard], vals, 1, 2, k=20)["target"]
    # gather the slices for the check only (the transfer itself exchanges nothing)
    shards = [None] * world
    dist.all_gather_object(shards, shard)
    parts = [None] * world
    dist.all_gather_object(parts, y)
    if rank == 0:
        full = assemble(parts, shards, len(tgt))
        ref = cpu.mls_transfer(src, tgt, vals, 1, 2, k=20)["target"]
        out.put(float(np.abs(full - ref).max()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_match_single_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    err = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert err == 0.0
