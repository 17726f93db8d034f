"""Multi-rank host logic on CPU (gloo, world size 2): target shards cover the
targets exactly once, and the transfer computed shard by shard (each rank with
the whole source cloud, no data-path collective) equals the single-rank
transfer.  The per-rank transfer here is the CPU oracle; on GPUs each rank runs
the same shard through the library."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from datatransferkit_gb300.sharding import target_shard


def test_shards_partition():
    for n in (0, 1, 7, 100, 8_000_000):
        for world in (1, 2, 3, 8):
            spans = [target_shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        target_shard(10, 2, 2)


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
    from datatransferkit_gb300 import synthetic as syn
    src = syn.uniform_points(4000, 1)
    tgt = syn.uniform_points(1001, 2)
    vals = syn.smooth_field(src)
    b, e = target_shard(len(tgt), rank, world)
    y = cpu.mls_transfer(src, tgt[b:e], vals, 1, 2, k=20)["target"]
    # gather the slices for the check only (the transfer itself exchanges nothing)
    sizes = [None] * world
    dist.all_gather_object(sizes, (b, e))
    parts = [None] * world
    dist.all_gather_object(parts, y.tolist())
    if rank == 0:
        full = np.concatenate([np.asarray(p) for p in parts])
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
