"""The distributed operators on the GPU through the library: two ranks (gloo,
one process each, both on cuda:0; the collectives run on host tensors and no
kernel waits on another rank's) against the one-rank operator over the union
of the clouds in rank order.

Bars: the rows (global source indices) equal the one-rank search's; the
coefficients equal the one-rank operator's bit for bit (same coordinates,
same rows, same kernels); the values agree to 1e-13 relative L2 in FP64 and
2^-40 in the mixed form (the apply kernels of the two handles may sum a row
in a different order).  The reference's grid case reproduces its polynomial
to 1e-14 (tstMeshfreeOperators.cpp:226-300), and the nearest-neighbour
operator finds the one-rank nearest source of every target.
"""
import json
import os
import socket
import time
import traceback

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _gather_all(x):
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, x)
    return parts


def _rel_l2(a, b):
    return float(torch.linalg.vector_norm(a - b) / max(float(torch.linalg.vector_norm(b)), 1e-300))


def _case(src, tgt, vals, rbf, basis, k, precision):
    import datatransferkit_gb300 as dtk
    dev = torch.device("cuda", 0)
    s, t = torch.from_numpy(src).to(dev), torch.from_numpy(tgt).to(dev)
    op = dtk.MovingLeastSquaresOperator(dist.group.WORLD, s, t, rbf, basis, k=k, precision=precision)
    assert isinstance(op, dtk.DistributedMovingLeastSquaresOperator)
    out = torch.empty(len(tgt), dtype=torch.float64, device=dev)
    op.apply(torch.from_numpy(vals).to(dev), out)
    torch.cuda.synchronize()
    union = torch.from_numpy(np.concatenate(_gather_all(src))).to(dev)
    uvals = torch.from_numpy(np.concatenate(_gather_all(vals))).to(dev)
    if len(tgt):
        one = dtk.MovingLeastSquaresOperator(None, union, t, rbf, basis, k=k, precision=precision)
        ref = torch.empty_like(out)
        one.apply(uvals, ref)
        _, idx1, c1 = one.csr()
        _, gid, c2 = op.csr()
        assert torch.equal(gid.to(torch.int64), idx1.to(torch.int64)), "rows differ"
        assert torch.equal(c1, c2), "coefficients differ"
        tol = 1e-13 if precision == "fp64" else 2.0 ** -40
        err = _rel_l2(out, ref)
        assert err <= tol, (precision, err)
        one.close()
    op.close()
    return op


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    report = {}
    try:
        import datatransferkit_gb300 as dtk
        from datatransferkit_gb300.operators import (Linear, MultivariatePolynomialBasis, Quadratic,
                                                     Wendland)
        lin, quad = MultivariatePolynomialBasis(Linear, 3), MultivariatePolynomialBasis(Quadratic, 3)
        dev = torch.device("cuda", 0)

        # random clouds of unequal sizes, overlapping in part
        src = syn.uniform_points(20000 if rank == 0 else 12000, 10 + rank) * (1.0 + 0.5 * rank)
        tgt = syn.uniform_points(5000 if rank == 0 else 3000, 20 + rank)
        vals = syn.smooth_field(src)
        for precision in ("fp64", "mixed"):
            _case(src, tgt, vals, Wendland(2), quad, 20, precision)
            _case(src, tgt, vals, Wendland(0), lin, None, precision)

        # side-by-side slabs (queries cross only near the interface)
        slab = syn.uniform_points(40000, 40 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        near = syn.uniform_points(8000, 50 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        op = _case(slab, near, syn.smooth_field(slab), Wendland(4), quad, 32, "fp64")
        assert 0 < sum(op.queries_sent) < 0.5 * len(near), op.queries_sent

        # one rank without sources; fewer sources than k in total; a rank without targets
        src0 = syn.uniform_points(3000, 30) if rank == 0 else np.zeros((0, 3))
        _case(src0, tgt, syn.smooth_field(src0) if len(src0) else np.zeros(0), Wendland(0), lin, 8, "fp64")
        src1 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]) if rank == 0 else np.array([[0.0, 1.0, 0.0]])
        tgt1 = np.array([[0.25, 0.25, 0.0]]) if rank == 0 else np.array([[0.5, 0.5, 0.0], [0.1, 0.9, 0.0]])
        op = _case(src1, tgt1, src1[:, 0] + 2.0, Wendland(0), lin, 4, "fp64")
        assert op.row == 3
        _case(src, tgt if rank == 0 else np.zeros((0, 3)), vals, Wendland(2), quad, 20, "fp64")

        # the reference's grid case across the two ranks
        for basis in (lin, quad):
            g = syn.grid_points((40, 40, 1), (0.0, 0.0, float(rank)))
            t = syn.grid_points((1, 1, 1), (19.0, 19.0, float(rank)))
            f = syn.polynomial_of_basis(basis.size)
            op = dtk.MovingLeastSquaresOperator(dist.group.WORLD, torch.from_numpy(g).to(dev),
                                                torch.from_numpy(t).to(dev), Wendland(0), basis)
            out = torch.empty(1, dtype=torch.float64, device=dev)
            op.apply(torch.from_numpy(f(g)).to(dev), out)
            exact = float(f(t)[0])
            assert abs(out.item() - exact) <= 1e-14 * abs(exact), (out.item(), exact)

        # nearest neighbour over both ranks, rank-1 and rank-2 values
        s, t = torch.from_numpy(src).to(dev), torch.from_numpy(tgt).to(dev)
        nn = dtk.NearestNeighborOperator(dist.group.WORLD, s, t)
        assert isinstance(nn, dtk.DistributedNearestNeighborOperator)
        union = torch.from_numpy(np.concatenate(_gather_all(src))).to(dev)
        one = dtk.NearestNeighborOperator(None, union, t)
        assert torch.equal(nn.indices, one.indices.to(torch.int64))
        uv = torch.from_numpy(np.stack([np.concatenate(_gather_all(vals))] * 2, 1)).to(dev)
        v2 = torch.from_numpy(np.stack([vals, vals], 1)).to(dev)
        out2 = torch.empty((len(tgt), 2), dtype=torch.float64, device=dev)
        nn.apply(v2, out2)
        assert torch.equal(out2, uv[one.indices.to(torch.int64)])

        # a larger case, timed: 1M sources and 1M targets in Morton-compact slabs
        # of 500k each (Quadratic3, Wendland<4>, k = 32, FP64)
        n = 500_000
        big_s = syn.uniform_points(n, 60 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        big_t = syn.uniform_points(n, 70 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        bs, bt = torch.from_numpy(big_s).to(dev), torch.from_numpy(big_t).to(dev)
        bv = torch.from_numpy(syn.smooth_field(big_s)).to(dev)
        bo = torch.empty(n, dtype=torch.float64, device=dev)
        for precision in ("fp64", "mixed"):
            dist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            op = dtk.MovingLeastSquaresOperator(dist.group.WORLD, bs, bt, Wendland(4), quad, k=32,
                                                precision=precision)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            for _ in range(3):
                op.apply(bv, bo)
            torch.cuda.synchronize()
            dist.barrier()
            t2 = time.perf_counter()
            for _ in range(10):
                op.apply(bv, bo)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            report[precision] = {"setup_s": t1 - t0, "apply_ms": (t3 - t2) * 100.0,
                                 "queries_sent": sum(op.queries_sent), "fetched": op._plan.n_fetched}
            op.close()
        q.put((rank, "ok", report))
    except Exception:
        q.put((rank, traceback.format_exc(), report))
    finally:
        dist.destroy_process_group()


def test_two_ranks_on_one_gpu_match_the_one_rank_operator():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = {}
    for _ in procs:
        rank, status, report = q.get(timeout=900)
        results[rank] = (status, report)
    for p in procs:
        p.join(timeout=120)
    bad = [s for s, _ in results.values() if s != "ok"]
    assert not bad, "\n".join(bad)
    assert all(p.exitcode == 0 for p in procs)
    out = os.environ.get("DTK_DISTRIBUTED_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump({str(r): rep for r, (_, rep) in results.items()}, f, indent=1)
