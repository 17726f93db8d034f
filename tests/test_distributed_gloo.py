"""The distributed operators' host logic on CPU: gloo, world size 2.

Each rank holds its own sources and targets; the search, the query routing,
the merge by (d2, global index) and the value-fetch plan run as in the
product, with the CPU oracle standing in for the library's kNN and setup
(injected through the operators' test hooks).  The results must equal the
one-rank oracle over the union of the clouds in rank order bit for bit: the
rows, the coefficients (same coordinates in the same order) and the values.

Cases follow the reference's tests: random clouds of unequal sizes, a rank
with no sources, fewer sources than k in total (rows of min(k, N),
tstMeshfreeOperatorsSimpleProblem.cpp:113-147), a rank with no targets, the
40x40 grid per rank with the target on a source and ties at the k-th
neighbour (tstMeshfreeOperators.cpp:226-300), the fetch helper
(tstDetailsCommunicationHelpers.cpp:167-222) and the nearest-neighbour
operator.
"""
import os
import socket
import traceback

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from datatransferkit_gb300 import synthetic as syn


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class _OracleSearch:
    """kNN rows by (d2, index) and their d2, from the oracle."""

    def knn(self, src, tgt, k):
        from oracle import cpu
        row = min(int(k), src.shape[0])
        if tgt.shape[0] == 0 or row == 0:
            return (torch.empty((tgt.shape[0], row), dtype=torch.int64),
                    torch.empty((tgt.shape[0], row), dtype=torch.float64))
        _, idx, d2 = cpu.knn(src.numpy(), tgt.numpy(), k)
        return (torch.from_numpy(idx.astype(np.int64)).view(tgt.shape[0], row),
                torch.from_numpy(d2).view(tgt.shape[0], row))


class _OracleRows:
    """The operator of given rows, set up and applied by the oracle."""

    def __init__(self, tgt, row, nb_points, indices, n_sources, rbf, basis, precision="fp64", stream=None):
        from oracle import cpu
        n = tgt.shape[0]
        self.offset = np.arange(n + 1, dtype=np.int32) * row
        self.idx = indices.numpy().astype(np.int32)
        self.n_sources = n_sources
        entry = np.arange(n * row, dtype=np.int32)
        self.coeff = (cpu.mls_coefficients(nb_points.numpy(), tgt.numpy(), self.offset, entry, rbf.id,
                                           basis.id)[0] if n * row else np.zeros(0))

    def apply(self, values, out, stream=None):
        from oracle import cpu
        assert values.shape[0] == self.n_sources
        if out.numel() == 0:
            return
        v = values.numpy().reshape(values.shape[0], -1)
        res = np.stack([cpu.apply(self.offset, self.idx, self.coeff, v[:, c]) for c in range(v.shape[1])], 1)
        out.copy_(torch.from_numpy(res.reshape(out.shape)))

    def csr(self):
        return torch.from_numpy(self.offset), torch.from_numpy(self.idx), torch.from_numpy(self.coeff)


def _gather_all(x):
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, x)
    return parts


def _mls_case(rank, src, tgt, vals, rbf, basis, k):
    """Distributed vs the one-rank oracle over the union: max |difference| of
    values, rows equal, coefficients equal."""
    from oracle import cpu
    from datatransferkit_gb300.distributed import DistributedMovingLeastSquaresOperator
    op = DistributedMovingLeastSquaresOperator(
        dist.group.WORLD, torch.from_numpy(src), torch.from_numpy(tgt), rbf, basis, k=k,
        _search=_OracleSearch(), _build=_OracleRows)
    out = torch.empty(len(tgt), dtype=torch.float64)
    op.apply(torch.from_numpy(vals), out)
    srcs, valss = _gather_all(src), _gather_all(vals)
    union, uvals = np.concatenate(srcs), np.concatenate(valss)
    kk = k if k is not None else basis.size
    if len(tgt):
        ref = cpu.mls_transfer(union, tgt, uvals, rbf.id, basis.id, k=kk)
        row = ref["offset"][1] - ref["offset"][0]
        assert op.row == row
        assert np.array_equal(op.neighbors.numpy().reshape(-1), ref["idx"]), "rows differ"
        assert np.array_equal(op._local.coeff, ref["coeff"]), "coefficients differ"
        assert np.array_equal(out.numpy(), ref["target"]), "values differ"
    # rank-2 values: each component alike
    v2 = torch.from_numpy(np.stack([vals, 2.0 * vals], 1))
    out2 = torch.empty((len(tgt), 2), dtype=torch.float64)
    op.apply(v2, out2)
    assert torch.equal(out2[:, 0], out) and torch.equal(out2[:, 1], torch.from_numpy(2.0 * out.numpy()))
    return op


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from datatransferkit_gb300 import InvalidArgument
        from datatransferkit_gb300.distributed import DistributedNearestNeighborOperator, fetch
        from datatransferkit_gb300.operators import (Linear, MultivariatePolynomialBasis, Quadratic,
                                                     Wendland)
        from oracle import cpu
        lin, quad = MultivariatePolynomialBasis(Linear, 3), MultivariatePolynomialBasis(Quadratic, 3)

        # 1. random clouds of unequal sizes that overlap in part
        src = syn.uniform_points(1500 if rank == 0 else 900, 10 + rank) * (1.0 + 0.5 * rank)
        tgt = syn.uniform_points(400 if rank == 0 else 250, 20 + rank)
        vals = syn.smooth_field(src)
        op = _mls_case(rank, src, tgt, vals, Wendland(2), quad, 20)
        _mls_case(rank, src, tgt, vals, Wendland(0), lin, None)

        # 1b. side-by-side slabs: a target goes to the other rank only when its
        #     own k-th neighbour is farther than that rank's box
        slab = syn.uniform_points(2000, 40 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        near = syn.uniform_points(300, 50 + rank) * np.array([0.5, 1.0, 1.0]) + np.array([0.5 * rank, 0, 0])
        op = _mls_case(rank, slab, near, syn.smooth_field(slab), Wendland(2), quad, 20)
        assert 0 < sum(op.queries_sent) < 0.5 * len(near), op.queries_sent

        # 2. one rank without sources
        src0 = syn.uniform_points(600, 30) if rank == 0 else np.zeros((0, 3))
        _mls_case(rank, src0, tgt, syn.smooth_field(src0) if len(src0) else np.zeros(0), Wendland(0), lin, 8)

        # 3. fewer sources than k in total: rows of min(k, N) = 3
        src1 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]) if rank == 0 else np.array([[0.0, 1.0, 0.0]])
        tgt1 = np.array([[0.25, 0.25, 0.0]]) if rank == 0 else np.array([[0.5, 0.5, 0.0], [0.1, 0.9, 0.0]])
        op = _mls_case(rank, src1, tgt1, src1[:, 0] + 2.0, Wendland(0), lin, 4)
        assert op.row == 3

        # 4. a rank without targets
        tgt2 = tgt if rank == 0 else np.zeros((0, 3))
        _mls_case(rank, src, tgt2, vals, Wendland(2), quad, 20)

        # 5. the reference's grid case: 40x40 sources at z = rank, the target on a
        #    source at (19, 19, rank); ties at the k-th neighbour across ranks
        for basis in (lin, quad):
            g = syn.grid_points((40, 40, 1), (0.0, 0.0, float(rank)))
            t = syn.grid_points((1, 1, 1), (19.0, 19.0, float(rank)))
            f = syn.polynomial_of_basis(basis.size)
            _mls_case(rank, g, t, f(g), Wendland(0), basis, None)
            from datatransferkit_gb300.distributed import DistributedMovingLeastSquaresOperator
            op = DistributedMovingLeastSquaresOperator(
                dist.group.WORLD, torch.from_numpy(g), torch.from_numpy(t), Wendland(0), basis,
                _search=_OracleSearch(), _build=_OracleRows)
            out = torch.empty(1, dtype=torch.float64)
            op.apply(torch.from_numpy(f(g)), out)
            exact = f(t)
            assert abs(out.item() - exact[0]) <= 1e-14 * abs(exact[0]), (out.item(), exact[0])

        # 6. the fetch helper, as tstDetailsCommunicationHelpers.cpp:167-222
        size = world
        indices = torch.tensor([(rank + i) % size for i in range(size)])
        ranks = torch.full((size,), size - 1 - rank)
        v = torch.arange(size) + rank * size
        got = fetch(dist.group.WORLD, ranks, indices, v)
        assert torch.equal(got, ranks * size + indices)
        dim = 2
        w = torch.stack([torch.arange(size) + i * size + rank * size * dim for i in range(dim)], 1)
        got = fetch(dist.group.WORLD, ranks, indices, w)
        ref = torch.stack([ranks * size * dim + indices + j * size for j in range(dim)], 1)
        assert torch.equal(got, ref)
        try:
            fetch(dist.group.WORLD, ranks, indices[:1], v)
            raise AssertionError("mismatched ranks / indices accepted")
        except InvalidArgument:
            pass

        # 7. the nearest-neighbour operator over both ranks
        nn = DistributedNearestNeighborOperator(dist.group.WORLD, torch.from_numpy(src), torch.from_numpy(tgt),
                                                _search=_OracleSearch())
        union = np.concatenate(_gather_all(src))
        _, idx, _ = cpu.knn(union, tgt, 1)
        assert np.array_equal(nn.indices.numpy(), idx)
        out = torch.empty(len(tgt), dtype=torch.float64)
        nn.apply(torch.from_numpy(vals), out)
        assert np.array_equal(out.numpy(), np.concatenate(_gather_all(vals))[idx])

        # 8. no sources anywhere: the reference's DTK_CHECK(!search_tree.empty())
        try:
            from datatransferkit_gb300.distributed import DistributedMovingLeastSquaresOperator
            DistributedMovingLeastSquaresOperator(dist.group.WORLD, torch.zeros((0, 3), dtype=torch.float64),
                                                  torch.from_numpy(tgt), _search=_OracleSearch(),
                                                  _build=_OracleRows)
            raise AssertionError("an empty source cloud was accepted")
        except InvalidArgument:
            pass
        q.put((rank, "ok"))
    except Exception:
        q.put((rank, traceback.format_exc()))
    finally:
        dist.destroy_process_group()


def test_two_rank_distributed_operators_match_one_rank_oracle():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert results == {0: "ok", 1: "ok"}, "\n".join(v for v in results.values() if v != "ok")
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_group_keeps_the_one_rank_operator():
    # no process group: the one-rank operator class (the dispatch looks for a
    # torch.distributed group of several ranks)
    from datatransferkit_gb300.operators import _multi_rank
    assert not _multi_rank(None) and not _multi_rank(1)
