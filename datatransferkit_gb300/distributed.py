"""Multi-rank operators over ``torch.distributed``: the distributed search and
the value fetch of DataTransferKit's MPI operators.

Mirrors (paths inside the DataTransferKit project):
  MovingLeastSquaresOperator(comm, ...) with more than one rank
      constructor  packages/Meshfree/src/DTK_MovingLeastSquaresOperator_def.hpp:24-119
                   (ArborX::DistributedTree over the sources :47-48, its
                   kNN query :52-60, the coordinate fetch :66-67)
      apply        DTK_MovingLeastSquaresOperator_def.hpp:121-141 (value fetch :133-134)
  NearestNeighborOperator(comm, ...) with more than one rank
                   DTK_NearestNeighborOperator_def.hpp:23-86
  fetch / pullSourceValues / pushTargetValues
                   DTK_DetailsNearestNeighborOperatorImpl.hpp:47-192

Each rank holds its own sources and targets (CUDA tensors).  A source's
global index is its rank's offset (the sources of the lower ranks) plus its
local index, so a row ordered by (d2, global index) is the row a one-rank
operator gives over the rank-ordered union of the clouds; every d2 is the
one the library's search computes ((dx*dx + dy*dy) + dz*dz in FP64 with
separately rounded operations, dtk_knn_search_d2).

The search (ArborX's DistributedTree is a third-party dependency, not in the
reference's tree; this restates its contract, exact kNN over all ranks):
  1. all ranks share their source counts and bounding boxes;
  2. each rank searches its own sources (the library's kNN); the k-th local
     d2 bounds each target's row (no bound when the rank has fewer than k
     sources);
  3. a target goes to every other rank whose box lies within that bound: the
     rounded box distance never exceeds the rounded distance to a point in the
     box (rounding is monotone), so no candidate is missed, ties included;
  4. the owners answer with their k nearest (d2, global index, coordinates);
  5. the rows merge by (d2, global index) and keep the first k.
The operator is then built from the rows (``dtk_mls_create_from_neighbors``),
with each distinct source of a rank's rows numbered once.  The value-fetch
plan is built once at setup, so each ``apply`` is one ``all_to_all_single``
of the distinct values a rank needs followed by the library's apply (the
reference rebuilds its Distributor and fetches one value per entry on every
call).

The collectives run on host tensors for gloo and on device tensors for NCCL.
There is no device-side exchange: the ranks' kernels never wait on one
another.
"""
from __future__ import annotations

import torch
import torch.distributed as dist

from . import _capi
from ._capi import check, lib
from .operators import (Linear, MovingLeastSquaresOperator, MultivariatePolynomialBasis, PointCloudOperator,
                        Wendland, _check_points, _multi_rank, _stream)

__all__ = ["DistributedMovingLeastSquaresOperator", "DistributedNearestNeighborOperator", "fetch",
           "is_multi_rank", "distributed_knn"]


def is_multi_rank(comm) -> bool:
    """True for a torch.distributed process group of more than one rank."""
    return _multi_rank(comm)


class _Comm:
    """The exchange steps of the operators over one process group."""

    def __init__(self, group):
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        nccl = dist.get_backend(group) == "nccl"
        self.device = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")

    def all_gather(self, t: torch.Tensor) -> torch.Tensor:
        """(size, *t.shape) on the host; t has the same shape on every rank."""
        t = t.to(self.device).contiguous()
        out = [torch.empty_like(t) for _ in range(self.size)]
        dist.all_gather(out, t, group=self.group)
        return torch.stack(out).cpu()

    def counts(self, send_counts: list[int]) -> list[int]:
        """What every rank sends to this one, given what this one sends to each."""
        t = torch.tensor(send_counts, dtype=torch.int64, device=self.device)
        r = torch.empty_like(t)
        dist.all_to_all_single(r, t, group=self.group)
        return [int(x) for x in r.cpu()]

    def exchange(self, send: torch.Tensor, send_counts: list[int], recv_counts: list[int]) -> torch.Tensor:
        """Rows of ``send`` grouped by destination rank -> rows grouped by source rank,
        on the device ``send`` came from."""
        home = send.device
        s = send.to(self.device).contiguous()
        r = torch.empty((sum(recv_counts),) + tuple(send.shape[1:]), dtype=send.dtype, device=self.device)
        dist.all_to_all_single(r, s, recv_counts, send_counts, group=self.group)
        return r.to(home)


def _box_d2(tgt: torch.Tensor, lo: torch.Tensor, hi: torch.Tensor) -> torch.Tensor:
    """Squared distance of each target to the box [lo, hi], less a relative
    2^-40: never above the d2 the search computes for a point in the box."""
    g = torch.clamp(torch.maximum(torch.sub(lo, tgt), torch.sub(tgt, hi)), min=0.0)
    gx, gy, gz = g[:, 0], g[:, 1], g[:, 2]
    d2 = torch.add(torch.add(torch.mul(gx, gx), torch.mul(gy, gy)), torch.mul(gz, gz))
    return d2 * (1.0 - 2.0 ** -40)


class _LibrarySearch:
    """The library's kNN: (indices, d2) of rows ascending by (d2, index)."""

    def knn(self, src: torch.Tensor, tgt: torch.Tensor, k: int):
        row = min(int(k), src.shape[0])
        n = tgt.shape[0]
        idx = torch.empty((n, row), dtype=torch.int32, device=tgt.device)
        d2 = torch.empty((n, row), dtype=torch.float64, device=tgt.device)
        if n and row:
            tgt = tgt.contiguous()
            check(lib().dtk_knn_search_d2(src.data_ptr(), src.shape[0], src.stride(0), src.stride(1),
                                          tgt.data_ptr(), n, tgt.stride(0), tgt.stride(1), row,
                                          idx.data_ptr(), d2.data_ptr(), _stream(None)))
        return idx.to(torch.int64), d2


class _Rows:
    """The merged kNN rows of this rank's targets and the value-fetch plan."""

    def __init__(self, gid, points, counts, first, row, sent):
        self.gid = gid          # (n_tgt, row) int64 global source index
        self.points = points    # (n_tgt, row, 3) float64 coordinates
        self.counts = counts    # sources per rank (host int64)
        self.first = first      # global index of each rank's first source
        self.row = row
        self.sent = sent        # queries this rank sent to each rank


def distributed_knn(comm: _Comm, src: torch.Tensor, tgt: torch.Tensor, k: int, search=None) -> _Rows:
    """The min(k, N) nearest sources of every local target among all ranks'
    sources (N in total), rows ascending by (d2, global index) (the
    DistributedTree kNN query, DTK_MovingLeastSquaresOperator_def.hpp:47-60)."""
    search = search or _LibrarySearch()
    dev = tgt.device
    n_loc, n_tgt = int(src.shape[0]), int(tgt.shape[0])
    counts = comm.all_gather(torch.tensor([n_loc], dtype=torch.int64)).view(-1)
    total = int(counts.sum())
    if total == 0:
        # DTK_CHECK( !search_tree.empty() ), DTK_MovingLeastSquaresOperator_def.hpp:49
        raise _capi.InvalidArgument(1, "the distributed source cloud is empty")
    first = torch.cumsum(counts, 0) - counts
    row = min(int(k), total)
    if n_loc:
        box = torch.cat([src.min(0).values, src.max(0).values]).cpu()
    else:
        inf = float("inf")
        box = torch.tensor([inf, inf, inf, -inf, -inf, -inf], dtype=torch.float64)
    boxes = comm.all_gather(box.to(torch.float64))

    # 2. the local rows and their bounds
    if n_loc:
        idx, d2 = search.knn(src, tgt, row)
        pts = src[idx]
    else:
        idx = torch.empty((n_tgt, 0), dtype=torch.int64, device=dev)
        d2 = torch.empty((n_tgt, 0), dtype=torch.float64, device=dev)
        pts = torch.empty((n_tgt, 0, 3), dtype=torch.float64, device=dev)
    row_l = idx.shape[1]
    gid = idx + int(first[comm.rank])
    if row_l == row and row_l > 0:
        bound = d2[:, -1]
    else:
        bound = torch.full((n_tgt,), float("inf"), dtype=torch.float64, device=dev)

    # 3. the queries, grouped by destination
    sel = []
    for q in range(comm.size):
        if q == comm.rank or int(counts[q]) == 0 or n_tgt == 0:
            sel.append(torch.empty(0, dtype=torch.int64, device=dev))
            continue
        bq = boxes[q].to(dev)
        sel.append(torch.nonzero(_box_d2(tgt, bq[:3], bq[3:]) <= bound).view(-1))
    send_counts = [int(s.numel()) for s in sel]
    recv_counts = comm.counts(send_counts)
    queries = tgt[torch.cat(sel)] if sum(send_counts) else torch.empty((0, 3), dtype=torch.float64, device=dev)
    asked = comm.exchange(queries, send_counts, recv_counts)

    # 4. this rank's answers: (d2, x, y, z) and the global index per entry
    row_o = min(row, n_loc)
    if asked.shape[0] and row_o:
        a_idx, a_d2 = search.knn(src, asked, row)
        a_pts = src[a_idx]
        answer = torch.cat([a_d2.unsqueeze(2), a_pts], 2).reshape(-1, 4)
        a_gid = (a_idx + int(first[comm.rank])).reshape(-1)
    else:
        answer = torch.empty((0, 4), dtype=torch.float64, device=dev)
        a_gid = torch.empty(0, dtype=torch.int64, device=dev)
    back_send = [c * row_o for c in recv_counts]
    back_recv = [send_counts[q] * min(row, int(counts[q])) for q in range(comm.size)]
    answers = comm.exchange(answer, back_send, back_recv)
    answer_gid = comm.exchange(a_gid, back_send, back_recv)

    # 5. merge by (d2, global index) and keep the first `row` of each target;
    #    a target that asked no other rank keeps its local row (then full)
    asked_any = torch.zeros(n_tgt, dtype=torch.bool, device=dev)
    for q in range(comm.size):
        asked_any[sel[q]] = True
    touched = torch.nonzero(asked_any).view(-1)
    out_gid = torch.empty((n_tgt, row), dtype=torch.int64, device=dev)
    out_pts = torch.empty((n_tgt, row, 3), dtype=torch.float64, device=dev)
    if row_l == row:
        out_gid.copy_(gid)
        out_pts.copy_(pts)
    elif touched.numel() != n_tgt:
        raise _capi.DTKError(6, "distributed search: a short row asked no other rank")
    if touched.numel():
        t_parts = [touched.repeat_interleave(row_l)]
        d2_parts, gid_parts = [d2[touched].reshape(-1)], [gid[touched].reshape(-1)]
        pts_parts = [pts[touched].reshape(-1, 3)]
        at = 0
        for q in range(comm.size):
            rq = min(row, int(counts[q]))
            n = send_counts[q] * rq
            if n == 0:
                continue
            t_parts.append(sel[q].repeat_interleave(rq))
            d2_parts.append(answers[at:at + n, 0])
            pts_parts.append(answers[at:at + n, 1:4])
            gid_parts.append(answer_gid[at:at + n])
            at += n
        t_all, d2_all = torch.cat(t_parts), torch.cat(d2_parts)
        gid_all, pts_all = torch.cat(gid_parts), torch.cat(pts_parts)
        order = torch.sort(gid_all, stable=True).indices
        order = order[torch.sort(d2_all[order], stable=True).indices]
        order = order[torch.sort(t_all[order], stable=True).indices]
        per = torch.bincount(t_all, minlength=n_tgt)
        begin = torch.cumsum(per, 0) - per
        keep = order[(torch.arange(order.numel(), device=dev) - begin[t_all[order]]) < row]
        if keep.numel() != touched.numel() * row:
            raise _capi.DTKError(6, "distributed search: a row came back short")
        out_gid[touched] = gid_all[keep].view(-1, row)
        out_pts[touched] = pts_all[keep].view(-1, row, 3)
    return _Rows(out_gid, out_pts, counts, first, row, send_counts)


class _FetchPlan:
    """Values of given global sources, fetched from their owners (the
    Distributor plan of pullSourceValues / pushTargetValues,
    DTK_DetailsNearestNeighborOperatorImpl.hpp:47-146), built once.

    ``wanted`` are the distinct global indices this rank needs, ascending; the
    fetched array lists their values in that order."""

    def __init__(self, comm: _Comm, wanted: torch.Tensor, counts: torch.Tensor, first: torch.Tensor):
        self.comm = comm
        dev = wanted.device
        ends = torch.cumsum(counts, 0).to(dev)
        owner = torch.searchsorted(ends, wanted, right=True)
        local = wanted - first.to(dev)[owner]
        per_owner = [int(x) for x in torch.bincount(owner, minlength=comm.size).cpu()]
        # this rank's own values are gathered on the device (a contiguous run
        # of the fetched array, the owners being in rank order); only the
        # others' go through the collective
        a = sum(per_owner[:comm.rank])
        self.own = (a, a + per_owner[comm.rank])
        self.own_index = local[a:a + per_owner[comm.rank]]
        self.remote = torch.cat([torch.arange(0, a, device=dev),
                                 torch.arange(self.own[1], int(wanted.numel()), device=dev)])
        self.recv_counts = list(per_owner)
        self.recv_counts[comm.rank] = 0
        self.send_counts = comm.counts(self.recv_counts)
        # the owners learn which of their values to send, in the order asked
        self.send_index = comm.exchange(local[self.remote], self.recv_counts, self.send_counts)
        self.n_fetched = int(wanted.numel())

    def __call__(self, values: torch.Tensor) -> torch.Tensor:
        out = torch.empty((self.n_fetched,) + tuple(values.shape[1:]), dtype=values.dtype, device=values.device)
        out[self.own[0]:self.own[1]] = values[self.own_index]
        got = self.comm.exchange(values[self.send_index], self.send_counts, self.recv_counts)
        out[self.remote] = got
        return out


def fetch(group, ranks: torch.Tensor, indices: torch.Tensor, values: torch.Tensor) -> torch.Tensor:
    """out[i] = values on rank ranks[i] at indices[i] (rank-1 or rank-2 values),
    the reference's NearestNeighborOperatorImpl::fetch
    (DTK_DetailsNearestNeighborOperatorImpl.hpp:150-189, DTK_REQUIRE at :157)."""
    if ranks.shape != indices.shape or ranks.dim() != 1:
        raise _capi.InvalidArgument(1, "ranks.extent(0) == indices.extent(0)")
    comm = _Comm(group)
    dev = values.device
    ranks, indices = ranks.to(dev, torch.int64), indices.to(dev, torch.int64)
    if ranks.numel() and (int(ranks.min()) < 0 or int(ranks.max()) >= comm.size):
        raise _capi.InvalidArgument(1, "ranks must lie in [0, comm_size)")
    order = torch.sort(ranks, stable=True).indices
    send_counts = [int(x) for x in torch.bincount(ranks, minlength=comm.size).cpu()]
    recv_counts = comm.counts(send_counts)
    asked = comm.exchange(indices[order], send_counts, recv_counts)
    if asked.numel() and (int(asked.min()) < 0 or int(asked.max()) >= values.shape[0]):
        raise _capi.InvalidArgument(1, "indices must lie in [0, values.extent(0)) on their rank")
    answer = comm.exchange(values[asked], recv_counts, send_counts)
    out = torch.empty((ranks.numel(),) + tuple(values.shape[1:]), dtype=values.dtype, device=dev)
    out[order] = answer
    return out


def _check_values(t: torch.Tensor, n: int, what: str, extent: str):
    if not isinstance(t, torch.Tensor) or t.dtype != torch.float64 or t.dim() not in (1, 2):
        raise _capi.InvalidArgument(1, f"{what} must be a rank-1 or rank-2 float64 tensor")
    if t.shape[0] != n:
        raise _capi.InvalidArgument(1, extent)


class DistributedMovingLeastSquaresOperator(PointCloudOperator):
    """Moving least squares transfer with sources and targets spread over the
    ranks of a torch.distributed group.

    ``DistributedMovingLeastSquaresOperator(group, source_points,
    target_points, rbf=Wendland(0), basis=MultivariatePolynomialBasis(Linear, 3),
    k=None, precision="fp64")`` is collective: every rank passes its own
    sources and targets.  ``apply(source_values, target_values)`` (collective)
    takes this rank's source values and writes this rank's target values,
    equal to the one-rank operator over the union of the clouds in rank order.
    ``MovingLeastSquaresOperator(group, ...)`` returns one when the group has
    more than one rank.
    """

    def __init__(self, comm, source_points, target_points, rbf=None, basis=None, *,
                 k: int | None = None, precision="fp64", stream=None, _search=None, _build=None):
        # _search / _build: the kNN search and the setup from rows, replaceable
        # together by a test that runs the exchange on host tensors
        self.polynomial_basis = basis or MultivariatePolynomialBasis(Linear, 3)
        self.radial_basis_function = rbf or Wendland(0)
        src, tgt = source_points, target_points
        if _build is None:
            src = _check_points(src, "source_points")
            tgt = _check_points(tgt, "target_points")
        # DTK_MovingLeastSquaresOperator_def.hpp:39-42
        if src.shape[1] != tgt.shape[1]:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == target_points.extent(1)")
        if src.shape[1] != 3 or self.polynomial_basis.dim != 3:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == 3")
        k = self.polynomial_basis.size if k is None else int(k)
        if k < 1 or k > 32:
            raise _capi.Unsupported(2, "kNN search supports 1 <= k <= 32")
        self._comm = _Comm(comm)
        self._stream = stream
        rows = distributed_knn(self._comm, src, tgt, k, _search)
        wanted, local_idx = torch.unique(rows.gid.reshape(-1), sorted=True, return_inverse=True)
        self._plan = _FetchPlan(self._comm, wanted, rows.counts, rows.first)
        build = _build or MovingLeastSquaresOperator.from_neighbors
        self._local = build(tgt, rows.row, rows.points.reshape(-1, 3).contiguous(),
                            local_idx.to(torch.int32).contiguous(), self._plan.n_fetched,
                            self.radial_basis_function, self.polynomial_basis, precision=precision,
                            stream=stream)
        self.n_source_points = int(src.shape[0])
        self.n_target_points = int(tgt.shape[0])
        self.row = rows.row
        self.queries_sent = rows.sent
        self._global = rows.gid

    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor, stream=None) -> None:
        # DTK_REQUIRE at DTK_MovingLeastSquaresOperator_def.hpp:129-130
        _check_values(source_values, self.n_source_points, "source_values",
                      "source_values.extent(0) == n_source_points")
        _check_values(target_values, self.n_target_points, "target_values",
                      "target_values.extent(0) == n_target_points")
        fetched = self._plan(source_values)
        self._local.apply(fetched, target_values, stream=stream)

    @property
    def neighbors(self) -> torch.Tensor:
        """(n_targets, row) global source index of every entry, rows ascending by (d2, index)."""
        return self._global

    def csr(self):
        """(offset, global source indices, coefficients) of this rank's rows."""
        offset, _, coeff = self._local.csr()
        return offset, self._global.reshape(-1), coeff

    def close(self):
        if getattr(self, "_local", None) is not None and hasattr(self._local, "close"):
            self._local.close()


class DistributedNearestNeighborOperator(PointCloudOperator):
    """Nearest-neighbour transfer over the ranks of a torch.distributed group
    (DTK_NearestNeighborOperator_def.hpp:23-86 with more than one rank): every
    target takes the value of its nearest source on any rank, ties to the
    smaller global index.  Collective construction and apply; rank-1 or
    rank-2 values."""

    def __init__(self, comm, source_points, target_points, *, stream=None, _search=None):
        src, tgt = source_points, target_points
        if _search is None:
            src = _check_points(src, "source_points")
            tgt = _check_points(tgt, "target_points")
        if src.shape[1] != tgt.shape[1] or src.shape[1] != 3:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == target_points.extent(1) == 3")
        self._comm = _Comm(comm)
        rows = distributed_knn(self._comm, src, tgt, 1, _search)
        wanted, self._slot = torch.unique(rows.gid.reshape(-1), sorted=True, return_inverse=True)
        self._plan = _FetchPlan(self._comm, wanted, rows.counts, rows.first)
        self.n_source_points = int(src.shape[0])
        self.n_target_points = int(tgt.shape[0])
        self.queries_sent = rows.sent
        self._global = rows.gid.reshape(-1)

    @property
    def indices(self) -> torch.Tensor:
        """Global index of every target's nearest source."""
        return self._global

    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor, stream=None) -> None:
        _check_values(source_values, self.n_source_points, "source_values",
                      "source_values.extent(0) == n_source_points")
        _check_values(target_values, self.n_target_points, "target_values",
                      "target_values.extent(0) == n_target_points")
        if source_values.dim() != target_values.dim() or source_values.shape[1:] != target_values.shape[1:]:
            raise _capi.InvalidArgument(1, "source_values.extent(1) == target_values.extent(1)")
        fetched = self._plan(source_values)
        target_values.copy_(fetched[self._slot])
