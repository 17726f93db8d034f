"""Host-side mirror of DataTransferKit's MLS operator API over the C ABI.

Mirrors (paths inside the DataTransferKit project):
  PointCloudOperator<DeviceType>            packages/Meshfree/src/DTK_PointCloudOperator.hpp:24-37
  MovingLeastSquaresOperator<Device, RBF, Basis>
        constructor (setup) / apply          DTK_MovingLeastSquaresOperator_decl.hpp:36-63
  Wendland<k>, Wu<k>, Buhmann<k>             DTK_CompactlySupportedRadialBasisFunctions.hpp:42-147
  MultivariatePolynomialBasis<Basis, DIM>    DTK_MultivariatePolynomialBasis.hpp:79-92

Arrays are CUDA tensors (device memory, the analogue of Kokkos Views in a
CUDA memory space): points float64 of shape (n, 3) with any strides
(LayoutRight or LayoutLeft), values float64 of shape (n,).  Precondition
failures raise ``InvalidArgument`` (DTK_REQUIRE -> DataTransferKitException).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _capi
from ._capi import Options, check, lib


# ---------------------------------------------------------------------------
# Template-parameter types
# ---------------------------------------------------------------------------
class _RBF:
    family = ""
    orders = ()
    _ids = {}

    def __init__(self, k: int):
        if k not in self.orders:
            raise ValueError(f"{type(self).__name__}<{k}> does not exist (orders {self.orders})")
        self.k = k
        self.id = self._ids[k]

    def __repr__(self):
        return f"{type(self).__name__}<{self.k}>"

    def __eq__(self, other):
        return isinstance(other, _RBF) and other.id == self.id

    def __hash__(self):
        return hash(self.id)


class Wendland(_RBF):
    orders = (0, 2, 4, 6)
    _ids = {0: 0, 2: 1, 4: 2, 6: 3}


class Wu(_RBF):
    orders = (2, 4)
    _ids = {2: 4, 4: 5}


class Buhmann(_RBF):
    orders = (2, 3, 4)
    _ids = {2: 6, 3: 7, 4: 8}


class Constant:
    pass


class Linear:
    pass


class Quadratic:
    pass


class MultivariatePolynomialBasis:
    """Basis<Constant|Linear|Quadratic, DIM>; the MLS operator needs DIM = 3."""

    _sizes = {(Constant, 3): 1, (Linear, 3): 4, (Quadratic, 3): 10,
              (Constant, 2): 1, (Linear, 2): 3, (Quadratic, 2): 6}
    _ids = {Constant: 0, Linear: 1, Quadratic: 2}

    def __init__(self, kind, dim: int = 3):
        if (kind, dim) not in self._sizes:
            raise ValueError("unknown polynomial basis")
        self.kind = kind
        self.dim = dim
        self.size = self._sizes[(kind, dim)]
        self.id = self._ids[kind]

    def __repr__(self):
        return f"MultivariatePolynomialBasis<{self.kind.__name__}, {self.dim}>"


FP64 = 0
MIXED = 1
_PRECISIONS = {"fp64": FP64, "mixed": MIXED, FP64: FP64, MIXED: MIXED}


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def _check_points(p: torch.Tensor, what: str) -> torch.Tensor:
    if not isinstance(p, torch.Tensor) or not p.is_cuda:
        raise _capi.InvalidArgument(1, f"{what} must be a CUDA tensor")
    if p.dtype != torch.float64:
        raise _capi.InvalidArgument(1, f"{what} must be float64 (Coordinate = double)")
    if p.dim() != 2:
        raise _capi.InvalidArgument(1, f"{what} must be rank 2")
    return p


def _multi_rank(comm) -> bool:
    """True for a torch.distributed process group of more than one rank."""
    import torch.distributed as dist
    return (dist.is_available() and isinstance(comm, dist.ProcessGroup) and dist.is_initialized()
            and dist.get_world_size(comm) > 1)


def _comm_size(comm) -> int:
    if comm is None:
        return 1
    for attr in ("Get_size", "size"):
        f = getattr(comm, attr, None)
        if callable(f):
            return int(f())
    if isinstance(comm, int):
        return comm
    return 1


class PointCloudOperator:
    """Base class of the meshfree operators (virtual apply)."""

    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor) -> None:
        raise NotImplementedError


class MovingLeastSquaresOperator(PointCloudOperator):
    """Moving least squares transfer between point clouds (one rank).

    ``MovingLeastSquaresOperator(comm, source_points, target_points,
    rbf=Wendland(0), basis=MultivariatePolynomialBasis(Linear, 3))`` builds the
    operator (search, weights, moments, pseudo-inverse, coefficients) on the
    GPU; ``apply(source_values, target_values)`` writes every target value.
    Extensions beyond the reference: ``k`` (neighbours, default the basis
    size as in the reference), ``radius`` (radius search instead of kNN) and
    ``precision`` ("fp64" = the reference algorithm, "mixed") and
    ``keep_points`` (keep copies of the points for the coordinate adjoint).
    """

    def __new__(cls, comm=None, *args, **kwargs):
        # a torch.distributed group of several ranks: the distributed operator
        # (search and value fetch across the ranks)
        if cls is MovingLeastSquaresOperator and _multi_rank(comm):
            from .distributed import DistributedMovingLeastSquaresOperator
            for key in ("radius", "keep_points"):
                if kwargs.pop(key, None) not in (None, False):
                    raise _capi.Unsupported(2, f"{key} is single-rank only")
            return DistributedMovingLeastSquaresOperator(comm, *args, **kwargs)
        return super().__new__(cls)

    def __init__(self, comm, source_points, target_points, rbf=None, basis=None, *,
                 k: int | None = None, radius: float | None = None, precision="fp64",
                 keep_points: bool = False, stream=None):
        self.polynomial_basis = basis or MultivariatePolynomialBasis(Linear, 3)
        self.radial_basis_function = rbf or Wendland(0)
        src = _check_points(source_points, "source_points")
        tgt = _check_points(target_points, "target_points")
        # DTK_REQUIRE(source dim == target dim), DTK_REQUIRE(dim == 3):
        # DTK_MovingLeastSquaresOperator_def.hpp:39-42
        if src.shape[1] != tgt.shape[1]:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == target_points.extent(1)")
        if src.shape[1] != 3 or self.polynomial_basis.dim != 3:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == 3")
        o = Options()
        lib().dtk_mls_default_options(C.byref(o))
        o.rbf = self.radial_basis_function.id
        o.basis = self.polynomial_basis.id
        o.k = 0 if k is None else int(k)
        o.radius = 0.0 if radius is None else float(radius)
        o.precision = _PRECISIONS[precision]
        o.comm_size = _comm_size(comm)
        o.keep_points = 1 if keep_points else 0
        self.options = o
        self._h = C.c_void_p()
        self._stream = stream
        check(lib().dtk_mls_create(C.byref(o), src.data_ptr(), src.shape[0], src.stride(0),
                                   src.stride(1), tgt.data_ptr(), tgt.shape[0], tgt.stride(0),
                                   tgt.stride(1), _stream(stream), C.byref(self._h)))
        self.n_source_points = int(src.shape[0])
        self.n_target_points = int(tgt.shape[0])

    @classmethod
    def transfer_host(cls, comm, source_points, target_points, source_values, target_values,
                      rbf=None, basis=None, *, k: int | None = None, radius: float | None = None,
                      precision="fp64", keep: bool = False, stream=None):
        """Setup and one apply from HOST tensors (float64, contiguous: points
        (n, 3), values (n,)), with the copies overlapping the work (pinned
        tensors for asynchronous copies); writes ``target_values`` in place.
        Returns the operator when ``keep`` (for further device applies)."""
        basis = basis or MultivariatePolynomialBasis(Linear, 3)
        rbf = rbf or Wendland(0)
        for t, what, shape in ((source_points, "source_points", 2), (target_points, "target_points", 2),
                               (source_values, "source_values", 1), (target_values, "target_values", 1)):
            if not isinstance(t, torch.Tensor) or t.is_cuda or t.dtype != torch.float64:
                raise _capi.InvalidArgument(1, f"{what} must be a float64 host tensor")
            if t.dim() != shape or not t.is_contiguous():
                raise _capi.InvalidArgument(1, f"{what} must be contiguous of rank {shape}")
        if source_points.shape[1] != 3 or target_points.shape[1] != 3 or basis.dim != 3:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == 3")
        if source_values.shape[0] != source_points.shape[0]:
            raise _capi.InvalidArgument(1, "source_values.extent(0) == n_source_points")
        if target_values.shape[0] != target_points.shape[0]:
            raise _capi.InvalidArgument(1, "target_values.extent(0) == n_target_points")
        o = Options()
        lib().dtk_mls_default_options(C.byref(o))
        o.rbf = rbf.id
        o.basis = basis.id
        o.k = 0 if k is None else int(k)
        o.radius = 0.0 if radius is None else float(radius)
        o.precision = _PRECISIONS[precision]
        o.comm_size = _comm_size(comm)
        h = C.c_void_p()
        check(lib().dtk_mls_transfer_host(C.byref(o), source_points.data_ptr(), source_points.shape[0],
                                          target_points.data_ptr(), target_points.shape[0],
                                          source_values.data_ptr(), target_values.data_ptr(),
                                          _stream(stream), C.byref(h) if keep else None))
        if not keep:
            return None
        op = cls.__new__(cls)
        op.polynomial_basis, op.radial_basis_function = basis, rbf
        op.options, op._h, op._stream = o, h, stream
        op.n_source_points = int(source_points.shape[0])
        op.n_target_points = int(target_points.shape[0])
        return op

    @classmethod
    def from_neighbors(cls, target_points, row: int, neighbor_points, indices, n_sources: int,
                       rbf=None, basis=None, *, precision="fp64", stream=None):
        """The operator for given kNN rows (the constructor after its search and
        coordinate fetch, DTK_MovingLeastSquaresOperator_def.hpp:64-118): row i
        of ``row`` entries has its neighbours' coordinates in
        ``neighbor_points[i*row:(i+1)*row]`` ((n_tgt*row, 3) float64 CUDA) and
        the positions of their values in the source-value array ``apply`` takes
        in ``indices`` (int32 CUDA, in [0, n_sources))."""
        basis = basis or MultivariatePolynomialBasis(Linear, 3)
        rbf = rbf or Wendland(0)
        tgt = _check_points(target_points, "target_points")
        nb = neighbor_points
        if (not isinstance(nb, torch.Tensor) or not nb.is_cuda or nb.dtype != torch.float64
                or nb.dim() != 2 or nb.shape[1] != 3 or not nb.is_contiguous()):
            raise _capi.InvalidArgument(1, "neighbor_points must be a contiguous (n, 3) float64 CUDA tensor")
        if (not isinstance(indices, torch.Tensor) or not indices.is_cuda or indices.dtype != torch.int32
                or indices.dim() != 1 or not indices.is_contiguous()):
            raise _capi.InvalidArgument(1, "indices must be a contiguous int32 CUDA tensor")
        if tgt.shape[1] != 3 or basis.dim != 3:
            raise _capi.InvalidArgument(1, "target_points.extent(1) == 3")
        if nb.shape[0] != tgt.shape[0] * row or indices.shape[0] != tgt.shape[0] * row:
            raise _capi.InvalidArgument(1, "neighbour arrays must hold n_targets * row entries")
        o = Options()
        lib().dtk_mls_default_options(C.byref(o))
        o.rbf, o.basis, o.precision = rbf.id, basis.id, _PRECISIONS[precision]
        h = C.c_void_p()
        check(lib().dtk_mls_create_from_neighbors(C.byref(o), tgt.data_ptr(), tgt.shape[0], tgt.stride(0),
                                                  tgt.stride(1), int(row), nb.data_ptr(), indices.data_ptr(),
                                                  int(n_sources), _stream(stream), C.byref(h)))
        op = cls.__new__(cls)
        op.polynomial_basis, op.radial_basis_function = basis, rbf
        op.options, op._h, op._stream = o, h, stream
        op.n_source_points = int(n_sources)
        op.n_target_points = int(tgt.shape[0])
        return op

    # -- reference API ------------------------------------------------------
    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor, stream=None) -> None:
        """target_values = T source_values; rank-1 fields, or rank-2 (n, n_comp) fields
        with any strides (each component transferred alike)."""
        st = _stream(stream if stream is not None else self._stream)
        if source_values.dim() == 2 or target_values.dim() == 2:
            check(lib().dtk_mls_apply_multi(self._h, *_fields(source_values, target_values), st))
            return
        for t, what in ((source_values, "source_values"), (target_values, "target_values")):
            if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
                raise _capi.InvalidArgument(1, f"{what} must be a float64 CUDA tensor")
            if t.dim() != 1 or (t.numel() > 1 and t.stride(0) != 1):
                raise _capi.InvalidArgument(1, f"{what} must be rank 1 and contiguous")
        check(lib().dtk_mls_apply(self._h, source_values.data_ptr(), source_values.shape[0],
                                  target_values.data_ptr(), target_values.shape[0], st))

    # -- extensions ------------------------------------------------------------
    def apply_adjoint(self, cot: torch.Tensor, source_values: torch.Tensor | None = None,
                      coords: bool = False, stream=None):
        """(dL/d source_values, dL/d source coordinates or None) for dL/d target = cot."""
        gv = torch.empty(self.n_source_points, dtype=torch.float64, device=cot.device)
        gc = torch.empty((self.n_source_points, 3), dtype=torch.float64, device=cot.device) if coords else None
        check(lib().dtk_mls_apply_adjoint(
            self._h, cot.data_ptr(), cot.shape[0],
            source_values.data_ptr() if source_values is not None else None,
            gv.data_ptr(), gc.data_ptr() if gc is not None else None,
            _stream(stream if stream is not None else self._stream)))
        return gv, gc

    def to_bytes(self) -> bytes:
        """The operator product (offset, indices, coefficients) as a byte string."""
        n = C.c_int64()
        check(lib().dtk_mls_export_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        check(lib().dtk_mls_export(self._h, buf, n.value, _stream(self._stream)))
        return buf.raw

    @classmethod
    def from_bytes(cls, data: bytes, stream=None) -> "MovingLeastSquaresOperator":
        """An operator whose apply uses a product written by ``to_bytes`` (no setup)."""
        op = cls.__new__(cls)
        op._h = C.c_void_p()
        op._stream = stream
        check(lib().dtk_mls_import(data, len(data), _stream(stream), C.byref(op._h)))
        n_src, n_tgt = C.c_int64(), C.c_int64()
        check(lib().dtk_mls_get_sizes(op._h, C.byref(n_src), C.byref(n_tgt), None))
        op.n_source_points, op.n_target_points = n_src.value, n_tgt.value
        op.polynomial_basis = op.radial_basis_function = op.options = None
        return op

    def save(self, path) -> None:
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def load(cls, path, stream=None) -> "MovingLeastSquaresOperator":
        with open(path, "rb") as f:
            return cls.from_bytes(f.read(), stream)

    def csr(self):
        """(offset, indices, coefficients) device tensors (copies)."""
        off, idx, coeff = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnz, f32 = C.c_int64(), C.c_int32()
        check(lib().dtk_mls_get_csr(self._h, C.byref(off), C.byref(idx), C.byref(coeff),
                                    C.byref(nnz), C.byref(f32)))
        torch.cuda.synchronize()
        n = nnz.value
        o = _from_device(off.value, self.n_target_points + 1, torch.int32)
        i = _from_device(idx.value, n, torch.int32)
        c = _from_device(coeff.value, n, torch.float32 if f32.value else torch.float64)
        return o, i, c

    @property
    def nnz(self) -> int:
        n = C.c_int64()
        check(lib().dtk_mls_get_sizes(self._h, None, None, C.byref(n)))
        return n.value

    @property
    def underdetermined(self) -> int:
        n = C.c_int64()
        check(lib().dtk_mls_underdetermined_count(self._h, C.byref(n)))
        return n.value

    @property
    def rotations(self) -> int:
        """FP64 Jacobi rotations performed by the setup."""
        n = C.c_int64()
        check(lib().dtk_mls_get_rotation_count(self._h, C.byref(n), None))
        return n.value

    @property
    def rotations_fp32(self) -> int:
        """FP32 Jacobi rotations performed by the setup (mixed form)."""
        n = C.c_int64()
        check(lib().dtk_mls_get_rotation_count(self._h, None, C.byref(n)))
        return n.value

    @property
    def stage_times_ms(self):
        a, b = C.c_float(), C.c_float()
        check(lib().dtk_mls_get_stage_times(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    @property
    def search_times_ms(self):
        """(tree build + target sort, query kernels) device milliseconds of the create."""
        a, b = C.c_float(), C.c_float()
        check(lib().dtk_mls_get_search_times(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().dtk_mls_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MovingLeastSquaresBatch:
    """Many independent MLS transfers set up and applied together (extension).

    The reference builds one ``MovingLeastSquaresOperator`` per problem; this
    batch gives each problem the same results while sharing one search tree,
    one setup pass and one apply launch per row-length bin.  ``problems`` is a
    sequence of dicts with keys ``source_points``, ``target_points`` (float64
    CUDA (n, 3) tensors), and optionally ``rbf``, ``basis``, ``k`` or
    ``radius`` (every problem kNN, or every problem radius).  Values are packed
    problem after problem: ``apply(source_values, target_values)`` takes the
    concatenation of every problem's source values and writes the
    concatenation of the target values; ``source_offsets`` and
    ``target_offsets`` give each problem's range.  ``graph=True`` replays the
    apply schedule from a captured CUDA graph.
    """

    def __init__(self, problems, *, precision="fp64", stream=None):
        problems = list(problems)
        if not problems:
            raise _capi.InvalidArgument(1, "a batch needs at least one problem")
        n = len(problems)
        opts = (Options * n)()
        src_parts, tgt_parts = [], []
        src_off, tgt_off = [0], [0]
        for p, pr in enumerate(problems):
            src = _check_points(pr["source_points"], "source_points")
            tgt = _check_points(pr["target_points"], "target_points")
            if src.shape[1] != 3 or tgt.shape[1] != 3:
                raise _capi.InvalidArgument(1, "source_points.extent(1) == 3")
            o = opts[p]
            lib().dtk_mls_default_options(C.byref(o))
            o.rbf = (pr.get("rbf") or Wendland(0)).id
            o.basis = (pr.get("basis") or MultivariatePolynomialBasis(Linear, 3)).id
            o.k = int(pr.get("k") or 0)
            o.radius = float(pr.get("radius") or 0.0)
            o.precision = _PRECISIONS[precision]
            src_parts.append(src)
            tgt_parts.append(tgt)
            src_off.append(src_off[-1] + src.shape[0])
            tgt_off.append(tgt_off[-1] + tgt.shape[0])
        self.source_points = torch.cat(src_parts).contiguous()
        self.target_points = torch.cat(tgt_parts).contiguous()
        self.source_offsets = src_off
        self.target_offsets = tgt_off
        self.n_problems = n
        self._stream = stream
        so = (C.c_int64 * (n + 1))(*src_off)
        to = (C.c_int64 * (n + 1))(*tgt_off)
        self._h = C.c_void_p()
        check(lib().dtk_mls_batch_create(n, opts, so, self.source_points.data_ptr(), to,
                                         self.target_points.data_ptr(), _stream(stream),
                                         C.byref(self._h)))

    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor, graph: bool = True,
              stream=None) -> None:
        for t, n, what in ((source_values, self.source_offsets[-1], "source_values"),
                           (target_values, self.target_offsets[-1], "target_values")):
            if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
                raise _capi.InvalidArgument(1, f"{what} must be a float64 CUDA tensor")
            if t.dim() != 1 or t.shape[0] != n or (n > 1 and t.stride(0) != 1):
                raise _capi.InvalidArgument(1, f"{what} must be contiguous of length {n}")
        check(lib().dtk_mls_batch_apply(self._h, source_values.data_ptr(), target_values.data_ptr(),
                                        1 if graph else 0,
                                        _stream(stream if stream is not None else self._stream)))

    def resetup(self, source_points: torch.Tensor | None = None, target_points: torch.Tensor | None = None,
                stream=None) -> None:
        """Recompute the coefficients for new coordinates (packed like the
        create's, same counts), keeping the create's neighbour rows; replays a
        captured CUDA graph of the persistent setup when the point arrays are
        the ones of the previous call.  None keeps the current points."""
        src = self.source_points if source_points is None else source_points
        tgt = self.target_points if target_points is None else target_points
        for t, ref, what in ((src, self.source_points, "source_points"), (tgt, self.target_points, "target_points")):
            _check_points(t, what)
            if t.shape != ref.shape or not t.is_contiguous():
                raise _capi.InvalidArgument(1, f"{what} must be contiguous of shape {tuple(ref.shape)}")
        self.source_points, self.target_points = src, tgt
        check(lib().dtk_mls_batch_resetup(self._h, src.data_ptr(), tgt.data_ptr(),
                                          _stream(stream if stream is not None else self._stream)))

    @property
    def config(self) -> dict:
        """The tuned configuration: lanes a target of the setup per row class,
        lanes a row of the apply per length bin (non-empty bins), setup graph replays."""
        sl = (C.c_int32 * 3)()
        al = (C.c_int32 * 32)()
        n = C.c_int64()
        check(lib().dtk_mls_batch_get_config(self._h, sl, al, C.byref(n)))
        return {"setup_lanes": {"knn_rows": sl[0], "rows_le_32": sl[1], "rows_gt_32": sl[2]},
                "apply_lanes_by_bin": {f"<={1 << b}": al[b] for b in range(32) if al[b]},
                "setup_graph_replays": n.value}

    def csr(self):
        """(offset, indices, coefficients) over all problems; indices are packed source indices."""
        off, idx, coeff = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnz, f32 = C.c_int64(), C.c_int32()
        check(lib().dtk_mls_batch_get_csr(self._h, C.byref(off), C.byref(idx), C.byref(coeff),
                                          C.byref(nnz), C.byref(f32)))
        torch.cuda.synchronize()
        n = nnz.value
        o = _from_device(off.value, self.target_offsets[-1] + 1, torch.int32)
        i = _from_device(idx.value, n, torch.int32)
        c = _from_device(coeff.value, n, torch.float32 if f32.value else torch.float64)
        return o, i, c

    @property
    def stage_times_ms(self):
        """(search, setup) device milliseconds and the host planning milliseconds."""
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        check(lib().dtk_mls_batch_get_stage_times(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().dtk_mls_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fields(source_values, target_values):
    """(ptr, n, n_comp, point stride, component stride) of both rank-2 fields, flattened
    into the argument order of the *_apply_multi entry points (stream excluded)."""
    out = []
    n_comp = None
    for t, what in ((source_values, "source_values"), (target_values, "target_values")):
        if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
            raise _capi.InvalidArgument(1, f"{what} must be a float64 CUDA tensor")
        if t.dim() == 1:
            t = t.unsqueeze(1)
        if t.dim() != 2:
            raise _capi.InvalidArgument(1, f"{what} must be rank 1 or 2")
        if n_comp is not None and t.shape[1] != n_comp:
            raise _capi.InvalidArgument(1, "source_values.extent(1) == target_values.extent(1)")
        n_comp = t.shape[1]
        out.append((t.data_ptr(), t.shape[0], t.stride(0), t.stride(1)))
    (sp, sn, sps, scs), (tp, tn, tps, tcs) = out
    return sp, sn, n_comp, sps, scs, tp, tn, tps, tcs


class NearestNeighborOperator(PointCloudOperator):
    """Nearest-neighbour transfer between point clouds (one rank).

    ``NearestNeighborOperator(comm, source_points, target_points)`` finds the
    nearest source of every target (ties to the smaller source index);
    ``apply(source_values, target_values)`` copies each target's nearest
    source value (rank-1 or rank-2 fields).
    Mirrors DTK_NearestNeighborOperator_decl.hpp:27-49.
    """

    def __new__(cls, comm=None, *args, **kwargs):
        if cls is NearestNeighborOperator and _multi_rank(comm):
            from .distributed import DistributedNearestNeighborOperator
            return DistributedNearestNeighborOperator(comm, *args, **kwargs)
        return super().__new__(cls)

    def __init__(self, comm, source_points, target_points, *, stream=None):
        src = _check_points(source_points, "source_points")
        tgt = _check_points(target_points, "target_points")
        if src.shape[1] != tgt.shape[1] or src.shape[1] != 3:
            raise _capi.InvalidArgument(1, "source_points.extent(1) == target_points.extent(1) == 3")
        self._h = C.c_void_p()
        self._stream = stream
        check(lib().dtk_nn_create(src.data_ptr(), src.shape[0], src.stride(0), src.stride(1),
                                  tgt.data_ptr(), tgt.shape[0], tgt.stride(0), tgt.stride(1),
                                  _comm_size(comm), _stream(stream), C.byref(self._h)))
        self.n_source_points = int(src.shape[0])
        self.n_target_points = int(tgt.shape[0])

    def apply(self, source_values: torch.Tensor, target_values: torch.Tensor, stream=None) -> None:
        check(lib().dtk_nn_apply_multi(self._h, *_fields(source_values, target_values),
                                       _stream(stream if stream is not None else self._stream)))

    @property
    def indices(self) -> torch.Tensor:
        """Nearest source index of every target (a copy)."""
        p, n = C.c_void_p(), C.c_int64()
        check(lib().dtk_nn_get_indices(self._h, C.byref(p), C.byref(n)))
        torch.cuda.synchronize()
        return _from_device(p.value, n.value, torch.int32)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().dtk_nn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """Exposes a raw device pointer through __cuda_array_interface__."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3, "strides": None}


_TYPESTR = {torch.int32: "<i4", torch.float32: "<f4", torch.float64: "<f8"}


def _from_device(ptr: int, n: int, dtype) -> torch.Tensor:
    """Copy of n elements at a device pointer owned by the library."""
    if n == 0 or not ptr:
        return torch.empty(0, dtype=dtype, device="cuda")
    view = torch.as_tensor(_DeviceArray(ptr, n, _TYPESTR[dtype]), device="cuda")
    return view.clone()


def kernel_launch_count() -> int:
    """Kernels the library has launched so far in this process."""
    return int(lib().dtk_kernel_launch_count())


def release_cached_memory() -> None:
    """Return the device memory cached in the library's pools to the driver
    (memory that live operators own stays); the pools keep freed blocks, up
    to 1/8 of a device's memory, so that repeated setups need not map memory
    again."""
    check(lib().dtk_release_cached_memory())


def set_setup_lanes(rows_le_32: int = 0, rows_gt_32: int = 0) -> None:
    """Fix the lanes a target of the batched setup's gather phases (powers of
    two in [1, 32]) for the batches created afterwards; 0 = tuned by timing."""
    check(lib().dtk_set_setup_lanes(int(rows_le_32), int(rows_gt_32)))


def knn_search(source_points: torch.Tensor, target_points: torch.Tensor, k: int, stream=None):
    """(offset, indices) of the k nearest sources per target by (d2, index)."""
    src = _check_points(source_points, "source_points")
    tgt = _check_points(target_points, "target_points")
    row = min(int(k), src.shape[0])
    offset = torch.empty(tgt.shape[0] + 1, dtype=torch.int32, device=tgt.device)
    idx = torch.empty(max(1, tgt.shape[0] * row), dtype=torch.int32, device=tgt.device)
    check(lib().dtk_knn_search(src.data_ptr(), src.shape[0], src.stride(0), src.stride(1),
                               tgt.data_ptr(), tgt.shape[0], tgt.stride(0), tgt.stride(1),
                               int(k), offset.data_ptr(), idx.data_ptr(), _stream(stream)))
    return offset, idx[: tgt.shape[0] * row]


def svd_pinv(matrices: torch.Tensor, stream=None):
    """Batched DTK Jacobi pseudo-inverse of (count, n, n) float64 CUDA matrices."""
    a = matrices.contiguous()
    if a.dtype != torch.float64 or not a.is_cuda or a.dim() != 3 or a.shape[1] != a.shape[2]:
        raise _capi.InvalidArgument(1, "matrices must be a (count, n, n) float64 CUDA tensor")
    out = torch.empty_like(a)
    under = C.c_int64()
    check(lib().dtk_svd_pinv(a.shape[1], a.shape[0], a.data_ptr(), out.data_ptr(),
                             C.byref(under), _stream(stream)))
    return out, under.value
