/*
 * dtk_gb300.h -- C ABI of the GB300-native moving-least-squares (MLS)
 * point-cloud transfer of DataTransferKit, on one rank.
 *
 * Plain C: pointers, sizes and POD structs only.  Every function returns a
 * dtk_status; none throws.  All data pointers are DEVICE pointers unless
 * stated otherwise; the caller owns every input and output buffer, the
 * handle owns the operator's CSR product (offset, indices, coefficients).
 * Calls on one handle are ordered on the stream they are given and are not
 * re-entrant.  `stream` is a cudaStream_t (NULL = legacy default stream).
 * A handle's buffers live on the stream its create call was given: that
 * stream must stay valid until the handle is destroyed, where the buffers
 * are freed on it behind the work of the handle's last call (on whichever
 * stream that call was given).
 *
 * Reference interface replaced (paths inside the DataTransferKit project):
 *   DataTransferKit::MovingLeastSquaresOperator<DeviceType, RBF, Basis>
 *     packages/Meshfree/src/DTK_MovingLeastSquaresOperator_decl.hpp:36-63
 *   its constructor (setup: search, weights, moments, pseudo-inverse,
 *   coefficients)  DTK_MovingLeastSquaresOperator_def.hpp:24-119
 *   apply(source_values, target_values)
 *                   DTK_MovingLeastSquaresOperator_def.hpp:121-141
 */
#ifndef DTK_GB300_H
#define DTK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dtk_mls_s *dtk_mls_handle;
typedef struct CUstream_st *dtk_stream_t; /* == cudaStream_t */

typedef enum
{
    DTK_OK = 0,
    DTK_ERR_INVALID_ARG = 1, /* a DTK_REQUIRE precondition failed */
    DTK_ERR_UNSUPPORTED = 2, /* e.g. comm_size > 1, dimension != 3 */
    DTK_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    DTK_ERR_OOM = 4,         /* device allocation failed */
    DTK_ERR_TIMEOUT = 5,     /* a bounded device loop hit its cap */
    DTK_ERR_INTERNAL = 6
} dtk_status;

/* Compactly supported RBFs: DTK_CompactlySupportedRadialBasisFunctions.hpp:42-147 */
typedef enum
{
    DTK_WENDLAND0 = 0,
    DTK_WENDLAND2 = 1,
    DTK_WENDLAND4 = 2,
    DTK_WENDLAND6 = 3,
    DTK_WU2 = 4,
    DTK_WU4 = 5,
    DTK_BUHMANN2 = 6,
    DTK_BUHMANN3 = 7,
    DTK_BUHMANN4 = 8
} dtk_rbf;

/* MultivariatePolynomialBasis<., 3>: DTK_MultivariatePolynomialBasis.hpp:98-125 */
typedef enum
{
    DTK_CONSTANT3 = 0, /* m = 1  */
    DTK_LINEAR3 = 1,   /* m = 4  */
    DTK_QUADRATIC3 = 2 /* m = 10 */
} dtk_basis;

typedef enum
{
    /* The reference algorithm in FP64: unscaled relative coordinates,
     * two-sided largest-pivot Jacobi with DTK's absolute DBL_EPSILON stop and
     * truncation (DTK_DetailsSVDImpl.hpp:197-302). */
    DTK_FP64 = 0,
    /* Centring and scaling by the support radius, FP32 basis / weights /
     * moment assembly and FP32 coefficients for apply; the Jacobi rotations
     * and the pseudo-inverse truncation in FP64. */
    DTK_MIXED = 1
} dtk_precision;

typedef struct
{
    int32_t rbf;       /* dtk_rbf; reference default Wendland<0> */
    int32_t basis;     /* dtk_basis; reference default Linear3 */
    int32_t k;         /* neighbours per target; 0 = basis size (reference) */
    int32_t precision; /* dtk_precision */
    double radius;     /* > 0: radius search instead of kNN (extension) */
    int32_t comm_size; /* ranks of the communicator; must be 1 */
    int32_t keep_points; /* != 0: the handle keeps copies of the points
                            (24 B per point) for the coordinate adjoint */
} dtk_mls_options;

/* Options of MovingLeastSquaresOperator<Device> with its template defaults:
 * Wendland<0>, Linear3, k = basis size, FP64, comm_size 1, keep_points 0. */
void dtk_mls_default_options(dtk_mls_options *opts);

/* Setup.  Replaces the constructor, DTK_MovingLeastSquaresOperator_def.hpp:24-119.
 * src / tgt: n x 3 coordinates, element (i, d) at ptr[i*pt_stride + d*dim_stride]
 * (doubles; LayoutRight: (3, 1); LayoutLeft: (1, n)).  Preconditions as the
 * reference: dimension 3 (implied), n_src > 0 (DTK_CHECK(!tree.empty())).
 * A NaN or infinite coordinate in either cloud is DTK_ERR_INVALID_ARG,
 * detected before the search runs.
 * Returns when the product is complete (the reference fences). */
dtk_status dtk_mls_create(const dtk_mls_options *opts, const double *src,
                          int64_t n_src, int64_t src_pt_stride,
                          int64_t src_dim_stride, const double *tgt,
                          int64_t n_tgt, int64_t tgt_pt_stride,
                          int64_t tgt_dim_stride, dtk_stream_t stream,
                          dtk_mls_handle *out);

/* Setup from given neighbour rows (the distributed operator's setup, after
 * its neighbours have been found across ranks and fetched; the constructor's
 * stages after the search and the fetch of the coordinates,
 * DTK_MovingLeastSquaresOperator_def.hpp:64-118).  Row i holds `row` entries
 * (1..32): entry e = i*row + j has its neighbour's coordinates at
 * nb_points[3e .. 3e+2] (row-major, n_tgt*row x 3) and the index of its value
 * in the source-value array the handle's apply takes (indices[e] in
 * [0, n_src)).  The support radius is the row's farthest neighbour, so the
 * order of a row only orders its sums; rows ascending by (d2, global index)
 * give the coefficients a single-rank dtk_mls_create computes for the same
 * rows.  The handle applies like one from dtk_mls_create over n_src
 * sources (no coordinate adjoint: it keeps no points, and keep_points != 0
 * is DTK_ERR_UNSUPPORTED).  kNN rows only
 * (opts->radius > 0 -> DTK_ERR_UNSUPPORTED); opts->comm_size must be 1 (the
 * handle is this rank's part); indices out of range -> DTK_ERR_INVALID_ARG.
 * Synchronous. */
dtk_status dtk_mls_create_from_neighbors(const dtk_mls_options *opts, const double *tgt,
                                         int64_t n_tgt, int64_t tgt_pt_stride,
                                         int64_t tgt_dim_stride, int32_t row,
                                         const double *nb_points, const int32_t *indices,
                                         int64_t n_src, dtk_stream_t stream,
                                         dtk_mls_handle *out);

/* apply: target_values[i] = sum_j coeff_j * source_values[idx_j].
 * Replaces MovingLeastSquaresOperator::apply, DTK_MovingLeastSquaresOperator_def.hpp:121-141,
 * with its preconditions n_source_values == n_src and n_target_values ==
 * n_tgt (DTK_REQUIRE at :129-130).  Writes every target value; enqueued on
 * `stream`, asynchronous (the reference's apply fences: follow with
 * dtk_stream_synchronize for that behaviour, as the C++ drop-in does). */
dtk_status dtk_mls_apply(dtk_mls_handle h, const double *source_values,
                         int64_t n_source_values, double *target_values,
                         int64_t n_target_values, dtk_stream_t stream);

/* Adjoint of apply and of the setup (extension; the reference has none).
 * cot = dL/d(target values), n_cot == n_tgt.
 * grad_values[s] = sum over entries j with idx_j == s of coeff_j * cot[row(j)]
 * (deterministic transpose gather in ascending entry order; overwrites n_src
 * values).  When grad_coords is non-NULL it receives dL/d(source coordinates)
 * as an n_src x 3 row-major array (overwritten), through the weights, the
 * support radius (whose max sends its gradient to the farthest neighbour) and
 * the pseudo-inverse, recomputed per target in FP64 with the connectivity
 * fixed, and gathered deterministically like grad_values; this part needs
 * `source_values` (the field of the forward apply) and a handle created with
 * keep_points != 0.  Rows whose moments are rank-deficient use the truncated
 * pseudo-inverse in place of the inverse.  Synchronous. */
dtk_status dtk_mls_apply_adjoint(dtk_mls_handle h, const double *cot,
                                 int64_t n_cot, const double *source_values,
                                 double *grad_values, double *grad_coords,
                                 dtk_stream_t stream);

/* Read-only view of the CSR product for parity checks.  coeff points to
 * doubles (FP64 form) or floats (mixed form, *coeff_is_fp32 = 1). */
dtk_status dtk_mls_get_csr(dtk_mls_handle h, const int32_t **offset,
                           const int32_t **indices, const void **coeff,
                           int64_t *nnz, int32_t *coeff_is_fp32);

/* Sizes of the operator. */
dtk_status dtk_mls_get_sizes(dtk_mls_handle h, int64_t *n_src, int64_t *n_tgt,
                             int64_t *nnz);

/* Number of targets whose moment matrix was rank-deficient (the value the
 * reference returns from invertMoments, DTK_DetailsMovingLeastSquaresOperatorImpl.hpp:263-291). */
dtk_status dtk_mls_underdetermined_count(dtk_mls_handle h, int64_t *count);

/* Device-side timings of the last create (milliseconds): search, setup. */
dtk_status dtk_mls_get_stage_times(dtk_mls_handle h, float *search_ms,
                                   float *setup_ms);
/* The search stage split (milliseconds): tree build with the Morton sort of
 * the targets, and the kNN / radius query kernels. */
dtk_status dtk_mls_get_search_times(dtk_mls_handle h, float *build_ms,
                                    float *query_ms);

/* Jacobi rotations the create performed, in FP64 and (mixed form) in FP32;
 * the basis of the FLOP counts in the benchmark.  Either pointer may be NULL. */
dtk_status dtk_mls_get_rotation_count(dtk_mls_handle h, int64_t *rotations,
                                      int64_t *rotations_fp32);

/* Setup and apply in one call with HOST buffers (the constructor followed by
 * one apply, for callers whose points and values live in host memory):
 * src_host n_src x 3 and tgt_host n_tgt x 3 row-major points, values_host
 * n_src source values in, target_values_host n_tgt values out.  The copies
 * overlap the work: the targets and the values travel on a second stream
 * while the tree is built, and the results come back in row slices while the
 * apply finishes the rest.  The copies are asynchronous only from pinned
 * host memory (cudaHostAlloc / cudaHostRegister); from pageable memory the
 * results are the same.  Synchronous: returns after the results are in host
 * memory.  When `out` is not NULL it receives the operator (for further
 * applies on device buffers; destroy it with dtk_mls_destroy).  No
 * counterpart in the reference (its operator takes device Views). */
dtk_status dtk_mls_transfer_host(const dtk_mls_options *opts,
                                 const double *src_host, int64_t n_src,
                                 const double *tgt_host, int64_t n_tgt,
                                 const double *values_host,
                                 double *target_values_host,
                                 dtk_stream_t stream, dtk_mls_handle *out);

/* Blocks the calling host thread until the work queued on `stream` is done
 * (the fence the reference's apply ends with, Kokkos::deep_copy at
 * DTK_MovingLeastSquaresOperator_def.hpp:140; the C++ drop-in's apply calls
 * it).  An error of that work is DTK_ERR_CUDA. */
dtk_status dtk_stream_synchronize(dtk_stream_t stream);

/* Running count of the kernels this library has launched in the process
 * (diagnostics; not a reference interface). */
int64_t dtk_kernel_launch_count(void);

/* Device memory: the library allocates its handles' buffers and its scratch
 * in its own stream-ordered pool, one per device, which keeps freed blocks
 * cached across synchronizations (up to 1/8 of the device's memory) so that
 * repeated setups do not map memory again.  This returns the cached blocks
 * of every device's pool to the driver; memory that live handles own stays,
 * and so does memory whose free is still queued behind work on a stream.
 * No counterpart in the reference (Kokkos manages its own memory). */
dtk_status dtk_release_cached_memory(void);

dtk_status dtk_mls_destroy(dtk_mls_handle h);

/* ---- search only (the ArborX query the constructor runs,
 *      DTK_MovingLeastSquaresOperator_def.hpp:47-62) ----
 * kNN: row i = the min(k, n_src) nearest sources by (d2, index), ascending,
 * d2 = (dx*dx + dy*dy) + dz*dz in FP64 with separately rounded operations.
 * offset must hold n_tgt+1 and indices n_tgt*min(k, n_src) entries. */
dtk_status dtk_knn_search(const double *src, int64_t n_src,
                          int64_t src_pt_stride, int64_t src_dim_stride,
                          const double *tgt, int64_t n_tgt,
                          int64_t tgt_pt_stride, int64_t tgt_dim_stride,
                          int32_t k, int32_t *offset, int32_t *indices,
                          dtk_stream_t stream);

/* ---- device steps of a distributed operator (the exchange is the caller's) ----
 * A multi-rank host side (the C++ drop-in over an MPI-like communicator, the
 * Python operator over torch.distributed) runs the reference's distributed
 * search and fetch (DTK_MovingLeastSquaresOperator_def.hpp:47-67,133-134;
 * DTK_DetailsNearestNeighborOperatorImpl.hpp:47-192) with these and
 * dtk_mls_create_from_neighbors; all arrays are device arrays unless named
 * _host.
 * dtk_knn_search_d2: the rows of dtk_knn_search (min(k, n_src) entries a
 *   target, ascending by (d2, index)) and each entry's d2, (dx*dx + dy*dy)
 *   + dz*dz in FP64 with separately rounded operations.  Synchronous.
 * dtk_points_bounds: the box of a cloud, box_host = (min x, y, z, max x, y, z);
 *   (+inf, -inf) for an empty cloud.  Synchronous.
 * dtk_points_pack: a strided cloud copied to a row-major n x 3 array.
 * dtk_gather_points: out[e] = the point indices[e] names: source indices[e]
 *   when below n_src, else row indices[e] - n_src of `extra` (row-major); an
 *   index outside both -> DTK_ERR_INVALID_ARG.  Synchronous.
 * dtk_gather_values: out[i] = values[indices[i]]; an index outside [0, n) ->
 *   DTK_ERR_INVALID_ARG.  Synchronous. */
dtk_status dtk_knn_search_d2(const double *src, int64_t n_src, int64_t src_pt_stride,
                             int64_t src_dim_stride, const double *tgt, int64_t n_tgt,
                             int64_t tgt_pt_stride, int64_t tgt_dim_stride, int32_t k,
                             int32_t *indices, double *d2, dtk_stream_t stream);
dtk_status dtk_points_bounds(const double *pts, int64_t n, int64_t pt_stride, int64_t dim_stride,
                             double *box_host, dtk_stream_t stream);
dtk_status dtk_points_pack(const double *pts, int64_t n, int64_t pt_stride, int64_t dim_stride,
                           double *out, dtk_stream_t stream);
dtk_status dtk_gather_points(const double *src, int64_t n_src, int64_t src_pt_stride,
                             int64_t src_dim_stride, const double *extra, int64_t n_extra,
                             const int32_t *indices, int64_t nnz, double *out, dtk_stream_t stream);
dtk_status dtk_gather_values(const double *values, int64_t n, const int32_t *indices, int64_t m,
                             double *out, dtk_stream_t stream);

/* ---- the operator product on disk and on the wire (extension) ----
 * The CSR that create produces (offset, source indices, coefficients, the
 * members of DTK_MovingLeastSquaresOperator_decl.hpp:56-62) as a flat
 * little-endian byte string with a header and a checksum (layout in
 * csrc/dtk_io.cu), so that apply can be reused across restarts and shared
 * with other processes.  export copies into a HOST buffer of
 * dtk_mls_export_size bytes (synchronous); import validates a buffer
 * (magic, version, sizes, offsets, index range, checksum: otherwise
 * DTK_ERR_INVALID_ARG) and returns a handle whose apply and values-adjoint
 * work as the original's (no coordinate adjoint: the points are not stored). */
dtk_status dtk_mls_export_size(dtk_mls_handle h, int64_t *bytes);
dtk_status dtk_mls_export(dtk_mls_handle h, void *host_buffer, int64_t bytes,
                          dtk_stream_t stream);
dtk_status dtk_mls_import(const void *host_buffer, int64_t bytes,
                          dtk_stream_t stream, dtk_mls_handle *out);

/* ---- rank-2 (multi-component) fields ----
 * apply for n x n_comp fields with (point, component) strides in elements:
 * LayoutRight (component fastest): (n_comp, 1); LayoutLeft: (1, n).  Each
 * component is the rank-1 apply of that column.  Extension: the reference's
 * MLS apply takes rank-1 views (DTK_MovingLeastSquaresOperator_decl.hpp:52-54);
 * its fetch handles rank 2 (DTK_DetailsNearestNeighborOperatorImpl.hpp:53-56,89-93). */
dtk_status dtk_mls_apply_multi(dtk_mls_handle h, const double *source_values,
                               int64_t n_source_values, int64_t n_comp,
                               int64_t src_pt_stride, int64_t src_comp_stride,
                               double *target_values, int64_t n_target_values,
                               int64_t tgt_pt_stride, int64_t tgt_comp_stride,
                               dtk_stream_t stream);

/* ---- NearestNeighborOperator (DTK_NearestNeighborOperator_decl.hpp:27-49) ----
 * create (DTK_NearestNeighborOperator_def.hpp:23-71): the nearest source of
 * every target, (d^2, index) order (ties to the smaller source index);
 * comm_size > 1 -> DTK_ERR_UNSUPPORTED; an empty source cloud ->
 * DTK_ERR_INVALID_ARG (the reference's DTK_CHECK(!search_tree.empty())).
 * apply (:73-86): target_values[i] = source_values[nearest(i)]; the
 * DTK_REQUIREs on the extents -> DTK_ERR_INVALID_ARG.  Device pointers. */
typedef struct dtk_nn_s *dtk_nn_handle;
dtk_status dtk_nn_create(const double *src, int64_t n_src, int64_t src_pt_stride,
                         int64_t src_dim_stride, const double *tgt, int64_t n_tgt,
                         int64_t tgt_pt_stride, int64_t tgt_dim_stride,
                         int32_t comm_size, dtk_stream_t stream, dtk_nn_handle *out);
dtk_status dtk_nn_apply(dtk_nn_handle h, const double *source_values,
                        int64_t n_source_values, double *target_values,
                        int64_t n_target_values, dtk_stream_t stream);
dtk_status dtk_nn_apply_multi(dtk_nn_handle h, const double *source_values,
                              int64_t n_source_values, int64_t n_comp,
                              int64_t src_pt_stride, int64_t src_comp_stride,
                              double *target_values, int64_t n_target_values,
                              int64_t tgt_pt_stride, int64_t tgt_comp_stride,
                              dtk_stream_t stream);
/* The nearest source index of every target (device array of n_targets). */
dtk_status dtk_nn_get_indices(dtk_nn_handle h, const int32_t **indices,
                              int64_t *n_targets);
dtk_status dtk_nn_destroy(dtk_nn_handle h);

/* ---- batched pseudo-inverse (the SVDFunctor kernel, DTK_DetailsSVDImpl.hpp:39-309) ----
 * count row-major n x n matrices -> their pseudo-inverses with DTK's
 * absolute DBL_EPSILON tolerances; *underdetermined (host) receives the
 * number of matrices with a dropped singular value.  n <= 64. */
dtk_status dtk_svd_pinv(int32_t n, int64_t count, const double *a,
                        double *pinv, int64_t *underdetermined,
                        dtk_stream_t stream);

/* The same batched pseudo-inverse without any device allocation; it has no
 * counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: code that runs under a fixed device-memory budget or inside a
 * framework whose allocator owns the device memory, and code that cannot take
 * the implicit device synchronisation an allocation may cause.  The work
 * matrices (E, U, V: 3 n^2 doubles per matrix) and the counters live in one
 * static device array of DTK_SVD_NOALLOC_MAX_DOUBLES doubles (8 MiB), which
 * every GPU that loads this library holds until the process exits.  Requests
 * with 3 * n * n * count > DTK_SVD_NOALLOC_MAX_DOUBLES are rejected with
 * DTK_ERR_INVALID_ARG.  The first call on a device looks up the array's
 * device address, so make it before any stream capture.  Every call shares
 * the array (it keeps the last call's contents; each call clears its
 * counters), so calls that overlap on the GPU -- other streams, other host
 * threads -- race; serialise them.  Synchronises `stream` to return
 * *underdetermined. */
#define DTK_SVD_NOALLOC_MAX_DOUBLES (1 << 20)
dtk_status dtk_svd_pinv_noalloc(int32_t n, int64_t count, const double *a,
                                double *pinv, int64_t *underdetermined,
                                dtk_stream_t stream);

/* ---- batched uneven transfers (extension) ----
 * n_problems independent operators in one schedule.  Problem p uses
 * sources [src_offsets[p], src_offsets[p+1]) and targets
 * [tgt_offsets[p], tgt_offsets[p+1]) of the packed row-major n x 3 arrays,
 * and options opts[p] (HOST arrays: src_offsets, tgt_offsets, opts).
 * The batch's CSR product is one global CSR over all targets with global
 * source indices.  One search serves all problems; the setup is one
 * persistent launch over tasks of 32 targets of one (basis, rbf) bucket
 * (FP64 Jacobi rows; mixed-form kNN rows run the fused mixed kernel per
 * bucket), with the lanes a target of its gather phases tuned by timing on a
 * sample of the tasks at create (dtk_set_setup_lanes fixes them). */
typedef struct dtk_mls_batch_s *dtk_mls_batch_handle;
dtk_status dtk_mls_batch_create(int32_t n_problems, const dtk_mls_options *opts,
                                const int64_t *src_offsets, const double *src,
                                const int64_t *tgt_offsets, const double *tgt,
                                dtk_stream_t stream, dtk_mls_batch_handle *out);
/* All problems' apply: values/targets are packed like the points.  When
 * use_graph != 0 the apply schedule is captured once into a CUDA graph and
 * replayed. */
dtk_status dtk_mls_batch_apply(dtk_mls_batch_handle h, const double *src_values,
                               double *tgt_values, int32_t use_graph,
                               dtk_stream_t stream);
/* Re-setup on new coordinates (same packed layout and counts), keeping the
 * neighbour rows of the create: the coefficients are recomputed for the new
 * points (the support radius from the row's farthest entry).  The statistics
 * reset and the persistent setup launch are captured into a CUDA graph on the
 * first call for a pair of point arrays and replayed on later calls with the
 * same arrays.  Synchronous (reads the status).  With the create's points it
 * reproduces the create's coefficients bit for bit. */
dtk_status dtk_mls_batch_resetup(dtk_mls_batch_handle h, const double *src,
                                 const double *tgt, dtk_stream_t stream);
/* The chosen configuration: setup_lanes[3] = lanes a target per row class
 * (kNN rows, rows up to 32, longer rows), apply_lanes[32] = lanes a row per
 * length bin (0 for empty bins or before the first apply), and the number of
 * setup graph replays so far.  Any pointer may be NULL. */
dtk_status dtk_mls_batch_get_config(dtk_mls_batch_handle h, int32_t *setup_lanes,
                                    int32_t *apply_lanes, int64_t *setup_graph_replays);
dtk_status dtk_mls_batch_get_csr(dtk_mls_batch_handle h, const int32_t **offset,
                                 const int32_t **indices, const void **coeff,
                                 int64_t *nnz, int32_t *coeff_is_fp32);
dtk_status dtk_mls_batch_destroy(dtk_mls_batch_handle h);
/* Device time of the batch's search and setup stages (CUDA events), and the
 * host time the create call spent planning (bucketing targets, binning rows). */
dtk_status dtk_mls_batch_get_stage_times(dtk_mls_batch_handle h, float *search_ms,
                                         float *setup_ms, float *host_ms);

/* Caps of the bounded device loops, for tests and diagnostics (no
 * counterpart in the reference): Jacobi rotations per moment matrix (FP64
 * setup, split setup, batched pseudo-inverse) and tree-traversal steps per
 * query (kNN and radius search), for the calls made after it in this
 * process.  A loop that reaches its cap stops, sets a status bit, and the
 * call returns DTK_ERR_TIMEOUT with the device context intact, so a test can
 * drive the caps to exhaustion on an ordinary input.  0 restores the built-in
 * caps: 200 m^2 + 2000 rotations, and the tree's node count in steps (more
 * than a search takes).  Negative values -> DTK_ERR_INVALID_ARG. */
dtk_status dtk_set_loop_caps(int64_t jacobi_rotations, int64_t traversal_steps);

/* Rotations the FP64 Jacobi (FP64-form setup, persistent batched setup) logs
 * per moment matrix before it forms U explicitly, for tests (no counterpart
 * in the reference), for the calls made after it in this process.  Row 0 of
 * the pseudo-inverse is the logged rotations applied in reverse to one
 * vector; a matrix that takes more rotations forms U from the log and then
 * updates it rotation by rotation as the reference does.  0 forms U for
 * every matrix (the reference's product order); 160, the most, is the
 * default.  The two orders differ at rounding level.  Values outside
 * [0, 160] -> DTK_ERR_INVALID_ARG. */
dtk_status dtk_set_rotation_log(int32_t rotations);

/* Lanes a target in the gather phases of the persistent setup, for rows of
 * up to 32 entries and for longer rows (powers of two in [1, 32]; 0 = tuned
 * by timing, the default), for the batches created after it in this
 * process.  The lane count sets the order of the moment sums, so fixing it
 * makes the coefficients reproducible across processes.  Other values ->
 * DTK_ERR_INVALID_ARG. */
dtk_status dtk_set_setup_lanes(int32_t lanes_short, int32_t lanes_long);

/* Last error message of the calling host thread (never NULL). */
const char *dtk_last_error(void);
const char *dtk_status_string(dtk_status s);

#ifdef __cplusplus
}
#endif
#endif
