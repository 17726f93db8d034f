// Shared internals of the GB300 MLS transfer library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <vector>

#include <cfloat>
#include <climits>
#include <cstdint>
#include <exception>
#include <functional>
#include <new>
#include <string>

#include "../../include/dtk_gb300.h"

namespace dtk
{

// ---------------------------------------------------------------------------
// Host-side error plumbing: every C-ABI entry point returns a dtk_status and
// records a message for dtk_last_error().
// ---------------------------------------------------------------------------
void set_error( std::string const &msg );

struct Error
{
    dtk_status status;
    std::string msg;
};

#define DTK_CUDA_OR_THROW( expr )                                              \
    do                                                                         \
    {                                                                          \
        cudaError_t e__ = ( expr );                                            \
        if ( e__ != cudaSuccess )                                              \
            throw ::dtk::Error{e__ == cudaErrorMemoryAllocation                \
                                   ? DTK_ERR_OOM                               \
                                   : DTK_ERR_CUDA,                             \
                               std::string( #expr ) + ": " +                   \
                                   cudaGetErrorString( e__ )};                 \
    } while ( 0 )

#define DTK_REQUIRE_OR_THROW( cond, msg )                                      \
    do                                                                         \
    {                                                                          \
        if ( !( cond ) )                                                       \
            throw ::dtk::Error{DTK_ERR_INVALID_ARG,                            \
                               std::string( "DTK_REQUIRE( " #cond " ): " ) +   \
                                   ( msg )};                                   \
    } while ( 0 )

// Runs f and maps what it throws to a dtk_status (and the thread's last
// error message): every extern "C" entry point is one guarded call.
template <class F>
inline dtk_status guarded( F &&f )
{
    try
    {
        f();
        return DTK_OK;
    }
    catch ( Error const &e )
    {
        set_error( e.msg );
        return e.status;
    }
    catch ( std::bad_alloc const & )
    {
        set_error( "host allocation failed" );
        return DTK_ERR_OOM;
    }
    catch ( std::exception const &e )
    {
        set_error( e.what() );
        return DTK_ERR_INTERNAL;
    }
}

// Data the kernels read or write must be device memory (or managed, or
// mapped pinned host memory): pageable host memory is refused here with an
// error that says so, instead of faulting in a kernel.
inline void require_device_memory( void const *p, char const *what )
{
    if ( !p )
        return;
    cudaPointerAttributes a{};
    cudaError_t const e = cudaPointerGetAttributes( &a, p );
    if ( e != cudaSuccess )
    {
        cudaGetLastError();
        if ( e == cudaErrorInvalidValue )
            throw Error{DTK_ERR_INVALID_ARG, std::string( what ) + " is not a pointer CUDA can use"};
        throw Error{DTK_ERR_CUDA, std::string( what ) + ": " + cudaGetErrorString( e )};
    }
    if ( a.type == cudaMemoryTypeUnregistered )
        throw Error{DTK_ERR_INVALID_ARG, std::string( what ) +
                                             " is host memory unknown to CUDA: pass device memory "
                                             "(host buffers go through dtk_mls_transfer_host)"};
}

// Point-cloud arguments of an entry point: count, pointer and strides (the
// entry points check device memory after every argument check).
inline void validate_points( double const *p, int64_t n, int64_t ps, int64_t ds, char const *what )
{
    DTK_REQUIRE_OR_THROW( n >= 0, std::string( what ) + " count is negative" );
    DTK_REQUIRE_OR_THROW( n == 0 || p != nullptr, std::string( what ) + " pointer is null" );
    DTK_REQUIRE_OR_THROW( n <= INT32_MAX, std::string( what ) + " count exceeds int32 indices" );
    DTK_REQUIRE_OR_THROW( n == 0 || ( ps != 0 || n == 1 ) && ds != 0,
                          std::string( what ) + " strides are zero" );
}

// The library's stream-ordered memory pool on the current device: freed
// blocks stay cached across synchronizations up to 1/8 of the device's
// memory (the default pool returns them at every synchronization, and the
// next create pays to map them again); dtk_release_cached_memory trims it.
cudaMemPool_t device_pool();

// Stream-ordered device buffer from the library's pool (cudaFreeAsync frees).
template <class T>
struct DeviceBuffer
{
    T *ptr = nullptr;
    size_t n = 0;
    cudaStream_t stream = nullptr;

    DeviceBuffer() = default;
    DeviceBuffer( size_t count, cudaStream_t s ) { allocate( count, s ); }
    DeviceBuffer( DeviceBuffer const & ) = delete;
    DeviceBuffer &operator=( DeviceBuffer const & ) = delete;
    DeviceBuffer( DeviceBuffer &&o ) noexcept { *this = std::move( o ); }
    DeviceBuffer &operator=( DeviceBuffer &&o ) noexcept
    {
        release();
        ptr = o.ptr;
        n = o.n;
        stream = o.stream;
        o.ptr = nullptr;
        o.n = 0;
        return *this;
    }
    ~DeviceBuffer() { release(); }

    void allocate( size_t count, cudaStream_t s )
    {
        release();
        stream = s;
        n = count;
        if ( count )
            DTK_CUDA_OR_THROW( cudaMallocFromPoolAsync( (void **)&ptr, count * sizeof( T ), device_pool(), s ) );
    }
    void release()
    {
        if ( ptr )
            cudaFreeAsync( ptr, stream );
        ptr = nullptr;
        n = 0;
    }
    T *get() const { return ptr; }
};

// Lifetime of a handle's device buffers: the stream they were allocated on
// (the create call's; it must stay valid until the handle is destroyed) and
// an event recorded on a call's stream after the work of every call that
// uses them (TouchOnExit).  At destroy the home stream waits for that event
// and the buffers are freed there, so a call queued on another stream never
// races the free, and the home stream's next allocations reuse the blocks.
struct HandleLife
{
    cudaStream_t home = nullptr;
    cudaEvent_t last_use = nullptr;
    explicit HandleLife( cudaStream_t s )
        : home( s )
    {
        DTK_CUDA_OR_THROW( cudaEventCreateWithFlags( &last_use, cudaEventDisableTiming ) );
    }
    HandleLife( HandleLife const & ) = delete;
    HandleLife &operator=( HandleLife const & ) = delete;
    ~HandleLife()
    {
        if ( last_use )
            cudaEventDestroy( last_use );
    }
    void touch( cudaStream_t s ) { cudaEventRecord( last_use, s ); }
    // Moves the buffers' frees to the home stream, behind last_use (called
    // from a handle's destructor, which does not throw).
    template <class... Buffers>
    void retire( Buffers &...buffers ) noexcept
    {
        cudaStreamWaitEvent( home, last_use, 0 );
        ( ( buffers.stream = home ), ... );
    }
};

// Records the handle's last-use event on the call's stream when the entry
// point returns or throws, so that its buffers outlive the work it queued.
struct TouchOnExit
{
    HandleLife *life;
    cudaStream_t s;
    ~TouchOnExit()
    {
        if ( life )
            life->touch( s );
    }
};

// A named NVTX range over the host code that enqueues a stage (the labels
// of the reference's DTK_MARK_REGION, "DTK_" + name, where a stage has one;
// no-ops unless a profiling tool is attached).
struct NvtxRange
{
    explicit NvtxRange( char const *name ) { nvtxRangePushA( name ); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange( NvtxRange const & ) = delete;
    NvtxRange &operator=( NvtxRange const & ) = delete;
};

// Running count of this library's kernel launches (diagnostics).
long long &launch_counter();

// Launch-error check after a kernel launch (also counts the launch).
inline void check_launch( char const *what )
{
    ++launch_counter();
    cudaError_t e = cudaGetLastError();
    if ( e != cudaSuccess )
        throw Error{DTK_ERR_CUDA, std::string( what ) + ": " + cudaGetErrorString( e )};
}

// SM count of the current device (cached per device).
int num_sms();

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current
// device.  The attribute is per device, so it is set once per (device,
// kernel) and again whenever a larger size is asked for; thread-safe.
void set_dynamic_smem( void const *kernel, size_t bytes );
template <class K>
inline void ensure_dynamic_smem( K *kernel, size_t bytes )
{
    set_dynamic_smem( reinterpret_cast<void const *>( kernel ), bytes );
}

// Caps of the bounded device loops (dtk_set_loop_caps; 0 = built in):
// Jacobi rotations per moment matrix of size m (built in: 200 m^2 + 2000)
// and tree-traversal steps per query (built in: the tree's wide-node count,
// which a search never exceeds).
unsigned long long jacobi_cap( int m );
int jacobi_log_cap(); // rotations logged before U is formed (JACOBI_LOG unless lowered for a test)
int64_t traversal_cap( int64_t wide_nodes );

inline int basis_size( int basis )
{
    return basis == DTK_CONSTANT3 ? 1 : basis == DTK_LINEAR3 ? 4 : basis == DTK_QUADRATIC3 ? 10 : -1;
}

// Device status word bits (set by bounded device loops).
enum : unsigned
{
    DEV_TIMEOUT = 1u,
    DEV_STACK_OVERFLOW = 2u,
    DEV_BAD_INDEX = 4u,
    DEV_NONFINITE_SOURCE = 8u, // a source coordinate is NaN or infinite
    DEV_NONFINITE_TARGET = 16u, // a target coordinate is NaN or infinite
    DEV_BAD_TASK = 32u          // a task of the persistent setup out of range (skipped)
};

// NaN or infinite: all exponent bits set (integer pipe).
__device__ __forceinline__ bool nonfinite_bits( double v )
{
    return ( (unsigned long long)__double_as_longlong( v ) & 0x7ff0000000000000ull ) ==
           0x7ff0000000000000ull;
}

// ---------------------------------------------------------------------------
// Device math shared by the kernels.
// ---------------------------------------------------------------------------

// Squared distance with the contract's association and separately rounded
// operations: (dx*dx + dy*dy) + dz*dz, dx = s.x - t.x.
__device__ __forceinline__ double dist2_rn( double sx, double sy, double sz,
                                            double tx, double ty, double tz )
{
    double const dx = __dsub_rn( sx, tx );
    double const dy = __dsub_rn( sy, ty );
    double const dz = __dsub_rn( sz, tz );
    return __dadd_rn( __dadd_rn( __dmul_rn( dx, dx ), __dmul_rn( dy, dy ) ),
                      __dmul_rn( dz, dz ) );
}

// Compactly supported RBFs on the scaled argument x = distance / radius
// (DTK_CompactlySupportedRadialBasisFunctions.hpp:45-147).
template <class T>
__device__ __forceinline__ T rbf_eval( int rbf, T x )
{
    T const y = T( 1 ) - x;
    switch ( rbf )
    {
    case DTK_WENDLAND0:
        return y * y;
    case DTK_WENDLAND2:
        return y * y * y * y * ( T( 4 ) * x + T( 1 ) );
    case DTK_WENDLAND4:
        return y * y * y * y * y * y * ( T( 35 ) * x * x + T( 18 ) * x + T( 3 ) );
    case DTK_WENDLAND6:
        return y * y * y * y * y * y * y * y *
               ( T( 32 ) * x * x * x + T( 25 ) * x * x + T( 8 ) * x + T( 1 ) );
    case DTK_WU2:
        return y * y * y * y * ( T( 3 ) * x * x * x + T( 12 ) * x * x + T( 16 ) * x + T( 4 ) );
    case DTK_WU4:
        return y * y * y * y * y * y *
               ( T( 5 ) * x * x * x * x * x + T( 30 ) * x * x * x * x +
                 T( 72 ) * x * x * x + T( 82 ) * x * x + T( 36 ) * x + T( 6 ) );
    case DTK_BUHMANN2:
        return T( 2 ) * x * x * x * x * log( x ) - T( 7.0 / 2.0 ) * x * x * x * x +
               T( 16 / 3.0 ) * x * x * x - T( 2 ) * x * x + T( 1.0 / 6.0 );
    case DTK_BUHMANN3:
        return x * x * x * x * x * x * x * x - T( 84.0 / 5.0 ) * x * x * x * x * x * x +
               T( 1024.0 / 5.0 ) * x * x * x * x * sqrt( x ) -
               T( 378 ) * x * x * x * x + T( 1024.0 / 5.0 ) * x * x * x * sqrt( x ) -
               T( 84.0 / 5.0 ) * x * x + T( 1 );
    default: // DTK_BUHMANN4
        return T( 99.0 / 35.0 ) * x * x * x * x * x * x * x * x -
               T( 132 ) * x * x * x * x * x * x +
               T( 9216.0 / 35.0 ) * x * x * x * x * x * sqrt( x ) -
               T( 11264.0 / 35.0 ) * x * x * x * x * sqrt( x ) +
               T( 198 ) * x * x * x * x - T( 396.0 / 5.0 ) * x * x + T( 1 );
    }
}

// d rbf / dx (hand-derived; used by the adjoint).
__device__ __forceinline__ double rbf_deriv( int rbf, double x )
{
    double const y = 1.0 - x;
    switch ( rbf )
    {
    case DTK_WENDLAND0:
        return -2.0 * y;
    case DTK_WENDLAND2:
        return -20.0 * x * y * y * y;
    case DTK_WENDLAND4:
        return -56.0 * x * ( 5.0 * x + 1.0 ) * y * y * y * y * y;
    case DTK_WENDLAND6:
        return -22.0 * x * ( 16.0 * x * x + 7.0 * x + 1.0 ) * y * y * y * y * y * y * y;
    case DTK_WU2:
        return -7.0 * x * ( 3.0 * x * x + 9.0 * x + 8.0 ) * y * y * y;
    case DTK_WU4:
        return -11.0 * x * ( 5.0 * x * x * x * x + 25.0 * x * x * x + 48.0 * x * x + 40.0 * x + 8.0 ) *
               y * y * y * y * y;
    case DTK_BUHMANN2:
        return x > 0.0 ? 8.0 * x * x * x * log( x ) - 12.0 * x * x * x + 16.0 * x * x - 4.0 * x : 0.0;
    case DTK_BUHMANN3:
    {
        double const r = sqrt( x );
        double const x2 = x * x, x3 = x2 * x, x5 = x3 * x2, x7 = x5 * x2;
        return 8.0 * x7 - 504.0 / 5.0 * x5 + 4608.0 / 5.0 * x3 * r - 1512.0 * x3 +
               3584.0 / 5.0 * x2 * r - 168.0 / 5.0 * x;
    }
    default:
    {
        double const r = sqrt( x );
        double const x2 = x * x, x3 = x2 * x, x4 = x2 * x2, x5 = x4 * x, x7 = x5 * x2;
        return 792.0 / 35.0 * x7 - 792.0 * x5 + 50688.0 / 35.0 * x4 * r -
               50688.0 / 35.0 * x3 * r + 792.0 * x3 - 792.0 / 5.0 * x;
    }
    }
}

// Polynomial basis in 3-D, order 1, x, y, z, x^2, xy, xz, y^2, yz, z^2
// (DTK_MultivariatePolynomialBasis.hpp:98-125).
template <int M, class T>
__device__ __forceinline__ void basis_eval( T x, T y, T z, T *p )
{
    p[0] = T( 1 );
    if constexpr ( M >= 4 )
    {
        p[1] = x;
        p[2] = y;
        p[3] = z;
    }
    if constexpr ( M == 10 )
    {
        p[4] = x * x;
        p[5] = x * y;
        p[6] = x * z;
        p[7] = y * y;
        p[8] = y * z;
        p[9] = z * z;
    }
}

// Rank-2 field (n points x n_comp components): element (i, c) at
// base[i*ps + c*cs] (LayoutRight: cs = 1; LayoutLeft: ps = 1, cs = n).
struct FieldView
{
    double const *base;
    double *wbase;
    int64_t n, n_comp, ps, cs;
};

// Strided point access: element (i, d) at base[i*ps + d*ds].
struct PointsView
{
    double const *base;
    int64_t n, ps, ds;
    __host__ __device__ double operator()( int64_t i, int d ) const
    {
        return base[i * ps + d * ds];
    }
};

// The neighbours of CSR entries: from the tree's Morton-sorted FP64 copy by
// sorted position when pos is set (consecutive targets' neighbours are then
// close in memory), else from the caller's points by original index.  Both
// give the same coordinates.
struct Neighbours
{
    PointsView src;
    int32_t const *idx;
    int32_t const *pos;
    double2 const *s2;
    // the entry's reference (position or index) for a bounds check against src.n
    __device__ __forceinline__ int32_t ref( int64_t e ) const { return pos ? pos[e] : idx[e]; }
    __device__ __forceinline__ void xyz( int64_t e, double &x, double &y, double &z ) const
    {
        if ( pos )
        {
            int64_t const p = pos[e];
            double2 const a = __ldg( s2 + 2 * p ), b = __ldg( s2 + 2 * p + 1 );
            x = a.x;
            y = a.y;
            z = b.x;
        }
        else
        {
            int64_t const sj = idx[e];
            x = src( sj, 0 );
            y = src( sj, 1 );
            z = src( sj, 2 );
        }
    }
};

// ---------------------------------------------------------------------------
// Internal library API shared between translation units.
// ---------------------------------------------------------------------------

// Device-wide exclusive scan of n int64 counts (out may alias nothing);
// out has n+1 entries, out[n] = total.  Returns nothing; total is on device.
void exclusive_scan_i64( int64_t const *in, int64_t *out, int64_t n, cudaStream_t s );

// Stable LSD radix sort of (keys, values) pairs by the low `bits` bits of
// the keys.  Buffers are swapped internally; the result ends in keys/values.
void radix_sort_pairs( uint32_t *keys, uint32_t *values, int64_t n, int bits,
                       cudaStream_t s );

// Linear BVH over source points with 32-point leaf buckets.
struct Lbvh
{
    int64_t n = 0;        // points
    int64_t n_leaves = 0; // leaves: the Morton cells of at most 32 points
    double lo[3], hi[3];  // scene bounds (host copy)
    DeviceBuffer<double2> s2;         // Morton-sorted coordinates: (x, y), (z, original index bits)
    DeviceBuffer<float4> f4;          // the same, centred on the scene box, FP32 (x, y, z), and the leaf's first position
    DeviceBuffer<uint32_t> codes;     // Morton codes in sorted order
    DeviceBuffer<uint32_t> grp;       // group (problem) of each sorted point; empty if ungrouped
    DeviceBuffer<uint32_t> perm;      // sorted position -> original index
    DeviceBuffer<int32_t> leaf_start; // first sorted position of each leaf, then n (n_leaves + 1)
    DeviceBuffer<int32_t> leaf_of;    // leaf of each sorted position
    DeviceBuffer<float4> nodes;       // 4 float4 per binary internal node (released after the collapse)
    DeviceBuffer<float4> wide;        // 16 float4 per 8-wide node (the queries' tree)
    DeviceBuffer<int2> wide_range;    // 8 leaf ranges per wide node (trees over several problems)
    DeviceBuffer<float4> wide_cell;   // per wide node: its Morton cell as a box (lo + parent, hi), inset
    int64_t n_wide = 0;
    int wide_levels = 0;              // the deepest wide node's level (root 0)
    DeviceBuffer<float4> root_box;    // box of the whole tree (2 float4)
    DeviceBuffer<double> scene;       // lo[3], Morton scale[3], hi[3], centre[3], bound S, FP32 lo/scale
};

// group (optional, per input point) makes the order problem-major: the
// points of group g then occupy one contiguous range of sorted positions.
// after_scene (optional) runs on the host once the scene box is enqueued on
// s (tree.scene), before the rest of the build.
void build_lbvh( PointsView src, Lbvh &tree, unsigned *status, cudaStream_t s,
                 uint32_t const *group = nullptr, int64_t n_groups = 0,
                 std::function<void()> const &after_scene = nullptr );

// Morton order of query points (sorted query ids) using the tree's scene box;
// with groups, problem-major and Morton within each problem.  An order buffer
// already holding max(1, tgt.n) entries is used as it is.
// (status, when not null, receives DEV_NONFINITE_TARGET for a target with a
// NaN or infinite coordinate.)
void sort_queries( Lbvh const &tree, PointsView tgt, DeviceBuffer<uint32_t> &order,
                   cudaStream_t s, uint32_t const *group = nullptr, int64_t n_groups = 0,
                   unsigned *status = nullptr );

// The tree over src on s and, on a second stream as soon as the scene box is
// known, the order of the queries, concurrently with the rest of the build;
// s waits for the order before this returns.
// (tgt_ready, when not null, is an event the query points wait for.)
// A NaN or infinite coordinate in either cloud is DTK_ERR_INVALID_ARG,
// thrown here before any search (one synchronisation of s).
void build_tree_and_order( PointsView src, PointsView tgt, Lbvh &tree, DeviceBuffer<uint32_t> &order,
                           unsigned *status, cudaStream_t s, uint32_t const *src_group = nullptr,
                           uint32_t const *tgt_group = nullptr, int64_t n_groups = 0,
                           cudaEvent_t tgt_ready = nullptr );

// Problems of a batch, all optional (null: one problem over all sources,
// uniform k / radius): per group the sorted-position range of its sources,
// the group of each target, per-group k and per-group radius.
struct GroupArgs
{
    int64_t const *src_off = nullptr;
    uint32_t const *tgt_grp = nullptr;
    int32_t const *k = nullptr;
    double const *r = nullptr;
};

// kNN: writes each row at offset[target] (ascending (d2, index)): the
// sources' original indices in idx and, when pos is not null, their sorted
// positions in the tree (tree.perm maps a position to its index).
void knn_query( Lbvh const &tree, PointsView tgt, uint32_t const *order, int k,
                GroupArgs const &groups, int32_t const *offset, int32_t *idx, unsigned *status,
                cudaStream_t s, int32_t *pos = nullptr );

// Radius: count pass (counts[n_tgt]) and fill pass given offsets.
void radius_count( Lbvh const &tree, PointsView tgt, uint32_t const *order, double r,
                   GroupArgs const &groups, int64_t *counts, unsigned *status, cudaStream_t s );
void radius_fill( Lbvh const &tree, PointsView tgt, uint32_t const *order, double r,
                  GroupArgs const &groups, int32_t const *offset, int32_t *idx, unsigned *status,
                  cudaStream_t s );

// Setup (coefficients) kernels.
struct SetupArgs
{
    PointsView src, tgt;
    int32_t const *offset;
    int32_t const *idx;
    uint32_t const *order; // target processing order (may be null)
    int64_t n_tgt;
    int rbf, basis;
    bool rows_sorted;     // rows ascending by distance (kNN)
    // when set: the neighbours' sorted positions (parallel to idx) and the
    // tree's Morton-sorted FP64 points, (x, y), (z, index bits) per position;
    // the kernels gather the neighbours from there (the same values as
    // src(idx), in the order the search walked them)
    int32_t const *pos = nullptr;
    double2 const *s2 = nullptr;
    double *coeff64;      // FP64 form output
    float *coeff32;       // mixed form output
    unsigned long long *underdetermined;
    unsigned long long *rotations;     // FP64 Jacobi rotations
    unsigned long long *rotations32;   // FP32 Jacobi rotations (mixed form)
    unsigned *status;
};
void setup_fp64( SetupArgs const &a, cudaStream_t s );
void setup_mixed( SetupArgs const &a, cudaStream_t s );
constexpr int FUSED_MAX_ROW = 32; // longest row the fused one-thread-per-target kernels take

// Persistent batched setup (FP64 Jacobi): the targets of a bucketed list in
// tasks of up to 32 targets of one bucket, taken by warps from a counter.
constexpr int SETUP_RBFS = 9, SETUP_PATHS = 3, SETUP_KEYS = 3 * SETUP_RBFS * SETUP_PATHS;
constexpr int BS_WARPS = 8; // warps a block of the persistent setup (one block an SM)
struct SetupTask
{
    int32_t first; // the task's first target in the bucketed list
    uint8_t count; // targets (1 .. 32)
    uint8_t key;   // bucket: (basis * SETUP_RBFS + rbf) * SETUP_PATHS + path
    uint8_t lanes; // lanes a target in the gather phases (a power of two, 1 .. 32)
    uint8_t pad;
};
// A Jacobi thread's global work area, interleaved by thread: the rotation
// log, JACOBI_LOG (cos, sin) pairs and JACOBI_LOG pivot bytes (p * 16 + q),
// then U (M x M, formed only for targets whose rotations outrun the log) from
// JACOBI_U0 doubles on.
constexpr int JACOBI_LOG = 160;
constexpr int JACOBI_U0 = 2 * JACOBI_LOG + JACOBI_LOG / 8;
constexpr int BS_MAX_M = 10;
__host__ __device__ constexpr int jacobi_work_doubles( int m )
{
    return JACOBI_U0 + m * m;
}
struct BatchSetupArgs
{
    Neighbours nb;
    PointsView tgt;
    int32_t const *offset;
    uint32_t const *list; // targets in bucket order
    int64_t n_list;       // its length (the tasks are checked against it)
    SetupTask const *tasks;
    int64_t const *n_tasks; // task count (device), read when t_end < 0
    int64_t t_begin = 0, t_end = -1;
    int force_lanes = 0; // > 0: every task with this many lanes (the tuner's samples)
    bool rows_sorted = false;
    double *coeff64 = nullptr;
    float *coeff32 = nullptr;
    unsigned long long *underdetermined, *rotations;
    unsigned *status;
    unsigned *counter; // zeroed by batch_setup before the launch
    double *u_work;    // jacobi_work_doubles( BS_MAX_M ) doubles per thread of the grid (batch_setup_threads)
    unsigned jcap[3] = {0, 0, 0};
    int jlog = JACOBI_LOG;
};
void batch_setup( BatchSetupArgs const &a, cudaStream_t s );
int64_t batch_setup_threads();

// The device plan of a setup over targets of mixed classes (kept by a batch
// handle for its re-setups): the targets in bucket order, the bucket sizes,
// the task list and the persistent kernel's work area.
struct SetupPlan
{
    int64_t n = 0;
    int precision = 0;
    bool with_path0 = true;            // path 0 rows in the persistent kernel
    int lanes[3] = {1, 8, 32};         // lanes a target per path (paths 1 and 2 tunable)
    bool tuned[3] = {false, false, false};
    DeviceBuffer<uint32_t> list;       // targets, bucket order
    DeviceBuffer<unsigned> hist;       // targets per bucket
    DeviceBuffer<int64_t> n_tasks, path_first, bucket_start, bucket_task;
    DeviceBuffer<SetupTask> tasks;
    DeviceBuffer<unsigned> counter;
    DeviceBuffer<double> u_work;
    struct Bucket
    {
        int key;
        int64_t start, count;
    };
    std::vector<Bucket> mixed_buckets; // mixed-form kNN buckets (fused mixed kernel), once known
    ~SetupPlan();
};
// plan_setup: bucket sort and task layout (no synchronisation); fill_setup_tasks:
// the task list with the plan's lane counts; run_planned_setup: the persistent
// launch (plus the fused mixed kernel per mixed kNN bucket).
void plan_setup( SetupArgs const &a, int precision, uint8_t const *basis_of_group, uint8_t const *rbf_of_group,
                 uint32_t const *tgt_group, bool split_all, SetupPlan &plan, cudaStream_t s );
void fill_setup_tasks( SetupPlan &plan, cudaStream_t s );
void run_planned_setup( SetupArgs const &a, SetupPlan &plan, cudaStream_t s );
// Lane counts fixed by the caller for paths 1 and 2 (0: tuned by timing).
void fixed_setup_lanes( int &lanes1, int &lanes2 );

// Setup over targets of mixed classes, planned on the device: a stable key
// sort of the processing order `a.order` partitions the targets into buckets
// (basis, rbf, path), path 0 = rows up to FUSED_MAX_ROW (unless split_all),
// 1 = split rows up to 32, 2 = longer rows; every bucket runs in one
// persistent launch (FP64 Jacobi), except mixed-form kNN rows (path 0 of the
// mixed form), which run the fused mixed kernel.  The class of a target
// comes from its group (basis_of_group / rbf_of_group indexed by
// tgt_group[target]; null: the uniform a.basis / a.rbf).  `keep` keeps the
// plan (for re-setups); `tune` times the lane counts of paths 1 and 2.
void run_setup_plan( SetupArgs const &a, int precision, uint8_t const *basis_of_group,
                     uint8_t const *rbf_of_group, uint32_t const *tgt_group, bool split_all,
                     cudaStream_t s, SetupPlan *keep = nullptr, bool tune = false );

// Batched SVD pseudo-inverse (general n <= 64), DTK SVDFunctor semantics.
void svd_pinv_batched( int n, int64_t count, double const *a, double *pinv,
                       unsigned long long *underdetermined, unsigned *status,
                       cudaStream_t s );
// The same kernel on a caller-provided work area of 3 n^2 count doubles.
void svd_pinv_batched_work( int n, int64_t count, double const *a, double *pinv, double *work,
                            unsigned long long *underdetermined, unsigned *status,
                            cudaStream_t s );

// Apply kernels.
// Rank-2 fields: out(i, c) = sum_j coeff_j in(idx_j, c).
void apply_csr_multi( int64_t n_tgt, int32_t const *offset, int32_t const *idx, double const *coeff64,
                      float const *coeff32, FieldView in, FieldView out, cudaStream_t s );
void apply_csr( int64_t n_tgt, int32_t const *offset, int32_t const *idx,
                double const *coeff64, float const *coeff32, int uniform_row, int mean_row,
                double const *values, double *target, cudaStream_t s );
// Uniform rows over sorted positions: the values are permuted into the
// tree's order (perm: sorted position -> index) and gathered by position.
bool apply_sorted_supported( int uniform_row );
struct SortedValues
{
    DeviceBuffer<double> v64; // FP64 form
    DeviceBuffer<float2> v32; // mixed form: (hi, lo) = (fl32(v), fl32(v - hi))
};
// (perm null: the values in their own order, for entries that hold indices)
SortedValues permute_values( int64_t n_src, uint32_t const *perm, double const *values, bool f32,
                             cudaStream_t s );
// n_rows uniform rows starting at pos / coeff (a slice of the operator's),
// taken in the given order (the targets' Morton order: consecutive rows then
// share most of their neighbours' values in L1) or in row order
void apply_pos( int64_t n_rows, int uniform_row, int32_t const *pos, double const *coeff64, float const *coeff32,
                SortedValues const &v, double *target, cudaStream_t s, uint32_t const *order = nullptr );
void apply_sorted( int64_t n_tgt, int uniform_row, int32_t const *pos, double const *coeff64,
                   float const *coeff32, int64_t n_src, uint32_t const *perm, double const *values,
                   double *target, cudaStream_t s, uint32_t const *order = nullptr );

// Adjoint kernels.
struct AdjointArgs
{
    int64_t n_src, n_tgt;
    int32_t const *offset, *idx;
    double const *coeff64;
    float const *coeff32;
    double const *cot;
    double *grad_values;
    // transpose CSR (source -> entries), built on demand
    int32_t const *t_offset, *t_entry;
    int32_t const *entry_row;
};
void build_transpose( int64_t n_src, int64_t n_tgt, int64_t nnz, int32_t const *offset,
                      int32_t const *idx, DeviceBuffer<int32_t> &t_offset,
                      DeviceBuffer<int32_t> &t_entry, DeviceBuffer<int32_t> &entry_row,
                      cudaStream_t s );
void apply_transpose( AdjointArgs const &a, cudaStream_t s );
void coord_grad( SetupArgs const &a, double const *values, double const *cot,
                 double *grad_xyz, cudaStream_t s );

} // namespace dtk
