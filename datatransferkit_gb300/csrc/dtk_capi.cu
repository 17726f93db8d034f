// C ABI of the GB300 MLS transfer (declared in include/dtk_gb300.h).
//
// The handle mirrors the data members of
// DataTransferKit::MovingLeastSquaresOperator
// (packages/Meshfree/src/DTK_MovingLeastSquaresOperator_decl.hpp:56-62):
// the CSR offset, the source indices and the coefficients, plus the source
// count.  The reference's `_ranks` array is absent: on one rank every rank is
// 0 and the fetch is a local gather fused into apply.
#include "dtk_common.cuh"
#include "dtk_handle.cuh"

#include <atomic>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace dtk
{

namespace
{
thread_local std::string g_error;
}

void set_error( std::string const &msg ) { g_error = msg; }

long long &launch_counter()
{
    static long long n = 0;
    return n;
}

namespace
{
std::mutex g_pool_mutex;
std::vector<cudaMemPool_t> g_pools; // per device, created on first use
} // namespace

cudaMemPool_t device_pool()
{
    int dev = 0;
    DTK_CUDA_OR_THROW( cudaGetDevice( &dev ) );
    std::lock_guard<std::mutex> lock( g_pool_mutex );
    if ( g_pools.size() <= (size_t)dev )
        g_pools.resize( dev + 1, nullptr );
    if ( !g_pools[dev] )
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        DTK_CUDA_OR_THROW( cudaMemPoolCreate( &pool, &props ) );
        size_t free_b = 0, total_b = 0;
        DTK_CUDA_OR_THROW( cudaMemGetInfo( &free_b, &total_b ) );
        unsigned long long keep = total_b / 8;
        DTK_CUDA_OR_THROW( cudaMemPoolSetAttribute( pool, cudaMemPoolAttrReleaseThreshold, &keep ) );
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

namespace
{
std::mutex g_attr_mutex;
std::map<std::pair<int, void const *>, size_t> g_smem_set; // (device, kernel) -> bytes set
std::vector<int> g_sms;                                    // per device, 0 = not queried
} // namespace

namespace
{
std::atomic<int64_t> g_jacobi_cap{0}, g_traversal_cap{0};
std::atomic<int> g_jacobi_log{JACOBI_LOG};
std::atomic<int> g_setup_lanes1{0}, g_setup_lanes2{0};
}

unsigned long long jacobi_cap( int m )
{
    int64_t const c = g_jacobi_cap.load( std::memory_order_relaxed );
    return c > 0 ? (unsigned long long)c : 200ull * m * m + 2000ull;
}

int jacobi_log_cap()
{
    return g_jacobi_log.load( std::memory_order_relaxed );
}

void fixed_setup_lanes( int &lanes1, int &lanes2 )
{
    lanes1 = g_setup_lanes1.load( std::memory_order_relaxed );
    lanes2 = g_setup_lanes2.load( std::memory_order_relaxed );
}

int64_t traversal_cap( int64_t wide_nodes )
{
    int64_t const c = g_traversal_cap.load( std::memory_order_relaxed );
    return c > 0 && c < wide_nodes ? c : wide_nodes;
}

int num_sms()
{
    int dev = 0;
    DTK_CUDA_OR_THROW( cudaGetDevice( &dev ) );
    std::lock_guard<std::mutex> lock( g_attr_mutex );
    if ( g_sms.size() <= (size_t)dev )
        g_sms.resize( dev + 1, 0 );
    if ( !g_sms[dev] )
    {
        int sms = 0;
        DTK_CUDA_OR_THROW( cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev ) );
        g_sms[dev] = sms > 0 ? sms : 1;
    }
    return g_sms[dev];
}

void set_dynamic_smem( void const *kernel, size_t bytes )
{
    int dev = 0;
    DTK_CUDA_OR_THROW( cudaGetDevice( &dev ) );
    std::lock_guard<std::mutex> lock( g_attr_mutex );
    size_t &done = g_smem_set[{dev, kernel}];
    if ( done >= bytes )
        return;
    DTK_CUDA_OR_THROW( cudaFuncSetAttribute( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes ) );
    done = bytes;
}

__global__ void k_fill_uniform_offsets( int32_t *offset, int64_t n_tgt, int row )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n_tgt )
        offset[i] = (int32_t)( i * row );
}

__global__ void k_iota32( int32_t *out, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < n )
        out[i] = (int32_t)i;
}

// DEV_BAD_INDEX for an index outside [0, n)
__global__ void k_check_indices( int32_t const *idx, int64_t nnz, int64_t n, unsigned *status )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < nnz && ( idx[i] < 0 || idx[i] >= n ) )
        atomicOr( status, DEV_BAD_INDEX );
}

__global__ void k_narrow_offsets( int64_t const *in, int32_t *out, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        out[i] = (int32_t)in[i];
}

__global__ void k_pack_points( PointsView p, double *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < p.n )
    {
        out[3 * i + 0] = p( i, 0 );
        out[3 * i + 1] = p( i, 1 );
        out[3 * i + 2] = p( i, 2 );
    }
}

struct Geometry
{
    dtk_mls_options opts;
    int m = 0, k = 0, row = 0;
    bool radius_mode = false;
};

Geometry check_options( dtk_mls_options const *o )
{
    DTK_REQUIRE_OR_THROW( o != nullptr, "options pointer is null" );
    if ( o->comm_size != 1 )
        throw Error{DTK_ERR_UNSUPPORTED,
                    "only a single-rank communicator (MPI_COMM_SELF) is supported"};
    DTK_REQUIRE_OR_THROW( o->rbf >= DTK_WENDLAND0 && o->rbf <= DTK_BUHMANN4, "unknown rbf" );
    DTK_REQUIRE_OR_THROW( o->basis >= DTK_CONSTANT3 && o->basis <= DTK_QUADRATIC3,
                          "unknown polynomial basis" );
    DTK_REQUIRE_OR_THROW( o->precision == DTK_FP64 || o->precision == DTK_MIXED,
                          "unknown precision form" );
    DTK_REQUIRE_OR_THROW( o->k >= 0, "k is negative" );
    DTK_REQUIRE_OR_THROW( std::isfinite( o->radius ) && o->radius >= 0.0,
                          "radius must be finite and >= 0" );
    Geometry g;
    g.opts = *o;
    g.m = basis_size( o->basis );
    g.radius_mode = o->radius > 0.0;
    g.k = o->k ? o->k : g.m;
    if ( !g.radius_mode && g.k > 32 )
        throw Error{DTK_ERR_UNSUPPORTED, "kNN search supports k <= 32"};
    return g;
}

} // namespace dtk

using namespace dtk;

namespace dtk
{
// The create's work on stream s, for validated points; the targets are read
// only after `tgt_ready` (when not null) has fired.  Returns the handle.
std::unique_ptr<dtk_mls_s> create_impl( Geometry const &g, dtk_mls_options const *opts, PointsView sv,
                                        PointsView tv, cudaStream_t s, cudaEvent_t tgt_ready )
{
    int64_t const n_src = sv.n, n_tgt = tv.n;
    auto h = new dtk_mls_s( s );
    std::unique_ptr<dtk_mls_s> guard( h );
    TouchOnExit const touch{&h->life, s};
    h->opts = *opts;
    h->n_src = n_src;
    h->n_tgt = n_tgt;
    h->m = g.m;
    if ( opts->keep_points )
    {
        if ( tgt_ready )
            DTK_CUDA_OR_THROW( cudaStreamWaitEvent( s, tgt_ready, 0 ) );
        // packed n x 3 copies for the coordinate adjoint
        h->src_copy.allocate( 3 * n_src, s );
        h->tgt_copy.allocate( std::max<int64_t>( 1, 3 * n_tgt ), s );
        k_pack_points<<<(unsigned)( ( n_src + 255 ) / 256 ), 256, 0, s>>>( sv, h->src_copy.get() );
        check_launch( "k_pack_points" );
        if ( n_tgt )
        {
            k_pack_points<<<(unsigned)( ( n_tgt + 255 ) / 256 ), 256, 0, s>>>( tv, h->tgt_copy.get() );
            check_launch( "k_pack_points" );
        }
    }

    cudaEvent_t ev[4];
    for ( auto &e : ev )
        DTK_CUDA_OR_THROW( cudaEventCreate( &e ) );
    struct EvGuard
    {
        cudaEvent_t *e;
        ~EvGuard()
        {
            for ( int i = 0; i < 4; ++i )
                cudaEventDestroy( e[i] );
        }
    } evg{ev};
    DeviceBuffer<unsigned> status( 1, s );
    DeviceBuffer<unsigned long long> counters( 3, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( counters.get(), 0, 3 * sizeof( unsigned long long ), s ) );
    DTK_CUDA_OR_THROW( cudaEventRecord( ev[0], s ) );

    // --- search (ArborX tree + query, _def.hpp:47-62) ---
    Lbvh tree;
    // (the targets may still be arriving: the query order waits for them on
    // its own stream while the tree is built)
    build_tree_and_order( sv, tv, tree, h->order, status.get(), s, nullptr, nullptr, 0, tgt_ready );
    DTK_CUDA_OR_THROW( cudaEventRecord( ev[3], s ) );
    h->offset.allocate( n_tgt + 1, s );
    if ( !g.radius_mode )
    {
        int const row = (int)std::min<int64_t>( g.k, n_src );
        DTK_REQUIRE_OR_THROW( n_tgt * (int64_t)row <= INT32_MAX,
                              "n_targets * k exceeds int32 CSR offsets" );
        h->uniform_row = row;
        h->mean_row = row;
        h->nnz = n_tgt * (int64_t)row;
        k_fill_uniform_offsets<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>(
            h->offset.get(), n_tgt, row );
        check_launch( "k_fill_uniform_offsets" );
        h->idx.allocate( std::max<int64_t>( 1, h->nnz ), s );
        if ( apply_sorted_supported( row ) )
            h->pos.allocate( std::max<int64_t>( 1, h->nnz ), s );
        knn_query( tree, tv, h->order.get(), g.k, GroupArgs{}, h->offset.get(), h->idx.get(), status.get(), s,
                   h->pos.get() );
    }
    else
    {
        DeviceBuffer<int64_t> counts( std::max<int64_t>( 1, n_tgt ), s ),
            offs( n_tgt + 1, s );
        radius_count( tree, tv, h->order.get(), g.opts.radius, GroupArgs{}, counts.get(), status.get(), s );
        exclusive_scan_i64( counts.get(), offs.get(), n_tgt, s );
        int64_t total = 0;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &total, offs.get() + n_tgt, sizeof( int64_t ),
                                            cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        DTK_REQUIRE_OR_THROW( total <= INT32_MAX, "neighbour count exceeds int32 CSR offsets" );
        h->nnz = total;
        h->mean_row = n_tgt ? (int)( ( total + n_tgt - 1 ) / n_tgt ) : 0;
        k_narrow_offsets<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( offs.get(),
                                                                              h->offset.get(), n_tgt );
        check_launch( "k_narrow_offsets" );
        h->idx.allocate( std::max<int64_t>( 1, total ), s );
        radius_fill( tree, tv, h->order.get(), g.opts.radius, GroupArgs{}, h->offset.get(), h->idx.get(),
                     status.get(), s );
    }
    DTK_CUDA_OR_THROW( cudaEventRecord( ev[1], s ) );

    // --- setup numerics (def.hpp:136-185) ---
    SetupArgs a{};
    a.src = sv;
    a.tgt = tv;
    a.offset = h->offset.get();
    a.idx = h->idx.get();
    a.order = h->order.get();
    a.n_tgt = n_tgt;
    a.rbf = g.opts.rbf;
    a.basis = g.opts.basis;
    a.rows_sorted = !g.radius_mode;
    if ( h->pos.get() )
    {
        a.pos = h->pos.get();
        a.s2 = tree.s2.get();
    }
    a.underdetermined = counters.get();
    a.rotations = counters.get() + 1;
    a.rotations32 = counters.get() + 2;
    a.status = status.get();
    if ( g.opts.precision == DTK_FP64 )
    {
        h->coeff64.allocate( std::max<int64_t>( 1, h->nnz ), s );
        a.coeff64 = h->coeff64.get();
    }
    else
    {
        h->coeff32.allocate( std::max<int64_t>( 1, h->nnz ), s );
        a.coeff32 = h->coeff32.get();
    }
    if ( g.radius_mode )
        // radius rows are uneven (0 to thousands of entries): the persistent
        // setup with 8 or 32 lanes a target for the gathers, by row length
        run_setup_plan( a, g.opts.precision, nullptr, nullptr, nullptr, true, s );
    else if ( g.opts.precision == DTK_FP64 )
        setup_fp64( a, s );
    else
        setup_mixed( a, s );
    DTK_CUDA_OR_THROW( cudaEventRecord( ev[2], s ) );

    unsigned st = 0;
    unsigned long long cnt[3] = {0, 0, 0};
    DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( unsigned ),
                                        cudaMemcpyDeviceToHost, s ) );
    DTK_CUDA_OR_THROW( cudaMemcpyAsync( cnt, counters.get(), sizeof( cnt ),
                                        cudaMemcpyDeviceToHost, s ) );
    // The apply's position -> index map stays; the rest of the tree and the
    // scratch are released before returning (stream ordered).
    if ( h->pos.get() )
        h->perm = std::move( tree.perm );
    tree = Lbvh();
    DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
    if ( st & DEV_TIMEOUT )
        throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (Jacobi rotations or tree traversal) hit its cap"};
    if ( st )
        throw Error{DTK_ERR_INTERNAL, "search traversal reported an internal error"};
    h->underdetermined = (int64_t)cnt[0];
    h->rotations = (int64_t)cnt[1];
    h->rotations32 = (int64_t)cnt[2];
    DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->search_ms, ev[0], ev[1] ) );
    DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->setup_ms, ev[1], ev[2] ) );
    DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->build_ms, ev[0], ev[3] ) );
    DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->query_ms, ev[3], ev[1] ) );
    return guard;
}
} // namespace dtk

extern "C" {

void dtk_mls_default_options( dtk_mls_options *o )
{
    if ( !o )
        return;
    o->rbf = DTK_WENDLAND0;
    o->basis = DTK_LINEAR3;
    o->k = 0;
    o->precision = DTK_FP64;
    o->radius = 0.0;
    o->comm_size = 1;
    o->keep_points = 0;
}

dtk_status dtk_set_loop_caps( int64_t jacobi_rotations, int64_t traversal_steps )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( jacobi_rotations >= 0 && traversal_steps >= 0, "caps must be >= 0" );
        DTK_REQUIRE_OR_THROW( jacobi_rotations <= UINT32_MAX, "Jacobi cap exceeds 2^32 - 1" );
        g_jacobi_cap.store( jacobi_rotations, std::memory_order_relaxed );
        g_traversal_cap.store( traversal_steps, std::memory_order_relaxed );
    } );
}

dtk_status dtk_set_rotation_log( int32_t rotations )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( rotations >= 0 && rotations <= JACOBI_LOG, "rotations must be in [0, 160]" );
        g_jacobi_log.store( rotations, std::memory_order_relaxed );
    } );
}

dtk_status dtk_set_setup_lanes( int32_t lanes_short, int32_t lanes_long )
{
    return guarded( [&] {
        auto ok = []( int v ) { return v == 0 || ( v >= 1 && v <= 32 && ( v & ( v - 1 ) ) == 0 ); };
        DTK_REQUIRE_OR_THROW( ok( lanes_short ) && ok( lanes_long ),
                              "lanes must be 0 (tuned) or a power of two in [1, 32]" );
        g_setup_lanes1.store( lanes_short, std::memory_order_relaxed );
        g_setup_lanes2.store( lanes_long, std::memory_order_relaxed );
    } );
}

const char *dtk_last_error( void ) { return g_error.c_str(); }

const char *dtk_status_string( dtk_status s )
{
    switch ( s )
    {
    case DTK_OK: return "DTK_OK";
    case DTK_ERR_INVALID_ARG: return "DTK_ERR_INVALID_ARG";
    case DTK_ERR_UNSUPPORTED: return "DTK_ERR_UNSUPPORTED";
    case DTK_ERR_CUDA: return "DTK_ERR_CUDA";
    case DTK_ERR_OOM: return "DTK_ERR_OOM";
    case DTK_ERR_TIMEOUT: return "DTK_ERR_TIMEOUT";
    case DTK_ERR_INTERNAL: return "DTK_ERR_INTERNAL";
    }
    return "unknown dtk_status";
}

dtk_status dtk_mls_create( const dtk_mls_options *opts, const double *src, int64_t n_src,
                           int64_t src_pt_stride, int64_t src_dim_stride, const double *tgt,
                           int64_t n_tgt, int64_t tgt_pt_stride, int64_t tgt_dim_stride,
                           dtk_stream_t stream_, dtk_mls_handle *out )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr, "output handle pointer is null" );
        *out = nullptr;
        Geometry const g = check_options( opts );
        validate_points( src, n_src, src_pt_stride, src_dim_stride, "source points" );
        validate_points( tgt, n_tgt, tgt_pt_stride, tgt_dim_stride, "target points" );
        // DTK_CHECK( !search_tree.empty() ), DTK_MovingLeastSquaresOperator_def.hpp:49
        DTK_REQUIRE_OR_THROW( n_src > 0, "the source point cloud is empty" );
        require_device_memory( src, "source points" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        PointsView const sv{src, n_src, src_pt_stride, src_dim_stride};
        PointsView const tv{tgt, n_tgt, tgt_pt_stride, tgt_dim_stride};
        *out = create_impl( g, opts, sv, tv, s, nullptr ).release();
    } );
}

dtk_status dtk_mls_create_from_neighbors( const dtk_mls_options *opts, const double *tgt, int64_t n_tgt,
                                          int64_t tgt_pt_stride, int64_t tgt_dim_stride, int32_t row,
                                          const double *nb_points, const int32_t *indices, int64_t n_src,
                                          dtk_stream_t stream_, dtk_mls_handle *out )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr, "output handle pointer is null" );
        *out = nullptr;
        Geometry const g = check_options( opts );
        if ( g.radius_mode )
            throw Error{DTK_ERR_UNSUPPORTED, "neighbour rows are kNN rows (radius must be 0)"};
        if ( g.opts.keep_points )
            throw Error{DTK_ERR_UNSUPPORTED, "a handle from neighbour rows keeps no points"};
        validate_points( tgt, n_tgt, tgt_pt_stride, tgt_dim_stride, "target points" );
        DTK_REQUIRE_OR_THROW( row >= 1 && row <= FUSED_MAX_ROW, "row length must be in [1, 32]" );
        int64_t const nnz = n_tgt * (int64_t)row;
        DTK_REQUIRE_OR_THROW( n_src >= ( nnz ? 1 : 0 ) && n_src <= INT32_MAX,
                              "n_src must be in [1, 2^31) (0 only without targets)" );
        DTK_REQUIRE_OR_THROW( nnz <= INT32_MAX, "n_targets * row exceeds int32 CSR offsets" );
        DTK_REQUIRE_OR_THROW( nnz == 0 || ( nb_points && indices ), "null neighbour arrays" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        require_device_memory( nnz ? nb_points : nullptr, "neighbour points" );
        require_device_memory( nnz ? indices : nullptr, "indices" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        auto h = std::make_unique<dtk_mls_s>( s );
        TouchOnExit const touch{&h->life, s};
        h->opts = *opts;
        h->n_src = n_src;
        h->n_tgt = n_tgt;
        h->m = g.m;
        h->nnz = nnz;
        h->uniform_row = row;
        h->mean_row = row;
        h->offset.allocate( n_tgt + 1, s );
        k_fill_uniform_offsets<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( h->offset.get(), n_tgt, row );
        check_launch( "k_fill_uniform_offsets" );
        h->idx.allocate( std::max<int64_t>( 1, nnz ), s );
        DeviceBuffer<unsigned> status( 1, s );
        DeviceBuffer<unsigned long long> counters( 3, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( counters.get(), 0, 3 * sizeof( unsigned long long ), s ) );
        if ( nnz )
        {
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->idx.get(), indices, nnz * sizeof( int32_t ),
                                                cudaMemcpyDeviceToDevice, s ) );
            k_check_indices<<<(unsigned)( ( nnz + 255 ) / 256 ), 256, 0, s>>>( h->idx.get(), nnz, n_src,
                                                                              status.get() );
            check_launch( "k_check_indices" );
        }
        // the setup reads entry e's neighbour at nb_points[e]: an identity
        // index over the entries in place of the search's rows
        DeviceBuffer<int32_t> entry( std::max<int64_t>( 1, nnz ), s );
        k_iota32<<<(unsigned)( ( nnz + 256 ) / 256 ), 256, 0, s>>>( entry.get(), nnz );
        check_launch( "k_iota32" );
        SetupArgs a{};
        a.src = PointsView{nb_points, std::max<int64_t>( 1, nnz ), 3, 1};
        a.tgt = PointsView{tgt, n_tgt, tgt_pt_stride, tgt_dim_stride};
        a.offset = h->offset.get();
        a.idx = entry.get();
        a.order = nullptr;
        a.n_tgt = n_tgt;
        a.rbf = g.opts.rbf;
        a.basis = g.opts.basis;
        a.rows_sorted = false; // the radius is the row's farthest, in any order
        a.underdetermined = counters.get();
        a.rotations = counters.get() + 1;
        a.rotations32 = counters.get() + 2;
        a.status = status.get();
        if ( g.opts.precision == DTK_FP64 )
        {
            h->coeff64.allocate( std::max<int64_t>( 1, nnz ), s );
            a.coeff64 = h->coeff64.get();
            if ( nnz )
                setup_fp64( a, s );
        }
        else
        {
            h->coeff32.allocate( std::max<int64_t>( 1, nnz ), s );
            a.coeff32 = h->coeff32.get();
            if ( nnz )
                setup_mixed( a, s );
        }
        unsigned st = 0;
        unsigned long long cnt[3] = {0, 0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( unsigned ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( cnt, counters.get(), sizeof( cnt ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_BAD_INDEX )
            throw Error{DTK_ERR_INVALID_ARG, "DTK_REQUIRE: indices must lie in [0, n_src)"};
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (Jacobi rotations) hit its cap"};
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "the setup reported an internal error"};
        h->underdetermined = (int64_t)cnt[0];
        h->rotations = (int64_t)cnt[1];
        h->rotations32 = (int64_t)cnt[2];
        *out = h.release();
    } );
}

dtk_status dtk_mls_apply( dtk_mls_handle h, const double *source_values, int64_t n_source_values,
                          double *target_values, int64_t n_target_values, dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_compute_values" );
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        // DTK_REQUIRE at DTK_MovingLeastSquaresOperator_def.hpp:129-130
        DTK_REQUIRE_OR_THROW( n_source_values == h->n_src,
                              "source_values.extent(0) == n_source_points" );
        DTK_REQUIRE_OR_THROW( n_target_values == h->n_tgt,
                              "target_values.extent(0) == n_target_points" );
        DTK_REQUIRE_OR_THROW( h->n_src == 0 || source_values != nullptr, "source_values is null" );
        DTK_REQUIRE_OR_THROW( h->n_tgt == 0 || target_values != nullptr, "target_values is null" );
        require_device_memory( source_values, "source_values" );
        require_device_memory( target_values, "target_values" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        // uniform rows: by sorted position when the search left them; the
        // mixed form always (its double-float sum), by index otherwise
        bool const by_pos = h->pos.get() && h->perm.get();
        if ( apply_sorted_supported( h->uniform_row ) && ( by_pos || h->coeff32.get() ) )
            apply_sorted( h->n_tgt, h->uniform_row, by_pos ? h->pos.get() : h->idx.get(), h->coeff64.get(),
                          h->coeff32.get(), h->n_src, by_pos ? h->perm.get() : nullptr, source_values,
                          target_values, s, by_pos ? h->order.get() : nullptr );
        else
            apply_csr( h->n_tgt, h->offset.get(), h->idx.get(), h->coeff64.get(), h->coeff32.get(),
                       h->uniform_row, h->mean_row, source_values, target_values, s );
    } );
}

dtk_status dtk_mls_transfer_host( const dtk_mls_options *opts, const double *src_host, int64_t n_src,
                                  const double *tgt_host, int64_t n_tgt, const double *values_host,
                                  double *target_values_host, dtk_stream_t stream_, dtk_mls_handle *out )
{
    return guarded( [&] {
        if ( out )
            *out = nullptr;
        Geometry const g = check_options( opts );
        validate_points( src_host, n_src, 3, 1, "source points" );
        validate_points( tgt_host, n_tgt, 3, 1, "target points" );
        DTK_REQUIRE_OR_THROW( n_src > 0, "the source point cloud is empty" );
        DTK_REQUIRE_OR_THROW( values_host != nullptr, "source values are null" );
        DTK_REQUIRE_OR_THROW( n_tgt == 0 || target_values_host != nullptr, "target values are null" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        // the side stream carries the target and value copies in and the
        // result slices out
        struct Side
        {
            cudaStream_t s2 = nullptr;
            std::vector<cudaEvent_t> ev;
            ~Side()
            {
                for ( cudaEvent_t e : ev )
                    cudaEventDestroy( e );
                if ( s2 )
                    cudaStreamDestroy( s2 );
            }
            cudaEvent_t event()
            {
                cudaEvent_t e = nullptr;
                DTK_CUDA_OR_THROW( cudaEventCreateWithFlags( &e, cudaEventDisableTiming ) );
                ev.push_back( e );
                return e;
            }
        } side;
        DTK_CUDA_OR_THROW( cudaStreamCreateWithFlags( &side.s2, cudaStreamNonBlocking ) );
        DeviceBuffer<double> d_src( 3 * n_src, s ), d_tgt( std::max<int64_t>( 1, 3 * n_tgt ), s ),
            d_vals( n_src, s ), d_out( std::max<int64_t>( 1, n_tgt ), s );
        cudaEvent_t const src_in = side.event(), tgt_ready = side.event(), vals_ready = side.event();
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_src.get(), src_host, 3 * n_src * sizeof( double ),
                                            cudaMemcpyHostToDevice, s ) );
        // the targets and values follow the sources over the host link (the
        // tree build needs only the sources; the later copies overlap it)
        DTK_CUDA_OR_THROW( cudaEventRecord( src_in, s ) );
        DTK_CUDA_OR_THROW( cudaStreamWaitEvent( side.s2, src_in, 0 ) );
        if ( n_tgt )
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_tgt.get(), tgt_host, 3 * n_tgt * sizeof( double ),
                                                cudaMemcpyHostToDevice, side.s2 ) );
        DTK_CUDA_OR_THROW( cudaEventRecord( tgt_ready, side.s2 ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_vals.get(), values_host, n_src * sizeof( double ),
                                            cudaMemcpyHostToDevice, side.s2 ) );
        DTK_CUDA_OR_THROW( cudaEventRecord( vals_ready, side.s2 ) );
        PointsView const sv{d_src.get(), n_src, 3, 1};
        PointsView const tv{d_tgt.get(), n_tgt, 3, 1};
        std::unique_ptr<dtk_mls_s> h = create_impl( g, opts, sv, tv, s, tgt_ready );
        TouchOnExit const touch{&h->life, s};
        DTK_CUDA_OR_THROW( cudaStreamWaitEvent( s, vals_ready, 0 ) );
        // the apply in row slices; each slice's results go back while the
        // next one computes
        int64_t const slices = n_tgt >= ( int64_t( 1 ) << 20 ) ? 8 : 1;
        int64_t const per = ( n_tgt + slices - 1 ) / std::max<int64_t>( 1, slices );
        int const R = h->uniform_row;
        bool const by_pos = h->pos.get() && h->perm.get();
        SortedValues sorted;
        if ( by_pos )
            sorted = permute_values( n_src, h->perm.get(), d_vals.get(), h->coeff32.get() != nullptr, s );
        for ( int64_t r0 = 0; r0 < n_tgt; r0 += per )
        {
            int64_t const r1 = std::min( n_tgt, r0 + per );
            if ( by_pos )
                apply_pos( r1 - r0, R, h->pos.get() + r0 * R, h->coeff64.get() ? h->coeff64.get() + r0 * R : nullptr,
                           h->coeff32.get() ? h->coeff32.get() + r0 * R : nullptr, sorted, d_out.get() + r0, s );
            else if ( R > 0 ) // uniform rows: offset[i] = i R also indexes the shifted slice
                apply_csr( r1 - r0, h->offset.get(), h->idx.get() + r0 * R,
                           h->coeff64.get() ? h->coeff64.get() + r0 * R : nullptr,
                           h->coeff32.get() ? h->coeff32.get() + r0 * R : nullptr, R, h->mean_row,
                           d_vals.get(), d_out.get() + r0, s );
            else // absolute offsets into the whole arrays
                apply_csr( r1 - r0, h->offset.get() + r0, h->idx.get(), h->coeff64.get(), h->coeff32.get(), 0,
                           h->mean_row, d_vals.get(), d_out.get() + r0, s );
            cudaEvent_t const done = side.event();
            DTK_CUDA_OR_THROW( cudaEventRecord( done, s ) );
            DTK_CUDA_OR_THROW( cudaStreamWaitEvent( side.s2, done, 0 ) );
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( target_values_host + r0, d_out.get() + r0,
                                                ( r1 - r0 ) * sizeof( double ), cudaMemcpyDeviceToHost,
                                                side.s2 ) );
        }
        // the buffers are freed on s: after the last copy out
        cudaEvent_t const copied = side.event();
        DTK_CUDA_OR_THROW( cudaEventRecord( copied, side.s2 ) );
        DTK_CUDA_OR_THROW( cudaStreamWaitEvent( s, copied, 0 ) );
        d_src = DeviceBuffer<double>();
        d_tgt = DeviceBuffer<double>();
        d_vals = DeviceBuffer<double>();
        d_out = DeviceBuffer<double>();
        sorted = SortedValues();
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( out )
            *out = h.release();
    } );
}

dtk_status dtk_mls_get_csr( dtk_mls_handle h, const int32_t **offset, const int32_t **indices,
                            const void **coeff, int64_t *nnz, int32_t *coeff_is_fp32 )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( offset )
            *offset = h->offset.get();
        if ( indices )
            *indices = h->idx.get();
        bool const f32 = h->coeff32.get() != nullptr;
        if ( coeff )
            *coeff = f32 ? (const void *)h->coeff32.get() : (const void *)h->coeff64.get();
        if ( nnz )
            *nnz = h->nnz;
        if ( coeff_is_fp32 )
            *coeff_is_fp32 = f32 ? 1 : 0;
    } );
}

dtk_status dtk_mls_get_sizes( dtk_mls_handle h, int64_t *n_src, int64_t *n_tgt, int64_t *nnz )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( n_src )
            *n_src = h->n_src;
        if ( n_tgt )
            *n_tgt = h->n_tgt;
        if ( nnz )
            *nnz = h->nnz;
    } );
}

dtk_status dtk_mls_underdetermined_count( dtk_mls_handle h, int64_t *count )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr && count != nullptr, "null argument" );
        *count = h->underdetermined;
    } );
}

dtk_status dtk_mls_get_stage_times( dtk_mls_handle h, float *search_ms, float *setup_ms )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( search_ms )
            *search_ms = h->search_ms;
        if ( setup_ms )
            *setup_ms = h->setup_ms;
    } );
}

dtk_status dtk_mls_get_search_times( dtk_mls_handle h, float *build_ms, float *query_ms )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( build_ms )
            *build_ms = h->build_ms;
        if ( query_ms )
            *query_ms = h->query_ms;
    } );
}

dtk_status dtk_mls_get_rotation_count( dtk_mls_handle h, int64_t *rotations,
                                       int64_t *rotations_fp32 )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( rotations )
            *rotations = h->rotations;
        if ( rotations_fp32 )
            *rotations_fp32 = h->rotations32;
    } );
}

int64_t dtk_kernel_launch_count( void ) { return launch_counter(); }

dtk_status dtk_stream_synchronize( dtk_stream_t stream )
{
    return guarded( [&] { DTK_CUDA_OR_THROW( cudaStreamSynchronize( reinterpret_cast<cudaStream_t>( stream ) ) ); } );
}

dtk_status dtk_release_cached_memory( void )
{
    return guarded( [&] {
        std::lock_guard<std::mutex> lock( g_pool_mutex );
        for ( cudaMemPool_t pool : g_pools )
            if ( pool )
                DTK_CUDA_OR_THROW( cudaMemPoolTrimTo( pool, 0 ) );
    } );
}

dtk_status dtk_mls_destroy( dtk_mls_handle h )
{
    return guarded( [&] { delete h; } );
}

dtk_status dtk_knn_search( const double *src, int64_t n_src, int64_t src_pt_stride,
                           int64_t src_dim_stride, const double *tgt, int64_t n_tgt,
                           int64_t tgt_pt_stride, int64_t tgt_dim_stride, int32_t k,
                           int32_t *offset, int32_t *indices, dtk_stream_t stream_ )
{
    return guarded( [&] {
        validate_points( src, n_src, src_pt_stride, src_dim_stride, "source points" );
        validate_points( tgt, n_tgt, tgt_pt_stride, tgt_dim_stride, "target points" );
        DTK_REQUIRE_OR_THROW( n_src > 0, "the source point cloud is empty" );
        DTK_REQUIRE_OR_THROW( k >= 0, "k is negative" );
        if ( k > 32 )
            throw Error{DTK_ERR_UNSUPPORTED, "kNN search supports k <= 32"};
        DTK_REQUIRE_OR_THROW( offset != nullptr, "offset is null" );
        int const row = (int)std::min<int64_t>( k, n_src );
        DTK_REQUIRE_OR_THROW( n_tgt * (int64_t)row <= INT32_MAX, "n_targets * k exceeds int32" );
        DTK_REQUIRE_OR_THROW( n_tgt * (int64_t)row == 0 || indices != nullptr, "indices is null" );
        require_device_memory( src, "source points" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        require_device_memory( offset, "offset" );
        require_device_memory( n_tgt * (int64_t)row != 0 ? indices : nullptr, "indices" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        PointsView const sv{src, n_src, src_pt_stride, src_dim_stride};
        PointsView const tv{tgt, n_tgt, tgt_pt_stride, tgt_dim_stride};
        DeviceBuffer<unsigned> status( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        k_fill_uniform_offsets<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( offset, n_tgt, row );
        check_launch( "k_fill_uniform_offsets" );
        Lbvh tree;
        DeviceBuffer<uint32_t> order;
        build_tree_and_order( sv, tv, tree, order, status.get(), s );
        knn_query( tree, tv, order.get(), k, GroupArgs{}, offset, indices, status.get(), s );
        unsigned st = 0;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( unsigned ),
                                            cudaMemcpyDeviceToHost, s ) );
        tree = Lbvh();
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (tree traversal) hit its cap"};
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "search traversal reported an internal error"};
    } );
}

dtk_status dtk_svd_pinv( int32_t n, int64_t count, const double *a, double *pinv,
                         int64_t *underdetermined, dtk_stream_t stream_ )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( n >= 1 && n <= 64, "matrix size must be in [1, 64]" );
        DTK_REQUIRE_OR_THROW( count >= 0, "count is negative" );
        DTK_REQUIRE_OR_THROW( count == 0 || ( a && pinv ), "null matrix pointer" );
        if ( count )
        {
            require_device_memory( a, "a" );
            require_device_memory( pinv, "pinv" );
        }
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        DeviceBuffer<unsigned> status( 1, s );
        DeviceBuffer<unsigned long long> under( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( under.get(), 0, sizeof( unsigned long long ), s ) );
        svd_pinv_batched( n, count, a, pinv, under.get(), status.get(), s );
        unsigned st = 0;
        unsigned long long u = 0;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &u, under.get(), sizeof( u ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (Jacobi rotations or tree traversal) hit its cap"};
        if ( underdetermined )
            *underdetermined = (int64_t)u;
    } );
}

} // extern "C"
