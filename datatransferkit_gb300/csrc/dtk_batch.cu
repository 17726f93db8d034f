// Batched uneven MLS transfers (extension; the reference builds one operator
// per problem) and the setup planner shared with the single operator.
//
// All problems share one LBVH over their packed sources, built in
// problem-major Morton order: problem p's sources occupy one contiguous range
// of sorted positions, every tree node records the leaf range it covers, and
// a query only enters nodes and points of its own problem.  Targets are
// processed in problem-major Morton order.  The setup buckets targets by
// (basis, rbf, row length): rows up to LONG_ROW run the fused one-thread-per-
// target kernel of the requested precision, longer radius rows the
// warp-cooperative FP64 path.  Apply runs one launch per row-length bin
// (rows of up to 2^b entries), each with the lanes-per-row an autotuner
// picked on the first call by timing the candidates on the actual data; the
// bin launches are captured once into a CUDA graph and replayed.
#include "dtk_common.cuh"

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <tuple>
#include <vector>

namespace dtk
{

void run_setup_plan( SetupArgs const &a, int precision, int32_t const *order_host,
                     int32_t const *offsets_host, uint8_t const *basis_of, uint8_t const *rbf_of,
                     cudaStream_t s )
{
    std::map<std::tuple<int, int, int>, std::vector<int32_t>> buckets;
    for ( int64_t g = 0; g < a.n_tgt; ++g )
    {
        int32_t const i = order_host[g];
        int const len = offsets_host[i + 1] - offsets_host[i];
        int const b = basis_of ? basis_of[i] : a.basis;
        int const r = rbf_of ? rbf_of[i] : a.rbf;
        buckets[std::make_tuple( b, r, len > LONG_ROW ? 1 : 0 )].push_back( i );
    }
    for ( auto const &kv : buckets )
    {
        std::vector<int32_t> const &list = kv.second;
        int64_t const n = (int64_t)list.size();
        DeviceBuffer<int32_t> d( n, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d.get(), list.data(), n * sizeof( int32_t ),
                                            cudaMemcpyHostToDevice, s ) );
        SetupArgs b = a;
        b.basis = std::get<0>( kv.first );
        b.rbf = std::get<1>( kv.first );
        b.n_tgt = n;
        b.order = reinterpret_cast<uint32_t const *>( d.get() );
        if ( std::get<2>( kv.first ) )
            setup_long_rows( b, d.get(), n, s );
        else if ( precision == DTK_FP64 )
            setup_fp64( b, s );
        else
            setup_mixed( b, s );
        // the stream-ordered free of `d` follows the launches
    }
}

namespace
{

__global__ void k_group_ids( int64_t const *off, int n_groups, int64_t n, uint32_t *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    int lo = 0, hi = n_groups; // largest g with off[g] <= i
    while ( hi - lo > 1 )
    {
        int const mid = ( lo + hi ) / 2;
        if ( off[mid] <= i )
            lo = mid;
        else
            hi = mid;
    }
    out[i] = (uint32_t)lo;
}

__global__ void k_narrow32( int64_t const *in, int32_t *out, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        out[i] = (int32_t)in[i];
}

constexpr unsigned FULL = 0xffffffffu;

// S lanes per row over a list of rows.
template <int S, bool F32>
__global__ void __launch_bounds__( 256 )
    k_apply_rows( int64_t n_rows, int32_t const *__restrict__ rows, int32_t const *__restrict__ offset,
                  int32_t const *__restrict__ idx, void const *__restrict__ coeff,
                  double const *__restrict__ values, double *__restrict__ target )
{
    int64_t const gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const r = gt / S;
    int const sub = (int)( gt % S );
    double acc = 0.0;
    int64_t row = 0;
    if ( r < n_rows )
    {
        row = rows[r];
        int const b = offset[row], e = offset[row + 1];
        for ( int j = b + sub; j < e; j += S )
        {
            double const c = F32 ? (double)static_cast<float const *>( coeff )[j]
                                 : static_cast<double const *>( coeff )[j];
            acc = fma( c, __ldg( values + idx[j] ), acc );
        }
    }
#pragma unroll
    for ( int o = S / 2; o > 0; o >>= 1 )
        acc += __shfl_xor_sync( FULL, acc, o );
    if ( r < n_rows && sub == 0 )
        target[row] = acc;
}

template <bool F32>
void launch_rows( int lanes, int64_t n_rows, int32_t const *rows, int32_t const *offset,
                  int32_t const *idx, void const *coeff, double const *values, double *target,
                  cudaStream_t s )
{
    unsigned const blocks = (unsigned)std::max<int64_t>( 1, ( n_rows * lanes + 255 ) / 256 );
    switch ( lanes )
    {
    case 1: k_apply_rows<1, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    case 2: k_apply_rows<2, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    case 4: k_apply_rows<4, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    case 8: k_apply_rows<8, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    case 16: k_apply_rows<16, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    default: k_apply_rows<32, F32><<<blocks, 256, 0, s>>>( n_rows, rows, offset, idx, coeff, values, target ); break;
    }
    check_launch( "k_apply_rows" );
}

} // namespace
} // namespace dtk

using namespace dtk;

struct dtk_mls_batch_s
{
    int32_t n_problems = 0;
    int precision = DTK_FP64;
    int64_t n_src = 0, n_tgt = 0, nnz = 0;
    DeviceBuffer<int32_t> offset, idx;
    DeviceBuffer<double> coeff64;
    DeviceBuffer<float> coeff32;
    struct Bin
    {
        int max_len;
        int lanes;
        int64_t n;
        DeviceBuffer<int32_t> rows;
    };
    std::vector<Bin> bins;
    bool tuned = false;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double const *g_src = nullptr;
    double *g_tgt = nullptr;
    int64_t underdetermined = 0, rotations = 0;
    ~dtk_mls_batch_s()
    {
        if ( exec )
            cudaGraphExecDestroy( exec );
        if ( graph )
            cudaGraphDestroy( graph );
        if ( capture )
            cudaStreamDestroy( capture );
    }
    void launch_bins( double const *src_values, double *tgt_values, cudaStream_t s )
    {
        bool const f32 = coeff32.get() != nullptr;
        void const *coeff = f32 ? (void const *)coeff32.get() : (void const *)coeff64.get();
        for ( auto const &b : bins )
        {
            if ( !b.n )
                continue;
            if ( f32 )
                launch_rows<true>( b.lanes, b.n, b.rows.get(), offset.get(), idx.get(), coeff,
                                   src_values, tgt_values, s );
            else
                launch_rows<false>( b.lanes, b.n, b.rows.get(), offset.get(), idx.get(), coeff,
                                    src_values, tgt_values, s );
        }
    }
};

namespace
{

template <class F>
dtk_status guarded_batch( F &&f )
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

int pow2_ceil( int v )
{
    int p = 1;
    while ( p < v )
        p <<= 1;
    return p;
}

} // namespace

extern "C" {

dtk_status dtk_mls_batch_create( int32_t n_problems, const dtk_mls_options *opts,
                                 const int64_t *src_offsets, const double *src,
                                 const int64_t *tgt_offsets, const double *tgt,
                                 dtk_stream_t stream_, dtk_mls_batch_handle *out )
{
    return guarded_batch( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr, "output handle pointer is null" );
        *out = nullptr;
        DTK_REQUIRE_OR_THROW( n_problems >= 1, "n_problems must be >= 1" );
        DTK_REQUIRE_OR_THROW( opts && src_offsets && tgt_offsets, "null host array" );
        DTK_REQUIRE_OR_THROW( src_offsets[0] == 0 && tgt_offsets[0] == 0, "offsets must start at 0" );
        bool const radius_mode = opts[0].radius > 0.0;
        int const precision = opts[0].precision;
        std::vector<int32_t> kq( n_problems );
        std::vector<double> rq( n_problems );
        for ( int p = 0; p < n_problems; ++p )
        {
            DTK_REQUIRE_OR_THROW( opts[p].comm_size == 1 || opts[p].comm_size == 0 ? true : false,
                                  "problem " + std::to_string( p ) + ": only single-rank operators" );
            dtk_mls_options o = opts[p];
            o.comm_size = 1;
            DTK_REQUIRE_OR_THROW( o.rbf >= DTK_WENDLAND0 && o.rbf <= DTK_BUHMANN4, "unknown rbf" );
            DTK_REQUIRE_OR_THROW( o.basis >= DTK_CONSTANT3 && o.basis <= DTK_QUADRATIC3, "unknown basis" );
            DTK_REQUIRE_OR_THROW( o.precision == precision, "all problems of a batch share one precision form" );
            DTK_REQUIRE_OR_THROW( ( o.radius > 0.0 ) == radius_mode,
                                  "all problems of a batch use kNN, or all use a radius search" );
            DTK_REQUIRE_OR_THROW( std::isfinite( o.radius ) && o.radius >= 0.0, "bad radius" );
            DTK_REQUIRE_OR_THROW( o.k >= 0, "k is negative" );
            kq[p] = o.k ? o.k : basis_size( o.basis );
            if ( !radius_mode && kq[p] > 32 )
                throw Error{DTK_ERR_UNSUPPORTED, "kNN search supports k <= 32"};
            rq[p] = o.radius;
            // DTK_CHECK( !search_tree.empty() ) for every problem
            DTK_REQUIRE_OR_THROW( src_offsets[p + 1] > src_offsets[p],
                                  "problem " + std::to_string( p ) + " has no source points" );
            DTK_REQUIRE_OR_THROW( tgt_offsets[p + 1] >= tgt_offsets[p], "target offsets decrease" );
        }
        int64_t const n_src = src_offsets[n_problems], n_tgt = tgt_offsets[n_problems];
        DTK_REQUIRE_OR_THROW( n_src <= INT32_MAX && n_tgt <= INT32_MAX, "too many points" );
        DTK_REQUIRE_OR_THROW( src != nullptr && ( n_tgt == 0 || tgt != nullptr ), "null points" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        auto h = std::make_unique<dtk_mls_batch_s>();
        h->n_problems = n_problems;
        h->precision = precision;
        h->n_src = n_src;
        h->n_tgt = n_tgt;
        PointsView const sv{src, n_src, 3, 1};
        PointsView const tv{tgt, n_tgt, 3, 1};

        DeviceBuffer<unsigned> status( 1, s );
        DeviceBuffer<unsigned long long> counters( 3, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( counters.get(), 0, 3 * sizeof( unsigned long long ), s ) );
        DeviceBuffer<int64_t> d_src_off( n_problems + 1, s ), d_tgt_off( n_problems + 1, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_src_off.get(), src_offsets, ( n_problems + 1 ) * 8,
                                            cudaMemcpyHostToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_tgt_off.get(), tgt_offsets, ( n_problems + 1 ) * 8,
                                            cudaMemcpyHostToDevice, s ) );
        DeviceBuffer<uint32_t> src_grp( n_src, s ), tgt_grp( std::max<int64_t>( 1, n_tgt ), s );
        k_group_ids<<<(unsigned)( ( n_src + 255 ) / 256 ), 256, 0, s>>>( d_src_off.get(), n_problems, n_src,
                                                                         src_grp.get() );
        check_launch( "k_group_ids(src)" );
        if ( n_tgt )
        {
            k_group_ids<<<(unsigned)( ( n_tgt + 255 ) / 256 ), 256, 0, s>>>( d_tgt_off.get(), n_problems,
                                                                             n_tgt, tgt_grp.get() );
            check_launch( "k_group_ids(tgt)" );
        }
        DeviceBuffer<int32_t> d_k( n_problems, s );
        DeviceBuffer<double> d_r( n_problems, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_k.get(), kq.data(), n_problems * 4, cudaMemcpyHostToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_r.get(), rq.data(), n_problems * 8, cudaMemcpyHostToDevice, s ) );

        // --- search over all problems at once ---
        Lbvh tree;
        build_lbvh( sv, tree, status.get(), s, src_grp.get(), n_problems );
        DeviceBuffer<uint32_t> order;
        sort_queries( tree, tv, order, s, tgt_grp.get(), n_problems );
        GroupArgs ga;
        ga.src_off = d_src_off.get();
        ga.tgt_grp = tgt_grp.get();
        ga.k = d_k.get();
        ga.r = d_r.get();
        h->offset.allocate( n_tgt + 1, s );
        std::vector<int32_t> off_h( n_tgt + 1, 0 );
        if ( !radius_mode )
        {
            int64_t acc = 0;
            for ( int p = 0; p < n_problems; ++p )
            {
                int64_t const row = std::min<int64_t>( kq[p], src_offsets[p + 1] - src_offsets[p] );
                for ( int64_t i = tgt_offsets[p]; i < tgt_offsets[p + 1]; ++i )
                {
                    off_h[i] = (int32_t)acc;
                    acc += row;
                    DTK_REQUIRE_OR_THROW( acc <= INT32_MAX, "neighbour count exceeds int32 offsets" );
                }
            }
            off_h[n_tgt] = (int32_t)acc;
            h->nnz = acc;
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->offset.get(), off_h.data(), ( n_tgt + 1 ) * 4,
                                                cudaMemcpyHostToDevice, s ) );
            h->idx.allocate( std::max<int64_t>( 1, acc ), s );
            knn_query( tree, tv, order.get(), 0, ga, h->offset.get(), h->idx.get(), status.get(), s );
        }
        else
        {
            DeviceBuffer<int64_t> counts( std::max<int64_t>( 1, n_tgt ), s ), offs( n_tgt + 1, s );
            radius_count( tree, tv, order.get(), 0.0, ga, counts.get(), status.get(), s );
            exclusive_scan_i64( counts.get(), offs.get(), n_tgt, s );
            int64_t total = 0;
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( &total, offs.get() + n_tgt, 8, cudaMemcpyDeviceToHost, s ) );
            DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
            DTK_REQUIRE_OR_THROW( total <= INT32_MAX, "neighbour count exceeds int32 offsets" );
            h->nnz = total;
            k_narrow32<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( offs.get(), h->offset.get(), n_tgt );
            check_launch( "k_narrow32" );
            h->idx.allocate( std::max<int64_t>( 1, total ), s );
            radius_fill( tree, tv, order.get(), 0.0, ga, h->offset.get(), h->idx.get(), status.get(), s );
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( off_h.data(), h->offset.get(), ( n_tgt + 1 ) * 4,
                                                cudaMemcpyDeviceToHost, s ) );
        }
        std::vector<int32_t> order_h( std::max<int64_t>( 1, n_tgt ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( order_h.data(), order.get(), n_tgt * 4, cudaMemcpyDeviceToHost, s ) );
        tree = Lbvh();
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );

        // --- setup, bucketed by (basis, rbf, row length) ---
        std::vector<uint8_t> basis_of( std::max<int64_t>( 1, n_tgt ) ), rbf_of( std::max<int64_t>( 1, n_tgt ) );
        for ( int p = 0; p < n_problems; ++p )
            for ( int64_t i = tgt_offsets[p]; i < tgt_offsets[p + 1]; ++i )
            {
                basis_of[i] = (uint8_t)opts[p].basis;
                rbf_of[i] = (uint8_t)opts[p].rbf;
            }
        SetupArgs a{};
        a.src = sv;
        a.tgt = tv;
        a.offset = h->offset.get();
        a.idx = h->idx.get();
        a.n_tgt = n_tgt;
        a.rows_sorted = !radius_mode;
        a.underdetermined = counters.get();
        a.rotations = counters.get() + 1;
        a.rotations32 = counters.get() + 2;
        a.status = status.get();
        if ( precision == DTK_FP64 )
        {
            h->coeff64.allocate( std::max<int64_t>( 1, h->nnz ), s );
            a.coeff64 = h->coeff64.get();
        }
        else
        {
            h->coeff32.allocate( std::max<int64_t>( 1, h->nnz ), s );
            a.coeff32 = h->coeff32.get();
        }
        run_setup_plan( a, precision, order_h.data(), off_h.data(), basis_of.data(), rbf_of.data(), s );

        // --- apply schedule: rows binned by length (power-of-two bounds) ---
        std::map<int, std::vector<int32_t>> bins;
        for ( int64_t i = 0; i < n_tgt; ++i )
            bins[pow2_ceil( std::max( 1, off_h[i + 1] - off_h[i] ) )].push_back( (int32_t)i );
        for ( auto const &kv : bins )
        {
            dtk_mls_batch_s::Bin b;
            b.max_len = kv.first;
            b.lanes = std::min( 32, std::max( 1, pow2_ceil( kv.first / 4 ) ) );
            b.n = (int64_t)kv.second.size();
            b.rows.allocate( b.n, s );
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( b.rows.get(), kv.second.data(), b.n * 4,
                                                cudaMemcpyHostToDevice, s ) );
            h->bins.push_back( std::move( b ) );
        }
        unsigned st = 0;
        unsigned long long cnt[3] = {0, 0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( cnt, counters.get(), sizeof( cnt ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop hit its cap"};
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "search or setup reported an internal error"};
        h->underdetermined = (int64_t)cnt[0];
        h->rotations = (int64_t)cnt[1];
        *out = h.release();
    } );
}

dtk_status dtk_mls_batch_apply( dtk_mls_batch_handle h, const double *src_values, double *tgt_values,
                                int32_t use_graph, dtk_stream_t stream_ )
{
    return guarded_batch( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        DTK_REQUIRE_OR_THROW( src_values != nullptr && ( h->n_tgt == 0 || tgt_values != nullptr ),
                              "null values" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        if ( !h->tuned )
        {
            // autotune the lanes per row of every bin on the actual data
            cudaEvent_t e0, e1;
            DTK_CUDA_OR_THROW( cudaEventCreate( &e0 ) );
            DTK_CUDA_OR_THROW( cudaEventCreate( &e1 ) );
            bool const f32 = h->coeff32.get() != nullptr;
            void const *coeff = f32 ? (void const *)h->coeff32.get() : (void const *)h->coeff64.get();
            for ( auto &b : h->bins )
            {
                if ( !b.n )
                    continue;
                float best = 1e30f;
                int best_lanes = b.lanes;
                for ( int lanes = 1; lanes <= 32; lanes <<= 1 )
                {
                    if ( lanes > 2 * b.max_len && lanes > 1 )
                        break;
                    float t = 0.f;
                    for ( int rep = 0; rep < 3; ++rep )
                    {
                        DTK_CUDA_OR_THROW( cudaEventRecord( e0, s ) );
                        if ( f32 )
                            launch_rows<true>( lanes, b.n, b.rows.get(), h->offset.get(), h->idx.get(), coeff,
                                               src_values, tgt_values, s );
                        else
                            launch_rows<false>( lanes, b.n, b.rows.get(), h->offset.get(), h->idx.get(), coeff,
                                                src_values, tgt_values, s );
                        DTK_CUDA_OR_THROW( cudaEventRecord( e1, s ) );
                        DTK_CUDA_OR_THROW( cudaEventSynchronize( e1 ) );
                        float ms = 0.f;
                        DTK_CUDA_OR_THROW( cudaEventElapsedTime( &ms, e0, e1 ) );
                        if ( rep > 0 )
                            t += ms;
                    }
                    if ( t < best )
                    {
                        best = t;
                        best_lanes = lanes;
                    }
                }
                b.lanes = best_lanes;
            }
            cudaEventDestroy( e0 );
            cudaEventDestroy( e1 );
            h->tuned = true;
        }
        if ( !use_graph )
        {
            h->launch_bins( src_values, tgt_values, s );
            return;
        }
        if ( !h->exec || h->g_src != src_values || h->g_tgt != tgt_values )
        {
            if ( h->exec )
            {
                cudaGraphExecDestroy( h->exec );
                h->exec = nullptr;
            }
            if ( h->graph )
            {
                cudaGraphDestroy( h->graph );
                h->graph = nullptr;
            }
            if ( !h->capture )
                DTK_CUDA_OR_THROW( cudaStreamCreateWithFlags( &h->capture, cudaStreamNonBlocking ) );
            DTK_CUDA_OR_THROW( cudaStreamBeginCapture( h->capture, cudaStreamCaptureModeThreadLocal ) );
            h->launch_bins( src_values, tgt_values, h->capture );
            DTK_CUDA_OR_THROW( cudaStreamEndCapture( h->capture, &h->graph ) );
            DTK_CUDA_OR_THROW( cudaGraphInstantiate( &h->exec, h->graph, 0 ) );
            h->g_src = src_values;
            h->g_tgt = tgt_values;
        }
        DTK_CUDA_OR_THROW( cudaGraphLaunch( h->exec, s ) );
    } );
}

dtk_status dtk_mls_batch_get_csr( dtk_mls_batch_handle h, const int32_t **offset, const int32_t **indices,
                                  const void **coeff, int64_t *nnz, int32_t *coeff_is_fp32 )
{
    return guarded_batch( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        bool const f32 = h->coeff32.get() != nullptr;
        if ( offset )
            *offset = h->offset.get();
        if ( indices )
            *indices = h->idx.get();
        if ( coeff )
            *coeff = f32 ? (const void *)h->coeff32.get() : (const void *)h->coeff64.get();
        if ( nnz )
            *nnz = h->nnz;
        if ( coeff_is_fp32 )
            *coeff_is_fp32 = f32 ? 1 : 0;
    } );
}

dtk_status dtk_mls_batch_destroy( dtk_mls_batch_handle h )
{
    return guarded_batch( [&] { delete h; } );
}

} // extern "C"
