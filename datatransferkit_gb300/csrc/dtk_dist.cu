// Device steps of the distributed operator's host side (the distributed
// search and value fetch of DTK's MPI operators: ArborX DistributedTree
// query, DTK_MovingLeastSquaresOperator_def.hpp:47-67, and the Distributor
// fetch, DTK_DetailsNearestNeighborOperatorImpl.hpp:47-192).  The exchange
// between ranks is the caller's (MPI, or any transport); these entries do
// the per-rank device work around it: the local kNN rows with their squared
// distances, the source box, contiguous copies of strided points, and the
// gathers of neighbour coordinates and source values.
#include "dtk_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace dtk
{
namespace
{

constexpr int DIST_THREADS = 256;

__global__ void k_row_offsets( int32_t *offset, int64_t n, int row )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        offset[i] = (int32_t)( i * row );
}

inline unsigned dist_blocks( int64_t n )
{
    return (unsigned)std::max<int64_t>( 1, ( n + DIST_THREADS - 1 ) / DIST_THREADS );
}

// d2 of every entry of uniform rows (row entries a target), with the
// search's formula
__global__ void k_rows_d2( PointsView src, PointsView tgt, int32_t const *idx, int64_t n_tgt, int row,
                           double *d2 )
{
    int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( e >= n_tgt * (int64_t)row )
        return;
    int64_t const i = e / row;
    int64_t const j = idx[e];
    d2[e] = dist2_rn( src( j, 0 ), src( j, 1 ), src( j, 2 ), tgt( i, 0 ), tgt( i, 1 ), tgt( i, 2 ) );
}

__global__ void k_pack_points( PointsView p, double *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= p.n )
        return;
    out[3 * i] = p( i, 0 );
    out[3 * i + 1] = p( i, 1 );
    out[3 * i + 2] = p( i, 2 );
}

// entry e's point: source idx[e] when below n_src, else row idx[e] - n_src
// of `extra` (row-major); DEV_BAD_INDEX for an index outside both
__global__ void k_gather_points( PointsView src, double const *extra, int64_t n_extra, int32_t const *idx,
                                 int64_t nnz, double *out, unsigned *status )
{
    int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( e >= nnz )
        return;
    int64_t const j = idx[e];
    double x = 0.0, y = 0.0, z = 0.0;
    if ( j >= 0 && j < src.n )
    {
        x = src( j, 0 );
        y = src( j, 1 );
        z = src( j, 2 );
    }
    else if ( j >= src.n && j < src.n + n_extra )
    {
        double const *p = extra + 3 * ( j - src.n );
        x = p[0];
        y = p[1];
        z = p[2];
    }
    else
        atomicOr( status, DEV_BAD_INDEX );
    out[3 * e] = x;
    out[3 * e + 1] = y;
    out[3 * e + 2] = z;
}

__global__ void k_gather_values( double const *values, int64_t n, int32_t const *idx, int64_t m, double *out,
                                 unsigned *status )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= m )
        return;
    int64_t const j = idx[i];
    if ( j < 0 || j >= n )
    {
        atomicOr( status, DEV_BAD_INDEX );
        out[i] = 0.0;
        return;
    }
    out[i] = values[j];
}

// order-preserving bits of a double (larger values, larger bits)
__device__ __forceinline__ unsigned long long ordered_bits( double v )
{
    long long const b = __double_as_longlong( v );
    return b < 0 ? ~(unsigned long long)b : (unsigned long long)b | ( 1ull << 63 );
}

// the box of a point cloud as ordered bits of (min, -max): a thread's own
// minima, then the warp's, then one atomic a warp and value
__global__ void k_box_bits( PointsView p, unsigned long long *box )
{
    unsigned long long m[6];
#pragma unroll
    for ( int d = 0; d < 6; ++d )
        m[d] = ~0ull;
    for ( int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x )
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            double const v = p( i, d );
            m[d] = min( m[d], ordered_bits( v ) );
            m[3 + d] = min( m[3 + d], ordered_bits( -v ) );
        }
#pragma unroll
    for ( int d = 0; d < 6; ++d )
    {
        for ( int o = 16; o; o >>= 1 )
            m[d] = min( m[d], __shfl_xor_sync( 0xffffffffu, m[d], o ) );
        if ( ( threadIdx.x & 31 ) == 0 && m[d] != ~0ull )
            atomicMin( &box[d], m[d] );
    }
}

double from_ordered( unsigned long long o )
{
    long long const b = ( o >> 63 ) ? (long long)( o & ~( 1ull << 63 ) ) : (long long)~o;
    double v;
    static_assert( sizeof( v ) == sizeof( b ), "64-bit double" );
    std::memcpy( &v, &b, sizeof( v ) );
    return v;
}

void finish_status( DeviceBuffer<unsigned> &status, cudaStream_t s, char const *what )
{
    unsigned st = 0;
    DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
    DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
    if ( st & DEV_BAD_INDEX )
        throw Error{DTK_ERR_INVALID_ARG, std::string( "DTK_REQUIRE: " ) + what};
    if ( st & DEV_TIMEOUT )
        throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (tree traversal) hit its cap"};
    if ( st )
        throw Error{DTK_ERR_INTERNAL, "the search reported an internal error"};
}

} // namespace
} // namespace dtk

using namespace dtk;

extern "C" {

dtk_status dtk_knn_search_d2( const double *src, int64_t n_src, int64_t src_pt_stride, int64_t src_dim_stride,
                              const double *tgt, int64_t n_tgt, int64_t tgt_pt_stride, int64_t tgt_dim_stride,
                              int32_t k, int32_t *indices, double *d2, dtk_stream_t stream_ )
{
    return guarded( [&] {
        validate_points( src, n_src, src_pt_stride, src_dim_stride, "source points" );
        validate_points( tgt, n_tgt, tgt_pt_stride, tgt_dim_stride, "target points" );
        DTK_REQUIRE_OR_THROW( n_src > 0, "the source point cloud is empty" );
        DTK_REQUIRE_OR_THROW( k >= 1, "k must be >= 1" );
        if ( k > 32 )
            throw Error{DTK_ERR_UNSUPPORTED, "kNN search supports k <= 32"};
        int const row = (int)std::min<int64_t>( k, n_src );
        int64_t const nnz = n_tgt * (int64_t)row;
        DTK_REQUIRE_OR_THROW( nnz <= INT32_MAX, "n_targets * k exceeds int32" );
        DTK_REQUIRE_OR_THROW( nnz == 0 || ( indices && d2 ), "null output" );
        require_device_memory( src, "source points" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        require_device_memory( nnz ? indices : nullptr, "indices" );
        require_device_memory( nnz ? d2 : nullptr, "d2" );
        if ( n_tgt == 0 )
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        PointsView const sv{src, n_src, src_pt_stride, src_dim_stride};
        PointsView const tv{tgt, n_tgt, tgt_pt_stride, tgt_dim_stride};
        DeviceBuffer<unsigned> status( 1, s );
        DeviceBuffer<int32_t> offset( n_tgt + 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        k_row_offsets<<<dist_blocks( n_tgt + 1 ), DIST_THREADS, 0, s>>>( offset.get(), n_tgt, row );
        check_launch( "k_row_offsets" );
        {
            Lbvh tree;
            DeviceBuffer<uint32_t> order;
            build_tree_and_order( sv, tv, tree, order, status.get(), s );
            knn_query( tree, tv, order.get(), k, GroupArgs{}, offset.get(), indices, status.get(), s );
        }
        k_rows_d2<<<dist_blocks( nnz ), DIST_THREADS, 0, s>>>( sv, tv, indices, n_tgt, row, d2 );
        check_launch( "k_rows_d2" );
        finish_status( status, s, "indices in range" );
    } );
}

dtk_status dtk_points_bounds( const double *pts, int64_t n, int64_t pt_stride, int64_t dim_stride,
                              double *box_host, dtk_stream_t stream_ )
{
    return guarded( [&] {
        validate_points( pts, n, pt_stride, dim_stride, "points" );
        DTK_REQUIRE_OR_THROW( box_host != nullptr, "box is null" );
        require_device_memory( n ? pts : nullptr, "points" );
        if ( n == 0 )
        {
            double const inf = HUGE_VAL;
            for ( int d = 0; d < 3; ++d )
            {
                box_host[d] = inf;
                box_host[3 + d] = -inf;
            }
            return;
        }
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        DeviceBuffer<unsigned long long> box( 6, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( box.get(), 0xff, 6 * sizeof( unsigned long long ), s ) );
        unsigned const blocks = (unsigned)std::min<int64_t>( 4 * num_sms(), ( n + 255 ) / 256 );
        k_box_bits<<<blocks, 256, 0, s>>>( PointsView{pts, n, pt_stride, dim_stride}, box.get() );
        check_launch( "k_box_bits" );
        unsigned long long h[6];
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( h, box.get(), sizeof( h ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        for ( int d = 0; d < 3; ++d )
        {
            box_host[d] = from_ordered( h[d] );
            box_host[3 + d] = -from_ordered( h[3 + d] );
        }
    } );
}

dtk_status dtk_points_pack( const double *pts, int64_t n, int64_t pt_stride, int64_t dim_stride, double *out,
                            dtk_stream_t stream_ )
{
    return guarded( [&] {
        validate_points( pts, n, pt_stride, dim_stride, "points" );
        DTK_REQUIRE_OR_THROW( n == 0 || out != nullptr, "output is null" );
        require_device_memory( n ? pts : nullptr, "points" );
        require_device_memory( n ? out : nullptr, "output" );
        if ( n == 0 )
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        k_pack_points<<<dist_blocks( n ), DIST_THREADS, 0, s>>>( PointsView{pts, n, pt_stride, dim_stride}, out );
        check_launch( "k_pack_points" );
    } );
}

dtk_status dtk_gather_points( const double *src, int64_t n_src, int64_t src_pt_stride, int64_t src_dim_stride,
                              const double *extra, int64_t n_extra, const int32_t *indices, int64_t nnz,
                              double *out, dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_get_source_values" );
        validate_points( src, n_src, src_pt_stride, src_dim_stride, "source points" );
        DTK_REQUIRE_OR_THROW( n_extra >= 0 && nnz >= 0, "negative count" );
        DTK_REQUIRE_OR_THROW( n_extra == 0 || extra != nullptr, "extra points are null" );
        DTK_REQUIRE_OR_THROW( nnz == 0 || ( indices && out ), "null indices or output" );
        require_device_memory( n_src ? src : nullptr, "source points" );
        require_device_memory( n_extra ? extra : nullptr, "extra points" );
        require_device_memory( nnz ? indices : nullptr, "indices" );
        require_device_memory( nnz ? out : nullptr, "output" );
        if ( nnz == 0 )
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        DeviceBuffer<unsigned> status( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        k_gather_points<<<dist_blocks( nnz ), DIST_THREADS, 0, s>>>(
            PointsView{src, n_src, src_pt_stride, src_dim_stride}, extra, n_extra, indices, nnz, out, status.get() );
        check_launch( "k_gather_points" );
        finish_status( status, s, "indices must lie in [0, n_src + n_extra)" );
    } );
}

dtk_status dtk_gather_values( const double *values, int64_t n, const int32_t *indices, int64_t m, double *out,
                              dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_get_source_values" );
        DTK_REQUIRE_OR_THROW( n >= 0 && m >= 0, "negative count" );
        DTK_REQUIRE_OR_THROW( m == 0 || ( values && indices && out ), "null values, indices or output" );
        require_device_memory( m ? values : nullptr, "values" );
        require_device_memory( m ? indices : nullptr, "indices" );
        require_device_memory( m ? out : nullptr, "output" );
        if ( m == 0 )
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        DeviceBuffer<unsigned> status( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        k_gather_values<<<dist_blocks( m ), DIST_THREADS, 0, s>>>( values, n, indices, m, out, status.get() );
        check_launch( "k_gather_values" );
        finish_status( status, s, "indices must lie in [0, n)" );
    } );
}

} // extern "C"
