// NearestNeighborOperator on one rank, and the rank-2 (multi-component)
// applies of both operators (sm_103a).
//
// The reference operator (packages/Meshfree/src/DTK_NearestNeighborOperator_def.hpp
// :23-81) builds an ArborX tree over the sources, queries the nearest source
// of every target, keeps (index, rank) per target, and its apply fetches
// source_values at those indices (DTK_DetailsNearestNeighborOperatorImpl.hpp
// :152-192, a gather on one rank).  Here the tree is the library's LBVH, the
// query is the kNN kernel with k = 1 under the (d^2, index) contract (the
// nearest source, ties to the smaller index), and apply is one gather kernel.
// Rank-2 fields (n x n_comp, any (point, component) strides: LayoutLeft or
// LayoutRight views) follow the reference's rank-2 fetch
// (DTK_DetailsNearestNeighborOperatorImpl.hpp:53-56,89-93).
#include "dtk_common.cuh"
#include "dtk_handle.cuh"

#include <algorithm>
#include <memory>

struct dtk_nn_s
{
    dtk::HandleLife life;
    int64_t n_src = 0, n_tgt = 0;
    dtk::DeviceBuffer<int32_t> idx; // nearest source of every target
    explicit dtk_nn_s( cudaStream_t home )
        : life( home )
    {
    }
    ~dtk_nn_s() { life.retire( idx ); }
};

namespace dtk
{
namespace
{

__global__ void k_iota_offsets( int32_t *offset, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        offset[i] = (int32_t)i;
}

// out(i, c) = in(idx_i, c); one thread per (target, component)
__global__ void k_gather( int64_t n_tgt, int32_t const *__restrict__ idx, FieldView in, FieldView out )
{
    int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( t >= n_tgt * in.n_comp )
        return;
    int64_t const i = t / in.n_comp;
    int64_t const c = t - i * in.n_comp;
    out.wbase[i * out.ps + c * out.cs] = __ldg( in.base + (int64_t)__ldg( idx + i ) * in.ps + c * in.cs );
}

FieldView field_in( double const *p, int64_t n, int64_t n_comp, int64_t ps, int64_t cs, char const *what )
{
    DTK_REQUIRE_OR_THROW( n_comp >= 1, std::string( what ) + ": n_comp >= 1" );
    DTK_REQUIRE_OR_THROW( n == 0 || p != nullptr, std::string( what ) + " is null" );
    DTK_REQUIRE_OR_THROW( n <= 1 || ps != 0, std::string( what ) + ": zero point stride" );
    DTK_REQUIRE_OR_THROW( n_comp == 1 || cs != 0, std::string( what ) + ": zero component stride" );
    if ( n > 0 )
        require_device_memory( p, what );
    return FieldView{p, nullptr, n, n_comp, ps, cs};
}

} // namespace
} // namespace dtk

using namespace dtk;

extern "C" {

dtk_status dtk_nn_create( const double *src, int64_t n_src, int64_t src_pt_stride, int64_t src_dim_stride,
                          const double *tgt, int64_t n_tgt, int64_t tgt_pt_stride, int64_t tgt_dim_stride,
                          int32_t comm_size, dtk_stream_t stream_, dtk_nn_handle *out )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr, "output handle pointer is null" );
        *out = nullptr;
        if ( comm_size > 1 )
            throw Error{DTK_ERR_UNSUPPORTED, "only single-rank operators (MPI_COMM_SELF)"};
        validate_points( src, n_src, src_pt_stride, src_dim_stride, "source points" );
        validate_points( tgt, n_tgt, tgt_pt_stride, tgt_dim_stride, "target points" );
        // DTK_CHECK( !search_tree.empty() ), DTK_NearestNeighborOperator_def.hpp:44
        DTK_REQUIRE_OR_THROW( n_src > 0, "the source point cloud is empty" );
        require_device_memory( src, "source points" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        auto h = std::make_unique<dtk_nn_s>( s );
        TouchOnExit const touch{&h->life, s};
        h->n_src = n_src;
        h->n_tgt = n_tgt;
        h->idx.allocate( std::max<int64_t>( 1, n_tgt ), s );
        if ( n_tgt > 0 )
        {
            PointsView const sv{src, n_src, src_pt_stride, src_dim_stride};
            PointsView const tv{tgt, n_tgt, tgt_pt_stride, tgt_dim_stride};
            DeviceBuffer<unsigned> status( 1, s );
            DeviceBuffer<int32_t> offset( n_tgt + 1, s );
            DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
            k_iota_offsets<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( offset.get(), n_tgt );
            check_launch( "k_iota_offsets" );
            Lbvh tree;
            DeviceBuffer<uint32_t> order;
            build_tree_and_order( sv, tv, tree, order, status.get(), s );
            knn_query( tree, tv, order.get(), 1, GroupArgs{}, offset.get(), h->idx.get(), status.get(), s );
            unsigned st = 0;
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
            tree = Lbvh();
            DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
            if ( st & DEV_TIMEOUT )
                throw Error{DTK_ERR_TIMEOUT, "a bounded device loop (tree traversal) hit its cap"};
            if ( st )
                throw Error{DTK_ERR_INTERNAL, "search traversal reported an internal error"};
        }
        *out = h.release();
    } );
}

dtk_status dtk_nn_apply( dtk_nn_handle h, const double *source_values, int64_t n_source_values,
                         double *target_values, int64_t n_target_values, dtk_stream_t stream )
{
    return dtk_nn_apply_multi( h, source_values, n_source_values, 1, 1, 1, target_values, n_target_values, 1,
                               1, stream );
}

dtk_status dtk_nn_apply_multi( dtk_nn_handle h, const double *source_values, int64_t n_source_values,
                               int64_t n_comp, int64_t src_pt_stride, int64_t src_comp_stride,
                               double *target_values, int64_t n_target_values, int64_t tgt_pt_stride,
                               int64_t tgt_comp_stride, dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_set_target_values" );
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        // DTK_REQUIRE at DTK_NearestNeighborOperator_def.hpp:79-80
        DTK_REQUIRE_OR_THROW( n_target_values == h->n_tgt, "_indices.extent(0) == target_values.extent(0)" );
        DTK_REQUIRE_OR_THROW( n_source_values == h->n_src, "_size == source_values.extent(0)" );
        FieldView const in = field_in( source_values, h->n_src, n_comp, src_pt_stride, src_comp_stride,
                                       "source_values" );
        FieldView out = field_in( target_values, h->n_tgt, n_comp, tgt_pt_stride, tgt_comp_stride,
                                  "target_values" );
        out.wbase = target_values;
        if ( h->n_tgt == 0 )
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        int64_t const n = h->n_tgt * n_comp;
        k_gather<<<(unsigned)( ( n + 255 ) / 256 ), 256, 0, s>>>( h->n_tgt, h->idx.get(), in, out );
        check_launch( "k_gather" );
    } );
}

dtk_status dtk_nn_get_indices( dtk_nn_handle h, const int32_t **indices, int64_t *n_targets )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( indices )
            *indices = h->idx.get();
        if ( n_targets )
            *n_targets = h->n_tgt;
    } );
}

dtk_status dtk_nn_destroy( dtk_nn_handle h )
{
    return guarded( [&] { delete h; } );
}

dtk_status dtk_mls_apply_multi( dtk_mls_handle h, const double *source_values, int64_t n_source_values,
                                int64_t n_comp, int64_t src_pt_stride, int64_t src_comp_stride,
                                double *target_values, int64_t n_target_values, int64_t tgt_pt_stride,
                                int64_t tgt_comp_stride, dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_compute_values" );
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        // DTK_REQUIRE at DTK_MovingLeastSquaresOperator_def.hpp:129-130, per component
        DTK_REQUIRE_OR_THROW( n_source_values == h->n_src, "source_values.extent(0) == n_source_points" );
        DTK_REQUIRE_OR_THROW( n_target_values == h->n_tgt, "target_values.extent(0) == n_target_points" );
        FieldView const in = field_in( source_values, h->n_src, n_comp, src_pt_stride, src_comp_stride,
                                       "source_values" );
        FieldView out = field_in( target_values, h->n_tgt, n_comp, tgt_pt_stride, tgt_comp_stride,
                                  "target_values" );
        out.wbase = target_values;
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        apply_csr_multi( h->n_tgt, h->offset.get(), h->idx.get(), h->coeff64.get(), h->coeff32.get(), in,
                         out, s );
    } );
}

} // extern "C"
