/*
 * Header-only drop-in for DataTransferKit's NearestNeighborOperator on one
 * rank, over the C ABI of dtk_gb300.h (link with libdtk_gb300.so).
 *
 * Mirrors (paths inside the DataTransferKit project):
 *   DataTransferKit::NearestNeighborOperator<DeviceType>
 *       packages/Meshfree/src/DTK_NearestNeighborOperator_decl.hpp:27-49
 *       packages/Meshfree/src/DTK_NearestNeighborOperator_def.hpp:23-86
 *
 * Views, communicator, exceptions and the synchronous apply (the reference's
 * ends in Kokkos::deep_copy, DTK_NearestNeighborOperator_def.hpp:85) as in
 * DTK_MovingLeastSquaresOperator.hpp; with a communicator of several ranks
 * the nearest source is searched on every rank and its value fetched
 * (rank-1 values), DTK_DistributedSearch.hpp.
 * The nearest source of a target is the smallest (d^2, source index): ties
 * go to the smaller source index.
 */
#ifndef DTK_GB300_NEAREST_NEIGHBOR_OPERATOR_HPP
#define DTK_GB300_NEAREST_NEIGHBOR_OPERATOR_HPP

#include "DTK_MovingLeastSquaresOperator.hpp"

namespace DataTransferKit
{

template <typename DeviceType>
class NearestNeighborOperator : public PointCloudOperator<DeviceType>
{
  public:
    using device_type = DeviceType;
    using ExecutionSpace = typename DeviceType::execution_space;

    template <typename Comm, typename SourceView, typename TargetView>
    NearestNeighborOperator( Comm comm, SourceView const &source_points, TargetView const &target_points,
                             dtk_stream_t stream = nullptr, bool asynchronous = false )
        : _size( source_points.extent( 0 ) )
        , _n_target_points( target_points.extent( 0 ) )
        , _stream( stream )
        , _asynchronous( asynchronous )
    {
        if constexpr ( Details::CommTraits<Comm>::exchange )
            if ( Details::comm_size( comm ) > 1 )
            {
                if ( source_points.extent( 1 ) != 3 || target_points.extent( 1 ) != 3 )
                    throw DataTransferKitException( "DTK_REQUIRE( source_points.extent_int( 1 ) == 3 )" );
                dtk_mls_options o;
                dtk_mls_default_options( &o );
                std::shared_ptr<Details::DistributedOperator> d;
                try
                {
                    d = Details::distributed_setup(
                        comm, o,
                        Details::PointsArg{reinterpret_cast<double const *>( source_points.data() ),
                                           (int64_t)source_points.extent( 0 ), (int64_t)source_points.stride( 0 ),
                                           (int64_t)source_points.stride( 1 )},
                        Details::PointsArg{reinterpret_cast<double const *>( target_points.data() ),
                                           (int64_t)target_points.extent( 0 ), (int64_t)target_points.stride( 0 ),
                                           (int64_t)target_points.stride( 1 )},
                        1, reinterpret_cast<cudaStream_t>( _stream ), false );
                }
                catch ( std::exception const &e )
                {
                    throw DataTransferKitException( e.what() );
                }
                _dist_apply = [comm, d]( double const *sv, double *tv ) {
                    Details::distributed_apply_nearest( comm, *d, sv, tv );
                };
                return;
            }
        dtk_nn_handle h = nullptr;
        Details::check( dtk_nn_create(
            reinterpret_cast<double const *>( source_points.data() ), (int64_t)source_points.extent( 0 ),
            (int64_t)source_points.stride( 0 ), (int64_t)source_points.stride( 1 ),
            reinterpret_cast<double const *>( target_points.data() ), (int64_t)target_points.extent( 0 ),
            (int64_t)target_points.stride( 0 ), (int64_t)target_points.stride( 1 ),
            Details::comm_size( comm ), _stream, &h ) );
        _handle.reset( h, []( dtk_nn_handle p ) { dtk_nn_destroy( p ); } );
    }

    template <typename SourceValues, typename TargetValues>
    void apply_values( SourceValues const &source_values, TargetValues const &target_values ) const
    {
        // DTK_REQUIRE at DTK_NearestNeighborOperator_def.hpp:79-80
        if ( (std::size_t)target_values.extent( 0 ) != _n_target_points )
            throw DataTransferKitException( "DTK_REQUIRE( _indices.extent( 0 ) == target_values.extent( 0 ) )" );
        if ( (std::size_t)source_values.extent( 0 ) != _size )
            throw DataTransferKitException( "DTK_REQUIRE( _size == source_values.extent_int( 0 ) )" );
        if ( _dist_apply )
        {
            if ( source_values.extent( 1 ) != 1 || target_values.extent( 1 ) != 1 )
                throw DataTransferKitException( "DTK_ERR_UNSUPPORTED: rank-2 values on one rank only" );
            try
            {
                _dist_apply( reinterpret_cast<double const *>( source_values.data() ),
                             const_cast<double *>( reinterpret_cast<double const *>( target_values.data() ) ) );
            }
            catch ( std::exception const &e )
            {
                throw DataTransferKitException( e.what() );
            }
            if ( !_asynchronous )
                Details::check( dtk_stream_synchronize( _stream ) );
            return;
        }
        Details::check( dtk_nn_apply_multi(
            _handle.get(), reinterpret_cast<double const *>( source_values.data() ),
            (int64_t)source_values.extent( 0 ), (int64_t)source_values.extent( 1 ),
            (int64_t)source_values.stride( 0 ), (int64_t)source_values.stride( 1 ),
            const_cast<double *>( reinterpret_cast<double const *>( target_values.data() ) ),
            (int64_t)target_values.extent( 0 ), (int64_t)target_values.stride( 0 ),
            (int64_t)target_values.stride( 1 ), _stream ) );
        if ( !_asynchronous )
            Details::check( dtk_stream_synchronize( _stream ) );
    }

    void apply( SourceValuesView<DeviceType> source_values,
                TargetValuesView<DeviceType> target_values ) const override
    {
        apply_values( source_values, target_values );
    }

    // apply(source_values, target_values) for any other view type, rank 1
    // or rank 2 (the reference's fetch handles both).
    template <typename SourceValues, typename TargetValues,
              typename = std::enable_if_t<!std::is_same<SourceValues, SourceValuesView<DeviceType>>::value>>
    void apply( SourceValues const &source_values, TargetValues const &target_values ) const
    {
        apply_values( source_values, target_values );
    }

    dtk_nn_handle handle() const { return _handle.get(); } // null with more than one rank

  private:
    std::size_t _size, _n_target_points;
    dtk_stream_t _stream;
    bool _asynchronous;
    std::shared_ptr<struct dtk_nn_s> _handle;
    std::function<void( double const *, double * )> _dist_apply; // set with more than one rank
};

} // namespace DataTransferKit

#endif
