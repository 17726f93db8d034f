/*
 * Header-only drop-in for DataTransferKit's MLS operator on one rank, over
 * the C ABI of dtk_gb300.h (link with libdtk_gb300.so).
 *
 * Mirrors (paths inside the DataTransferKit project):
 *   DataTransferKit::MovingLeastSquaresOperator<DeviceType, RBF, Basis>
 *       packages/Meshfree/src/DTK_MovingLeastSquaresOperator_decl.hpp:36-63
 *   DataTransferKit::PointCloudOperator<DeviceType>
 *       packages/Meshfree/src/DTK_PointCloudOperator.hpp:24-37
 *   Wendland<k>, Wu<k>, Buhmann<k>, RadialBasisFunction<RBF>
 *       packages/Meshfree/src/DTK_CompactlySupportedRadialBasisFunctions.hpp:22-147
 *   Constant / Linear / Quadratic, MultivariatePolynomialBasis<Basis, DIM>
 *       packages/Meshfree/src/DTK_MultivariatePolynomialBasis.hpp:79-125
 *   DataTransferKitException (DTK_REQUIRE failures)
 *       packages/Utils/src/DTK_DBC.hpp:36-89
 *
 * Views: any type with data(), extent(i) and stride(i) over device memory --
 * a Kokkos::View in a CUDA memory space satisfies this, as does the small
 * DataTransferKit::DeviceView below.  Points are rank-2 (n x 3) views of
 * double in either layout; values are rank-1 contiguous views of double.
 * PointCloudOperator<DeviceType>::apply is virtual over the reference's own
 * value views, Kokkos::View<double const *, DeviceType> and
 * Kokkos::View<double *, DeviceType>, when <Kokkos_Core.hpp> is included
 * before this header, and over DeviceView otherwise.
 * apply returns after the target values are written, like the reference's
 * apply, which ends in Kokkos::deep_copy (DTK_MovingLeastSquaresOperator_def.hpp:140);
 * MlsOptions::asynchronous leaves it queued on the operator's stream instead.
 * Communicators: MPI_Comm (with <mpi.h> included first) or any type with
 * rank(), size(), allgather() and alltoallv() (DTK_DistributedSearch.hpp);
 * with more than one rank the constructor and apply are collective and run
 * the distributed search and value fetch (kNN rows only).  Any other
 * communicator value is taken as one rank.  The header needs the CUDA
 * runtime's headers (cuda_runtime.h) for the multi-rank path.
 */
#ifndef DTK_GB300_MOVING_LEAST_SQUARES_OPERATOR_HPP
#define DTK_GB300_MOVING_LEAST_SQUARES_OPERATOR_HPP

#include "../dtk_gb300.h"
#include "DTK_DistributedSearch.hpp"

#include <cmath>
#include <functional>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace DataTransferKit
{

using Coordinate = double;

class DataTransferKitException : public std::logic_error
{
  public:
    explicit DataTransferKitException( std::string const &msg )
        : std::logic_error( msg )
    {
    }
};

namespace Details
{
inline void check( dtk_status s )
{
    if ( s != DTK_OK )
        throw DataTransferKitException( std::string( dtk_status_string( s ) ) + ": " +
                                        dtk_last_error() );
}
} // namespace Details

// ---------------------------------------------------------------------------
// Compactly supported radial basis functions (the id selects the GPU kernel;
// operator() evaluates the same formula on the host).
// ---------------------------------------------------------------------------
template <typename RBF>
class RadialBasisFunction
{
  public:
    explicit RadialBasisFunction( double radius )
        : _radius( radius )
    {
    }
    double operator()( double x ) const { return RBF()( x / _radius ); }

  private:
    double _radius;
};

template <int k>
struct Wendland;
template <>
struct Wendland<0>
{
    static constexpr int id = DTK_WENDLAND0;
    double operator()( double x ) const { return ( 1 - x ) * ( 1 - x ); }
};
template <>
struct Wendland<2>
{
    static constexpr int id = DTK_WENDLAND2;
    double operator()( double x ) const
    {
        double const y = 1 - x;
        return y * y * y * y * ( 4 * x + 1 );
    }
};
template <>
struct Wendland<4>
{
    static constexpr int id = DTK_WENDLAND4;
    double operator()( double x ) const
    {
        double const y = 1 - x;
        return y * y * y * y * y * y * ( 35 * x * x + 18 * x + 3 );
    }
};
template <>
struct Wendland<6>
{
    static constexpr int id = DTK_WENDLAND6;
    double operator()( double x ) const
    {
        double const y = 1 - x;
        return y * y * y * y * y * y * y * y * ( 32 * x * x * x + 25 * x * x + 8 * x + 1 );
    }
};

template <int k>
struct Wu;
template <>
struct Wu<2>
{
    static constexpr int id = DTK_WU2;
    double operator()( double x ) const
    {
        double const y = 1 - x;
        return y * y * y * y * ( 3 * x * x * x + 12 * x * x + 16 * x + 4 );
    }
};
template <>
struct Wu<4>
{
    static constexpr int id = DTK_WU4;
    double operator()( double x ) const
    {
        double const y = 1 - x;
        return y * y * y * y * y * y *
               ( 5 * x * x * x * x * x + 30 * x * x * x * x + 72 * x * x * x + 82 * x * x + 36 * x + 6 );
    }
};

template <int k>
struct Buhmann;
template <>
struct Buhmann<2>
{
    static constexpr int id = DTK_BUHMANN2;
    double operator()( double x ) const
    {
        return 2 * x * x * x * x * std::log( x ) - 3.5 * x * x * x * x + 16 / 3.0 * x * x * x -
               2 * x * x + 1.0 / 6.0;
    }
};
template <>
struct Buhmann<3>
{
    static constexpr int id = DTK_BUHMANN3;
    double operator()( double x ) const
    {
        double const r = std::sqrt( x );
        return std::pow( x, 8 ) - 84.0 / 5.0 * std::pow( x, 6 ) + 1024.0 / 5.0 * std::pow( x, 4 ) * r -
               378 * std::pow( x, 4 ) + 1024.0 / 5.0 * x * x * x * r - 84.0 / 5.0 * x * x + 1;
    }
};
template <>
struct Buhmann<4>
{
    static constexpr int id = DTK_BUHMANN4;
    double operator()( double x ) const
    {
        double const r = std::sqrt( x );
        return 99.0 / 35.0 * std::pow( x, 8 ) - 132 * std::pow( x, 6 ) +
               9216.0 / 35.0 * std::pow( x, 5 ) * r - 11264.0 / 35.0 * std::pow( x, 4 ) * r +
               198 * std::pow( x, 4 ) - 396.0 / 5.0 * x * x + 1;
    }
};

// ---------------------------------------------------------------------------
// Polynomial bases
// ---------------------------------------------------------------------------
struct Constant
{
};
struct Linear
{
};
struct Quadratic
{
};

namespace Details
{
template <typename Basis, int DIM>
struct Size;
template <int DIM>
struct Size<Constant, DIM>
{
    static constexpr int value = 1;
};
template <>
struct Size<Linear, 3>
{
    static constexpr int value = 4;
};
template <>
struct Size<Quadratic, 3>
{
    static constexpr int value = 10;
};
template <>
struct Size<Linear, 2>
{
    static constexpr int value = 3;
};
template <>
struct Size<Quadratic, 2>
{
    static constexpr int value = 6;
};
template <typename Basis>
struct BasisId;
template <>
struct BasisId<Constant>
{
    static constexpr int value = DTK_CONSTANT3;
};
template <>
struct BasisId<Linear>
{
    static constexpr int value = DTK_LINEAR3;
};
template <>
struct BasisId<Quadratic>
{
    static constexpr int value = DTK_QUADRATIC3;
};
} // namespace Details

template <typename Basis, int DIM>
struct MultivariatePolynomialBasis
{
    static constexpr int size = Details::Size<Basis, DIM>::value;
    static constexpr int dim = DIM;
    static constexpr int id = Details::BasisId<Basis>::value;
};

// ---------------------------------------------------------------------------
// Device and view helpers
// ---------------------------------------------------------------------------
struct CudaSpace
{
};
struct Cuda
{
    using execution_space = Cuda;
    using memory_space = CudaSpace;
};
// A device type for callers without Kokkos.
struct CudaDevice
{
    using execution_space = Cuda;
    using memory_space = CudaSpace;
};

// Minimal non-owning view over device memory (rank 1 or 2, element strides).
template <typename T>
struct DeviceView
{
    T *ptr = nullptr;
    std::size_t n0 = 0, n1 = 1;
    std::ptrdiff_t s0 = 1, s1 = 1;
    T *data() const { return ptr; }
    std::size_t extent( int d ) const { return d == 0 ? n0 : d == 1 ? n1 : 1; }
    std::ptrdiff_t stride( int d ) const { return d == 0 ? s0 : s1; }
};

// The value views of the virtual PointCloudOperator::apply: the reference's
// (DTK_PointCloudOperator.hpp:34-36) when Kokkos is included first, the
// DeviceView stand-ins otherwise.
#if defined( KOKKOS_VERSION )
template <typename DeviceType>
using SourceValuesView = Kokkos::View<double const *, DeviceType>;
template <typename DeviceType>
using TargetValuesView = Kokkos::View<double *, DeviceType>;
#else
template <typename DeviceType>
using SourceValuesView = DeviceView<double const>;
template <typename DeviceType>
using TargetValuesView = DeviceView<double>;
#endif

/* Extensions to the reference constructor: neighbours, radius search, the
 * precision form, the stream (it must outlive the operator, whose buffers
 * are freed on it), and whether apply may return before its results are
 * written (defaults reproduce the reference: k = basis size, kNN, FP64,
 * synchronous apply). */
struct MlsOptions
{
    int k = 0;
    double radius = 0.0;
    int precision = DTK_FP64;
    dtk_stream_t stream = nullptr;
    bool asynchronous = false;
};

namespace Details
{
template <typename Comm>
int comm_size( Comm const &comm )
{
    return CommTraits<Comm>::size( comm );
}
} // namespace Details

template <typename DeviceType>
class PointCloudOperator
{
  public:
    virtual ~PointCloudOperator() = default;
    virtual void apply( SourceValuesView<DeviceType> source_values,
                        TargetValuesView<DeviceType> target_values ) const = 0;
};

template <typename DeviceType, typename CompactlySupportedRadialBasisFunction = Wendland<0>,
          typename PolynomialBasis = MultivariatePolynomialBasis<Linear, 3>>
class MovingLeastSquaresOperator : public PointCloudOperator<DeviceType>
{
  public:
    using device_type = DeviceType;
    using ExecutionSpace = typename DeviceType::execution_space;
    using polynomial_basis = PolynomialBasis;
    using radial_basis_function = CompactlySupportedRadialBasisFunction;

    template <typename Comm, typename SourceView, typename TargetView>
    MovingLeastSquaresOperator( Comm comm, SourceView const &source_points,
                                TargetView const &target_points, MlsOptions const &ext = {} )
        : _n_source_points( source_points.extent( 0 ) )
        , _n_target_points( target_points.extent( 0 ) )
        , _stream( ext.stream )
        , _asynchronous( ext.asynchronous )
    {
        // DTK_REQUIRE(source dim == target dim), DTK_REQUIRE(dim == 3):
        // DTK_MovingLeastSquaresOperator_def.hpp:39-42
        if ( source_points.extent( 1 ) != target_points.extent( 1 ) )
            throw DataTransferKitException(
                "DTK_REQUIRE( source_points.extent_int( 1 ) == target_points.extent_int( 1 ) )" );
        if ( source_points.extent( 1 ) != 3 || PolynomialBasis::dim != 3 )
            throw DataTransferKitException( "DTK_REQUIRE( source_points.extent_int( 1 ) == 3 )" );
        dtk_mls_options o;
        dtk_mls_default_options( &o );
        o.rbf = CompactlySupportedRadialBasisFunction::id;
        o.basis = PolynomialBasis::id;
        o.k = ext.k;
        o.radius = ext.radius;
        o.precision = ext.precision;
        o.comm_size = Details::comm_size( comm );
        if constexpr ( Details::CommTraits<Comm>::exchange )
            if ( o.comm_size > 1 )
            {
                // the distributed search and fetch of the reference's MPI
                // operator (DTK_MovingLeastSquaresOperator_def.hpp:47-67)
                if ( ext.radius > 0.0 )
                    throw DataTransferKitException( "DTK_ERR_UNSUPPORTED: the distributed operator takes kNN rows" );
                int const k = ext.k ? ext.k : PolynomialBasis::size;
                if ( k > 32 )
                    throw DataTransferKitException( "DTK_ERR_UNSUPPORTED: kNN search supports k <= 32" );
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
                        k, reinterpret_cast<cudaStream_t>( _stream ) );
                }
                catch ( std::exception const &e )
                {
                    throw DataTransferKitException( e.what() );
                }
                _handle = d->handle;
                _dist_apply = [comm, d]( double const *sv, double *tv ) {
                    Details::distributed_apply( comm, *d, sv, tv );
                };
                return;
            }
        dtk_mls_handle h = nullptr;
        Details::check( dtk_mls_create(
            &o, reinterpret_cast<double const *>( source_points.data() ),
            (int64_t)source_points.extent( 0 ), (int64_t)source_points.stride( 0 ),
            (int64_t)source_points.stride( 1 ), reinterpret_cast<double const *>( target_points.data() ),
            (int64_t)target_points.extent( 0 ), (int64_t)target_points.stride( 0 ),
            (int64_t)target_points.stride( 1 ), _stream, &h ) );
        _handle.reset( h, []( dtk_mls_handle p ) { dtk_mls_destroy( p ); } );
    }

    template <typename SourceValues, typename TargetValues>
    void apply_values( SourceValues const &source_values, TargetValues const &target_values ) const
    {
        // DTK_REQUIRE at DTK_MovingLeastSquaresOperator_def.hpp:129-130
        if ( (std::size_t)source_values.extent( 0 ) != _n_source_points )
            throw DataTransferKitException(
                "DTK_REQUIRE( source_values.extent( 0 ) == _n_source_points )" );
        if ( (std::size_t)target_values.extent( 0 ) != _n_target_points )
            throw DataTransferKitException(
                "DTK_REQUIRE( target_values.extent( 0 ) == _offset.extent( 0 ) - 1 )" );
        if ( _dist_apply )
        {
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
        Details::check( dtk_mls_apply( _handle.get(),
                                       reinterpret_cast<double const *>( source_values.data() ),
                                       (int64_t)source_values.extent( 0 ),
                                       const_cast<double *>( reinterpret_cast<double const *>(
                                           target_values.data() ) ),
                                       (int64_t)target_values.extent( 0 ), _stream ) );
        if ( !_asynchronous ) // the reference's deep_copy fences
            Details::check( dtk_stream_synchronize( _stream ) );
    }

    void apply( SourceValuesView<DeviceType> source_values,
                TargetValuesView<DeviceType> target_values ) const override
    {
        apply_values( source_values, target_values );
    }

    // apply(source_values, target_values) for any other view type.
    template <typename SourceValues, typename TargetValues,
              typename = std::enable_if_t<!std::is_same<SourceValues, SourceValuesView<DeviceType>>::value>>
    void apply( SourceValues const &source_values, TargetValues const &target_values ) const
    {
        apply_values( source_values, target_values );
    }

    // Extensions
    // Rank-2 fields (n x n_comp views, any layout): every component alike.
    template <typename SourceValues, typename TargetValues>
    void apply_fields( SourceValues const &source_values, TargetValues const &target_values ) const
    {
        if ( _dist_apply )
            throw DataTransferKitException( "DTK_ERR_UNSUPPORTED: rank-2 fields on one rank only" );
        if ( source_values.extent( 1 ) != target_values.extent( 1 ) )
            throw DataTransferKitException(
                "DTK_REQUIRE( source_values.extent( 1 ) == target_values.extent( 1 ) )" );
        Details::check( dtk_mls_apply_multi(
            _handle.get(), reinterpret_cast<double const *>( source_values.data() ),
            (int64_t)source_values.extent( 0 ), (int64_t)source_values.extent( 1 ),
            (int64_t)source_values.stride( 0 ), (int64_t)source_values.stride( 1 ),
            const_cast<double *>( reinterpret_cast<double const *>( target_values.data() ) ),
            (int64_t)target_values.extent( 0 ), (int64_t)target_values.stride( 0 ),
            (int64_t)target_values.stride( 1 ), _stream ) );
        if ( !_asynchronous )
            Details::check( dtk_stream_synchronize( _stream ) );
    }
    int64_t underdetermined() const
    {
        int64_t n = 0;
        Details::check( dtk_mls_underdetermined_count( _handle.get(), &n ) );
        return n;
    }
    dtk_mls_handle handle() const { return _handle.get(); }

  private:
    std::size_t _n_source_points, _n_target_points;
    dtk_stream_t _stream;
    bool _asynchronous;
    std::shared_ptr<struct dtk_mls_s> _handle;
    std::function<void( double const *, double * )> _dist_apply; // set with more than one rank
};

} // namespace DataTransferKit

#endif
