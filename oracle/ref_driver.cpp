// TEST INFRASTRUCTURE ONLY: drives the reference's own MLS numerics headers
// (compiled where they lie in the DataTransferKit source tree, against the
// project-written API shim in oracle/ref_shim/) so that the oracle
// restatement and the golden fixtures can be checked against the reference's
// arithmetic.  Built only where the reference sources are present; never
// shipped, never linked by the product.
//
// The driver follows the stage order of
// packages/Meshfree/src/DTK_MovingLeastSquaresOperator_def.hpp:64-118 from
// the fetch onwards.  The ArborX search is not vendored, so the (offset,
// indices) connectivity is an input (the oracle's exact kNN), and the
// single-rank fetch is the gather points(j, :) = source(indices(j), :).
#include <DTK_DBC.hpp>
#include <DTK_DetailsMovingLeastSquaresOperatorImpl.hpp>
#include <DTK_DetailsSVDImpl.hpp>
#include <DTK_CompactlySupportedRadialBasisFunctions.hpp>
#include <DTK_MultivariatePolynomialBasis.hpp>

#include <cstdint>
#include <stdexcept>

namespace DataTransferKit
{
void throwDataTransferKitException( const std::string &cond,
                                    const std::string &file, const int line )
{
    throw DataTransferKitException( cond + " at " + file + ":" +
                                    std::to_string( line ) );
}
} // namespace DataTransferKit

namespace
{
using DeviceType = Kokkos::Device<Kokkos::Serial, Kokkos::HostSpace>;
using Impl = DataTransferKit::Details::MovingLeastSquaresOperatorImpl<DeviceType>;
using DataTransferKit::Coordinate;

template <class RBF, class Basis>
int64_t run_setup( double const *src, double const *tgt, int64_t n_tgt,
                   int32_t const *offset, int32_t const *idx, double *coeff )
{
    int64_t const nnz = offset[n_tgt];
    Kokkos::View<int *, DeviceType> off( "offset", n_tgt + 1 );
    for ( int64_t i = 0; i <= n_tgt; ++i )
        off( i ) = offset[i];
    Kokkos::View<Coordinate **, DeviceType> fetched( "source_points", nnz, 3 );
    for ( int64_t j = 0; j < nnz; ++j )
        for ( int d = 0; d < 3; ++d )
            fetched( j, d ) = src[3 * (int64_t)idx[j] + d];
    Kokkos::View<Coordinate **, DeviceType> targets( "target_points", n_tgt, 3 );
    for ( int64_t i = 0; i < n_tgt; ++i )
        for ( int d = 0; d < 3; ++d )
            targets( i, d ) = tgt[3 * i + d];

    Kokkos::View<Coordinate const **, DeviceType> source_points = fetched;
    source_points =
        Impl::transformSourceCoordinates( source_points, off, targets );
    auto p = Impl::computeVandermonde( source_points, Basis() );
    auto radius = Impl::computeRadius( source_points, off );
    auto phi = Impl::computeWeights( source_points, radius, RBF() );
    auto a = Impl::computeMoments( off, p, phi );
    auto t = Impl::invertMoments( a, Basis::size );
    auto inv_a = std::get<0>( t );
    auto c = Impl::computePolynomialCoefficients( off, inv_a, p, phi, Basis::size );
    for ( int64_t j = 0; j < nnz; ++j )
        coeff[j] = c( j );
    return (int64_t)std::get<1>( t );
}

template <class RBF>
int64_t by_basis( int basis, double const *src, double const *tgt, int64_t n_tgt,
                  int32_t const *offset, int32_t const *idx, double *coeff )
{
    using namespace DataTransferKit;
    switch ( basis )
    {
    case 0:
        return run_setup<RBF, MultivariatePolynomialBasis<Constant, 3>>(
            src, tgt, n_tgt, offset, idx, coeff );
    case 1:
        return run_setup<RBF, MultivariatePolynomialBasis<Linear, 3>>(
            src, tgt, n_tgt, offset, idx, coeff );
    case 2:
        return run_setup<RBF, MultivariatePolynomialBasis<Quadratic, 3>>(
            src, tgt, n_tgt, offset, idx, coeff );
    }
    return -1;
}

template <class RBF>
void eval_rbf( double const *x, int64_t n, double *out )
{
    RBF f;
    for ( int64_t i = 0; i < n; ++i )
        out[i] = f( x[i] );
}
} // namespace

extern "C" {

int64_t dtk_ref_mls_coefficients( double const *src, double const *tgt,
                                  int64_t n_tgt, int32_t const *offset,
                                  int32_t const *idx, int rbf, int basis,
                                  double *coeff )
{
    using namespace DataTransferKit;
    try
    {
        switch ( rbf )
        {
        case 0:
            return by_basis<Wendland<0>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 1:
            return by_basis<Wendland<2>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 2:
            return by_basis<Wendland<4>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 3:
            return by_basis<Wendland<6>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 4:
            return by_basis<Wu<2>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 5:
            return by_basis<Wu<4>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 6:
            return by_basis<Buhmann<2>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 7:
            return by_basis<Buhmann<3>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        case 8:
            return by_basis<Buhmann<4>>( basis, src, tgt, n_tgt, offset, idx, coeff );
        }
    }
    catch ( std::exception const & )
    {
        return -2;
    }
    return -1;
}

// computeTargetValues after the single-rank fetch (def.hpp:192-208).
int dtk_ref_apply( int64_t n_tgt, int32_t const *offset, int32_t const *idx,
                   double const *coeff, double const *values, double *target )
{
    int64_t const nnz = offset[n_tgt];
    Kokkos::View<int *, DeviceType> off( "offset", n_tgt + 1 );
    for ( int64_t i = 0; i <= n_tgt; ++i )
        off( i ) = offset[i];
    Kokkos::View<double *, DeviceType> c( "coeffs", nnz ), v( "values", nnz );
    for ( int64_t j = 0; j < nnz; ++j )
    {
        c( j ) = coeff[j];
        v( j ) = values[idx[j]];
    }
    auto out = Impl::computeTargetValues( off, c, v );
    for ( int64_t i = 0; i < n_tgt; ++i )
        target[i] = out( i );
    return 0;
}

// SVDFunctor over count n x n matrices (tstSVD.cpp:67-100 usage).
int64_t dtk_ref_svd_pinv( int n, int64_t count, double const *a, double *pinv )
{
    Kokkos::View<double *, DeviceType> m( "matrices", count * n * n ),
        inv( "inv_matrices", count * n * n );
    for ( int64_t i = 0; i < count * n * n; ++i )
        m( i ) = a[i];
    Kokkos::View<double **, DeviceType> aux( "aux", n, 3 * count * n );
    DataTransferKit::Details::SVDFunctor<DeviceType> f( n, m, inv, aux );
    size_t under = 0;
    Kokkos::parallel_reduce( "svd", Kokkos::RangePolicy<Kokkos::Serial>( 0, count ),
                             f, under );
    for ( int64_t i = 0; i < count * n * n; ++i )
        pinv[i] = inv( i );
    return (int64_t)under;
}

void dtk_ref_rbf( int rbf, double const *x, int64_t n, double *out )
{
    using namespace DataTransferKit;
    switch ( rbf )
    {
    case 0: eval_rbf<Wendland<0>>( x, n, out ); break;
    case 1: eval_rbf<Wendland<2>>( x, n, out ); break;
    case 2: eval_rbf<Wendland<4>>( x, n, out ); break;
    case 3: eval_rbf<Wendland<6>>( x, n, out ); break;
    case 4: eval_rbf<Wu<2>>( x, n, out ); break;
    case 5: eval_rbf<Wu<4>>( x, n, out ); break;
    case 6: eval_rbf<Buhmann<2>>( x, n, out ); break;
    case 7: eval_rbf<Buhmann<3>>( x, n, out ); break;
    case 8: eval_rbf<Buhmann<4>>( x, n, out ); break;
    }
}

void dtk_ref_basis( int basis, double const *pts, int64_t n, double *out )
{
    using namespace DataTransferKit;
    for ( int64_t i = 0; i < n; ++i )
    {
        ArborX::Point p{{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}};
        if ( basis == 0 )
        {
            auto b = MultivariatePolynomialBasis<Constant, 3>()( p );
            out[i] = b[0];
        }
        else if ( basis == 1 )
        {
            auto b = MultivariatePolynomialBasis<Linear, 3>()( p );
            for ( int c = 0; c < 4; ++c )
                out[4 * i + c] = b[c];
        }
        else
        {
            auto b = MultivariatePolynomialBasis<Quadratic, 3>()( p );
            for ( int c = 0; c < 10; ++c )
                out[10 * i + c] = b[c];
        }
    }
}

} // extern "C"
