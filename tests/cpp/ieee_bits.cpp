// The integer-pipe IEEE helpers of the FP64 Jacobi (datatransferkit_gb300/
// csrc/dtk_ieee.cuh), built for the host, against the host's IEEE
// arithmetic: comparisons, signs, negation, sign products, the half-angle's
// range test and its doubling, over signed zeros, subnormals, normals near
// the range bounds, the largest finite values, infinities, NaN and random
// bit patterns.  Built and run by tests/test_ieee_bits_cpu.py; prints "PASS".
#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#include "dtk_ieee.cuh"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <random>
#include <vector>

#define REQUIRE( c )                                                                                \
    do                                                                                              \
    {                                                                                               \
        if ( !( c ) )                                                                               \
        {                                                                                           \
            std::printf( "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c );                              \
            std::exit( 1 );                                                                         \
        }                                                                                           \
    } while ( 0 )

using dtk::bits_of;

// equal bits, or both NaN
static bool same( double a, double b )
{
    return ( std::isnan( a ) && std::isnan( b ) ) || bits_of( a ) == bits_of( b );
}

int main()
{
    double const inf = std::numeric_limits<double>::infinity();
    double const nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -2.0, DBL_MIN, -DBL_MIN, DBL_TRUE_MIN, -DBL_TRUE_MIN,
                             DBL_MAX, -DBL_MAX, inf, -inf, nan, -nan, 1e-280, 1e280, 3.0e-17, -7.25e12};
    for ( double b : {1e-280, 1e280, DBL_MIN, 1.0} )
    {
        v.push_back( std::nextafter( b, 0.0 ) );
        v.push_back( std::nextafter( b, inf ) );
    }
    std::mt19937_64 g( 7 );
    for ( int i = 0; i < 400; ++i )
        v.push_back( dtk::of_bits( g() ) ); // every exponent, sign, NaN payloads
    for ( int i = 0; i < 200; ++i )
        v.push_back( std::ldexp( std::uniform_real_distribution<double>( -1.0, 1.0 )( g ), (int)( g() % 2100 ) - 1075 ) );

    for ( double x : v )
    {
        REQUIRE( dtk::ieee_nonneg( x ) == ( x >= 0.0 ) );
        REQUIRE( dtk::ieee_sign( x ) == ( ( x > 0.0 ) - ( x < 0.0 ) ) );
        REQUIRE( same( dtk::ieee_neg( x ), -x ) );
        REQUIRE( dtk::nan_bits( bits_of( x ) ) == std::isnan( x ) );
        REQUIRE( dtk::zero_bits( bits_of( x ) ) == ( x == 0.0 ) );
        for ( double y : v )
        {
            REQUIRE( dtk::ieee_eq( x, y ) == ( x == y ) );
            REQUIRE( same( dtk::times_sign_of( x, y ), x * std::copysign( 1.0, y ) ) );
        }
        // the half-angle's r^2 >= 0 or NaN
        if ( x >= 0.0 || std::isnan( x ) )
            REQUIRE( dtk::r2_in_range( bits_of( x ) ) == ( x > 1e-280 && x < 1e280 ) );
        // its r: normal (and 2 r finite), +inf or NaN
        bool const normal = x >= DBL_MIN && x <= DBL_MAX / 2;
        if ( normal || x == inf || std::isnan( x ) )
            REQUIRE( same( dtk::twice_normal( x ), 2.0 * x ) );
    }
    std::printf( "PASS\n" );
    return 0;
}
