// The oracle under AddressSanitizer and UndefinedBehaviorSanitizer: every
// entry point of oracle/dtk_oracle.h on small clouds, including the edge
// shapes the tests use (fewer sources than k, empty targets, duplicates,
// collinear and coplanar rows, radius rows of length 0 and 1), and its
// argument checks.  Built and run by tests/test_oracle_sanitize.py; any
// sanitizer report fails the run.  Prints "PASS" on success.
#include "dtk_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
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

static std::vector<double> cloud( int n, unsigned seed, double scale = 1.0 )
{
    std::mt19937_64 g( seed );
    std::uniform_real_distribution<double> u( 0.0, 1.0 );
    std::vector<double> p( 3 * n );
    for ( auto &v : p )
        v = scale * u( g );
    return p;
}

static void mls_case( std::vector<double> const &src, std::vector<double> const &tgt, int k, double r )
{
    int64_t const ns = (int64_t)src.size() / 3, nt = (int64_t)tgt.size() / 3;
    std::vector<int32_t> offset( nt + 1 );
    std::vector<int32_t> idx;
    std::vector<double> d2;
    if ( r > 0 )
    {
        int64_t const nnz = dtk_oracle_radius_count( src.data(), ns, tgt.data(), nt, r, offset.data() );
        REQUIRE( nnz >= 0 );
        idx.resize( nnz );
        d2.resize( nnz );
        REQUIRE( dtk_oracle_radius_fill( src.data(), ns, tgt.data(), nt, r, offset.data(), idx.data(),
                                         d2.data() ) == 0 );
    }
    else
    {
        int const row = (int)std::min<int64_t>( k, ns );
        idx.resize( nt * row );
        d2.resize( nt * row );
        REQUIRE( dtk_oracle_knn( src.data(), ns, tgt.data(), nt, k, offset.data(), idx.data(), d2.data() ) == 0 );
        std::vector<int32_t> ob( nt + 1 ), ib( nt * row );
        std::vector<double> db( nt * row );
        REQUIRE( dtk_oracle_knn_brute( src.data(), ns, tgt.data(), nt, k, ob.data(), ib.data(), db.data() ) == 0 );
        REQUIRE( ib == idx && db == d2 );
    }
    std::vector<double> vals( ns ), out( nt ), cot( nt, 1.0 ), grad( ns ), gxyz( 3 * ns, 0.0 );
    for ( int64_t i = 0; i < ns; ++i )
        vals[i] = std::sin( src[3 * i] ) + src[3 * i + 1];
    for ( int basis = 0; basis < 3; ++basis )
        for ( int rbf = 0; rbf < 9; ++rbf )
        {
            int const m = dtk_oracle_basis_size( basis );
            std::vector<double> coeff( idx.size() ), rad( nt ), row0( nt * m );
            REQUIRE( dtk_oracle_mls_coefficients( src.data(), tgt.data(), nt, offset.data(), idx.data(), rbf,
                                                  basis, coeff.data(), rad.data(), row0.data() ) >= 0 );
            REQUIRE( dtk_oracle_apply( nt, offset.data(), idx.data(), coeff.data(), vals.data(), out.data() ) == 0 );
            REQUIRE( dtk_oracle_apply_transpose( nt, ns, offset.data(), idx.data(), coeff.data(), cot.data(),
                                                 grad.data() ) == 0 );
            if ( rbf < 6 ) // the coordinate gradient is defined for the Wendland and Wu functions here
                REQUIRE( dtk_oracle_coord_grad( src.data(), ns, tgt.data(), nt, offset.data(), idx.data(), rbf,
                                                basis, vals.data(), cot.data(), gxyz.data() ) == 0 );
        }
}

int main()
{
    dtk_oracle_set_threads( 2 );
    mls_case( cloud( 2000, 1 ), cloud( 300, 2 ), 20, 0.0 );
    mls_case( cloud( 2000, 3 ), cloud( 300, 4 ), 32, 0.0 );
    mls_case( cloud( 3, 5 ), cloud( 10, 6 ), 4, 0.0 );        // fewer sources than k
    mls_case( cloud( 500, 7 ), {}, 10, 0.0 );                 // no targets
    mls_case( cloud( 1500, 8 ), cloud( 200, 9 ), 0, 0.08 );   // radius rows (0 and 1 entries included)
    {
        // duplicates, collinear and coplanar sources
        std::vector<double> s;
        for ( int i = 0; i < 40; ++i )
            s.insert( s.end(), {double( i ), 0.0, 0.0} );
        for ( int i = 0; i < 40; ++i )
            for ( int j = 0; j < 40; ++j )
                s.insert( s.end(), {double( i ), double( j ), 5.0} );
        for ( int i = 0; i < 50; ++i )
            s.insert( s.end(), {0.3, 0.3, 0.3} );
        std::vector<double> t = {19.5, 0.0, 0.0, 19.0, 19.0, 5.0, 0.3, 0.3, 0.3, 100.0, -4.0, 2.0};
        mls_case( s, t, 10, 0.0 );
        mls_case( s, t, 0, 1.5 );
    }
    {
        // pseudo-inverses: full rank and with a zero column
        int const n = 12, count = 6;
        std::vector<double> a = cloud( n * n * count / 3 + 1, 11 ), pinv( n * n * count );
        a.resize( n * n * count );
        for ( int c = 0; c < count; c += 2 )
            for ( int i = 0; i < n; ++i )
                a[c * n * n + i * n + 3] = 0.0;
        REQUIRE( dtk_oracle_svd_pinv( n, count, a.data(), pinv.data() ) == count / 2 );
    }
    {
        std::vector<double> x = {0.0, 0.25, 0.5, 0.75, 1.0}, y( 5 ), p( 3 * 4 ), b( 10 * 4 );
        for ( int rbf = 0; rbf < 9; ++rbf )
            dtk_oracle_rbf( rbf, x.data(), 5, y.data() );
        dtk_oracle_basis( 2, p.data(), 4, b.data() );
    }
    // argument checks
    std::vector<int32_t> o( 2 ), i( 4 );
    std::vector<double> d( 4 ), one = {0.0, 0.0, 0.0};
    REQUIRE( dtk_oracle_knn( one.data(), 1, one.data(), 1, -1, o.data(), i.data(), d.data() ) == -1 );
    REQUIRE( dtk_oracle_svd_pinv( 0, 1, one.data(), d.data() ) == -1 );
    std::printf( "PASS\n" );
    return 0;
}
