// The reference's MLS and nearest-neighbour operator tests, written against
// the header-only drop-ins (include/dtk/DTK_MovingLeastSquaresOperator.hpp,
// include/dtk/DTK_NearestNeighborOperator.hpp) as a DTK user would:
//   tstMeshfreeOperators.cpp:130-376 (same_npoints_and_basis, grid, line)
//   tstMeshfreeOperatorsSimpleProblem.cpp:113-147 (corner_cases)
//   tstNearestNeighborOperator.cpp:85-273 (unique_source_point,
//     structured_clouds, mixed_clouds) on one rank
// plus a LayoutLeft input, a rank-2 field, the DTK_REQUIRE error convention,
// and apply called through PointCloudOperator<DeviceType>& with the
// operator's stream non-blocking, its result read on another stream with no
// other synchronisation (apply returns complete, as the reference's does).
// Built twice: plain, and with -DDTK_FAKE_KOKKOS, where the virtual apply
// takes Kokkos::View<double const *, DeviceType> / Kokkos::View<double *,
// DeviceType> (a test stand-in for Kokkos, tests/cpp/fake_kokkos.hpp).
// Prints "PASS <n>" on success; exits non-zero on the first failure.
#ifdef DTK_FAKE_KOKKOS
#include "fake_kokkos.hpp"
#endif
#include <dtk/DTK_MovingLeastSquaresOperator.hpp>
#include <dtk/DTK_NearestNeighborOperator.hpp>

#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <random>
#include <type_traits>
#include <vector>

using namespace DataTransferKit;
using Pt = std::array<double, 3>;
static int g_checks = 0;

#define CHECK( c )                                                                                  \
    do                                                                                              \
    {                                                                                               \
        ++g_checks;                                                                                 \
        if ( !( c ) )                                                                               \
        {                                                                                           \
            std::printf( "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c );                              \
            std::exit( 1 );                                                                         \
        }                                                                                           \
    } while ( 0 )

struct Buf
{
    double *d = nullptr;
    std::size_t n = 0;
    explicit Buf( std::size_t n_ ) : n( n_ ) { cudaMalloc( &d, std::max<std::size_t>( 1, n ) * 8 ); }
    ~Buf() { cudaFree( d ); }
};

// points: LayoutRight (i, d) at i*3 + d, or LayoutLeft at d*n + i
DeviceView<double const> points( Buf &b, std::vector<Pt> const &p, bool left = false )
{
    std::vector<double> h( 3 * p.size() );
    for ( std::size_t i = 0; i < p.size(); ++i )
        for ( int d = 0; d < 3; ++d )
            h[left ? d * p.size() + i : 3 * i + d] = p[i][d];
    cudaMemcpy( b.d, h.data(), h.size() * 8, cudaMemcpyHostToDevice );
    DeviceView<double const> v;
    v.ptr = b.d;
    v.n0 = p.size();
    v.n1 = 3;
    v.s0 = left ? 1 : 3;
    v.s1 = left ? (std::ptrdiff_t)p.size() : 1;
    return v;
}

DeviceView<double const> values( Buf &b, std::vector<double> const &x )
{
    cudaMemcpy( b.d, x.data(), x.size() * 8, cudaMemcpyHostToDevice );
    DeviceView<double const> v;
    v.ptr = b.d;
    v.n0 = x.size();
    return v;
}

DeviceView<double> out( Buf &b )
{
    DeviceView<double> v;
    v.ptr = b.d;
    v.n0 = b.n;
    return v;
}

std::vector<double> host( Buf &b )
{
    std::vector<double> h( b.n );
    cudaMemcpy( h.data(), b.d, b.n * 8, cudaMemcpyDeviceToHost );
    return h;
}

std::function<double( Pt )> poly( int size )
{
    if ( size == 1 )
        return []( Pt ) { return 3.0; };
    if ( size == 4 )
        return []( Pt p ) { return 4 + 2 * p[0] + 3 * p[1] - 2 * p[2]; };
    return []( Pt p ) {
        return 2 + 3 * p[0] - 5 * p[1] + 2 * p[2] + 3 * p[0] * p[0] + 4 * p[0] * p[1] -
               2 * p[0] * p[2] + p[1] * p[1] - 3 * p[1] * p[2] + 4 * p[2] * p[2];
    };
}

std::vector<Pt> grid( int nx, int ny, int nz, Pt o )
{
    std::vector<Pt> g;
    for ( int i = 0; i < nx; ++i )
        for ( int j = 0; j < ny; ++j )
            for ( int k = 0; k < nz; ++k )
                g.push_back( {o[0] + i, o[1] + j, o[2] + k} );
    return g;
}

template <typename Basis>
void run_basis()
{
    using Op = MovingLeastSquaresOperator<CudaDevice, Wendland<0>, Basis>;
    int const m = Basis::size;
    auto f = poly( m );
    // same_npoints_and_basis: clusters, one target each, exactly m sources
    {
        std::mt19937_64 g( 7 );
        std::uniform_real_distribution<double> rx( -0.5, 0.5 );
        std::vector<Pt> src, tgt;
        for ( int i = 0; i < 10; ++i )
        {
            double const c = i * std::ceil( 4 * 0.5 );
            tgt.push_back( {c + 0.5 * rx( g ), c + 0.5 * rx( g ), c + 0.5 * rx( g )} );
            for ( int k = 0; k < m; ++k )
                src.push_back( {c + rx( g ), c + rx( g ), c + rx( g )} );
        }
        Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( f( p ) );
        Op op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, sv ), out( bo ) );
        auto y = host( bo );
        for ( std::size_t i = 0; i < tgt.size(); ++i )
            CHECK( std::abs( y[i] - f( tgt[i] ) ) <= 1e-7 * std::abs( f( tgt[i] ) ) );
    }
    // grid 40x40x1, target (19,19,0); LayoutLeft inputs
    {
        auto src = grid( 40, 40, 1, {0, 0, 0} );
        std::vector<Pt> tgt = {{19, 19, 0}};
        Buf bs( 3 * src.size() ), bt( 3 ), bv( src.size() ), bo( 1 );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( f( p ) );
        Op op( 0, points( bs, src, true ), points( bt, tgt, true ) );
        op.apply( values( bv, sv ), out( bo ) );
        CHECK( std::abs( host( bo )[0] - f( tgt[0] ) ) <= 1e-14 * std::abs( f( tgt[0] ) ) );
    }
    // line: 40 collinear sources, 39 midpoint targets
    {
        auto src = grid( 40, 1, 1, {0, 0, 0} );
        auto tgt = grid( 39, 1, 1, {0.5, 0, 0} );
        Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( f( p ) );
        Op op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, sv ), out( bo ) );
        auto y = host( bo );
        for ( std::size_t i = 0; i < tgt.size(); ++i )
            CHECK( std::abs( y[i] - f( tgt[i] ) ) <= 1e-14 * std::abs( f( tgt[i] ) ) );
    }
}

// makeStructuredCloud of the reference tests: (i Lx / nx, j Ly / ny, k Lz / nz) + offset
std::vector<Pt> structured( double Lx, double Ly, double Lz, int nx, int ny, int nz )
{
    std::vector<Pt> c;
    for ( int k = 0; k < nz; ++k )
        for ( int j = 0; j < ny; ++j )
            for ( int i = 0; i < nx; ++i )
                c.push_back( {i * Lx / nx, j * Ly / ny, k * Lz / nz} );
    return c;
}

void run_nearest()
{
    using NN = NearestNeighborOperator<CudaDevice>;
    // unique_source_point: source at (comm_size, ...) = (1, 1, 1), target at the origin
    {
        std::vector<Pt> src = {{1, 1, 1}}, tgt = {{0, 0, 0}};
        Buf bs( 3 ), bt( 3 ), bv( 1 ), bo( 1 );
        NN op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, {255.0} ), out( bo ) );
        CHECK( host( bo )[0] == 255.0 );
    }
    // structured_clouds: the target cloud is the source cloud
    {
        auto src = structured( 2., 3., 5., 7, 11, 13 );
        Buf bs( 3 * src.size() ), bt( 3 * src.size() ), bv( src.size() ), bo( src.size() );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( p[0] );
        NN op( 0, points( bs, src ), points( bt, src, true ) );
        op.apply( values( bv, sv ), out( bo ) );
        auto y = host( bo );
        for ( std::size_t i = 0; i < src.size(); ++i )
            CHECK( std::abs( y[i] - src[i][0] ) <= 1e-14 * std::abs( src[i][0] ) );
    }
    // mixed_clouds: random targets in the structured source box
    {
        double const Lx = 17., Ly = 19., Lz = 23.;
        int const nx = 29;
        auto src = structured( Lx, Ly, Lz, nx, 31, 37 );
        std::mt19937_64 g( 0 );
        std::uniform_real_distribution<double> u( 0., 1. );
        std::vector<Pt> tgt;
        for ( int i = 0; i < 41; ++i )
            tgt.push_back( {Lx * u( g ), Ly * u( g ), Lz * u( g )} );
        Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( p[0] );
        NN op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, sv ), out( bo ) );
        auto y = host( bo );
        for ( std::size_t i = 0; i < tgt.size(); ++i )
        {
            double ref = std::round( tgt[i][0] / Lx * nx ) * Lx / nx;
            if ( ref == Lx )
                ref -= Lx / nx;
            CHECK( std::abs( y[i] - ref ) <= 1e-14 * std::abs( ref ) );
        }
    }
    // rank-2 field (LayoutRight, 2 components) and the error convention
    {
        auto src = structured( 1., 1., 1., 4, 4, 4 );
        Buf bs( 3 * src.size() ), bt( 3 * src.size() ), bv( 2 * src.size() ), bo( 2 * src.size() );
        std::vector<double> sv;
        for ( auto &p : src )
        {
            sv.push_back( p[0] );
            sv.push_back( p[2] );
        }
        NN op( 0, points( bs, src ), points( bt, src ) );
        cudaMemcpy( bv.d, sv.data(), sv.size() * 8, cudaMemcpyHostToDevice );
        DeviceView<double const> in;
        in.ptr = bv.d;
        in.n0 = src.size();
        in.n1 = 2;
        in.s0 = 2;
        DeviceView<double> o;
        o.ptr = bo.d;
        o.n0 = src.size();
        o.n1 = 2;
        o.s0 = 2;
        op.apply( in, o );
        CHECK( host( bo ) == sv );
        bool threw = false;
        try
        {
            in.n0 = src.size() - 1;
            op.apply( in, o );
        }
        catch ( DataTransferKitException const & )
        {
            threw = true; // DTK_REQUIRE( _size == source_values.extent_int( 0 ) )
        }
        CHECK( threw );
    }
}

// apply through the base class, with the reference's value view types
void run_polymorphic()
{
#ifdef DTK_FAKE_KOKKOS
    using SrcV = Kokkos::View<double const *, CudaDevice>;
    using TgtV = Kokkos::View<double *, CudaDevice>;
    auto src_view = []( Buf &b ) { return SrcV( b.d, b.n ); };
    auto tgt_view = []( Buf &b ) { return TgtV( b.d, b.n ); };
#else
    using SrcV = DeviceView<double const>;
    using TgtV = DeviceView<double>;
    auto src_view = []( Buf &b ) {
        SrcV v;
        v.ptr = b.d;
        v.n0 = b.n;
        return v;
    };
    auto tgt_view = []( Buf &b ) { return out( b ); };
#endif
    static_assert( std::is_same<SrcV, SourceValuesView<CudaDevice>>::value, "reference value views" );
    static_assert( std::is_same<TgtV, TargetValuesView<CudaDevice>>::value, "reference value views" );
    cudaStream_t s = nullptr, reader = nullptr;
    cudaStreamCreateWithFlags( &s, cudaStreamNonBlocking );
    cudaStreamCreateWithFlags( &reader, cudaStreamNonBlocking );
    auto f = poly( 10 );
    std::mt19937_64 g( 11 );
    std::uniform_real_distribution<double> u( 0., 1. );
    std::vector<Pt> src, tgt;
    for ( int i = 0; i < 200000; ++i )
        src.push_back( {u( g ), u( g ), u( g )} );
    for ( int i = 0; i < 50000; ++i )
        tgt.push_back( {0.1 + 0.8 * u( g ), 0.1 + 0.8 * u( g ), 0.1 + 0.8 * u( g )} );
    Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
    std::vector<double> sv;
    for ( auto &p : src )
        sv.push_back( f( p ) );
    values( bv, sv );
    // (the operators live in this scope: the stream they were created on
    // must outlive them)
    {
        MlsOptions ext;
        ext.k = 32;
        ext.stream = reinterpret_cast<dtk_stream_t>( s );
        using Op = MovingLeastSquaresOperator<CudaDevice, Wendland<2>, MultivariatePolynomialBasis<Quadratic, 3>>;
        Op op( 0, points( bs, src ), points( bt, tgt ), ext );
        PointCloudOperator<CudaDevice> const &base = op;
        for ( int rep = 0; rep < 3; ++rep )
        {
            cudaMemsetAsync( bo.d, 0xff, bo.n * 8, s ); // NaN, queued on the operator's stream
            base.apply( src_view( bv ), tgt_view( bo ) );
            std::vector<double> y( tgt.size() );
            cudaMemcpyAsync( y.data(), bo.d, y.size() * 8, cudaMemcpyDeviceToHost, reader );
            cudaStreamSynchronize( reader );
            for ( std::size_t i = 0; i < tgt.size(); ++i )
                CHECK( std::abs( y[i] - f( tgt[i] ) ) <= 1e-9 * std::max( 1.0, std::abs( f( tgt[i] ) ) ) );
        }
        using NN = NearestNeighborOperator<CudaDevice>;
        NN nn( 0, points( bs, src ), points( bt, tgt ), reinterpret_cast<dtk_stream_t>( s ) );
        PointCloudOperator<CudaDevice> const &nbase = nn;
        cudaMemsetAsync( bo.d, 0xff, bo.n * 8, s );
        nbase.apply( src_view( bv ), tgt_view( bo ) );
        std::vector<double> y( tgt.size() );
        cudaMemcpyAsync( y.data(), bo.d, y.size() * 8, cudaMemcpyDeviceToHost, reader );
        cudaStreamSynchronize( reader );
        for ( std::size_t i = 0; i < tgt.size(); ++i )
            CHECK( std::isfinite( y[i] ) );
    }
    cudaStreamDestroy( s );
    cudaStreamDestroy( reader );
}

int main()
{
    run_polymorphic();
    run_nearest();
    run_basis<MultivariatePolynomialBasis<Constant, 3>>();
    run_basis<MultivariatePolynomialBasis<Linear, 3>>();
    run_basis<MultivariatePolynomialBasis<Quadratic, 3>>();
    // corner_cases: two sources, k = 4 neighbours requested -> rows of 2
    {
        std::vector<Pt> src = {{1, 1, 1}, {2, 2, 2}}, tgt = {{1.5, 1.5, 1.5}};
        Buf bs( 6 ), bt( 3 ), bv( 2 ), bo( 1 );
        MovingLeastSquaresOperator<CudaDevice> op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, {255.0, 255.0} ), out( bo ) );
        CHECK( std::abs( host( bo )[0] - 255.0 ) <= 1e-12 * 255.0 );
    }
    {
        std::vector<Pt> src = {{1, 1, 1}}, tgt = {};
        Buf bs( 3 ), bt( 3 ), bv( 1 ), bo( 0 );
        MovingLeastSquaresOperator<CudaDevice> op( 0, points( bs, src ), points( bt, tgt ) );
        op.apply( values( bv, {255.0} ), out( bo ) );
    }
    // error convention: DTK_REQUIRE -> DataTransferKitException
    {
        std::vector<Pt> src = {{1, 1, 1}, {2, 2, 2}}, tgt = {{1.5, 1.5, 1.5}};
        Buf bs( 6 ), bt( 3 ), bv( 3 ), bo( 1 );
        MovingLeastSquaresOperator<CudaDevice> op( 0, points( bs, src ), points( bt, tgt ) );
        bool threw = false;
        try
        {
            op.apply( values( bv, {1.0, 2.0, 3.0} ), out( bo ) ); // 3 values for 2 sources
        }
        catch ( DataTransferKitException const & )
        {
            threw = true;
        }
        CHECK( threw );
        threw = false;
        try
        {
            std::vector<Pt> none = {};
            Buf b0( 3 );
            MovingLeastSquaresOperator<CudaDevice> bad( 0, points( b0, none ), points( bt, tgt ) );
        }
        catch ( DataTransferKitException const & )
        {
            threw = true; // DTK_CHECK( !search_tree.empty() )
        }
        CHECK( threw );
    }
    std::printf( "PASS %d\n", g_checks );
    return 0;
}
