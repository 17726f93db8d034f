// The C++ drop-in's multi-rank path: MovingLeastSquaresOperator constructed
// with a communicator of two ranks (here two host threads, each with its own
// CUDA stream on one GPU, exchanging through shared memory; an MPI_Comm
// takes the same path when <mpi.h> is included first).  Each rank holds its
// own sources and targets; its results must equal the one-rank operator over
// the union of the clouds in rank order, and the reference's grid case
// (tstMeshfreeOperators.cpp:226-300: 40x40 sources at z = rank, the target on
// a source) must reproduce its polynomial to 1e-14.  NearestNeighborOperator
// over both ranks must copy the one-rank operator's nearest values exactly.
// No kernel of one rank waits on the other's: the exchange runs on the host
// between the steps.
// Built twice: with the shared-memory communicator below, and with
// -DDTK_FAKE_MPI, where the communicator is MPI_COMM_WORLD of a test
// stand-in for MPI (tests/cpp/fake_mpi.hpp) and the drop-in takes its
// MPI_Comm path.
// Prints "PASS <n>" on success; exits non-zero on the first failure.
#ifdef DTK_FAKE_MPI
#include "fake_mpi.hpp"
#endif
#include <dtk/DTK_MovingLeastSquaresOperator.hpp>
#include <dtk/DTK_NearestNeighborOperator.hpp>

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

using namespace DataTransferKit;
using Pt = std::array<double, 3>;

static std::atomic<int> g_checks{0};
static std::mutex g_print;

#define CHECK( c )                                                                                  \
    do                                                                                              \
    {                                                                                               \
        ++g_checks;                                                                                 \
        if ( !( c ) )                                                                               \
        {                                                                                           \
            std::lock_guard<std::mutex> lock( g_print );                                            \
            std::printf( "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c );                              \
            std::exit( 1 );                                                                         \
        }                                                                                           \
    } while ( 0 )

// Two ranks as two threads: blocks exchanged through shared pointers between
// two barriers.
struct Shared
{
    int n;
    std::mutex m;
    std::condition_variable cv;
    int arrived = 0;
    long generation = 0;
    std::vector<void const *> ptr;
    std::vector<std::vector<int64_t> const *> bytes;
    explicit Shared( int n_ ) : n( n_ ), ptr( n_ ), bytes( n_ ) {}
    void barrier()
    {
        std::unique_lock<std::mutex> lock( m );
        long const g = generation;
        if ( ++arrived == n )
        {
            arrived = 0;
            ++generation;
            cv.notify_all();
        }
        else
            cv.wait( lock, [&] { return generation != g; } );
    }
};

struct ThreadComm
{
    Shared *sh;
    int r;
    int rank() const { return r; }
    int size() const { return sh->n; }
    void allgather( void const *send, int64_t bytes, void *recv ) const
    {
        sh->ptr[r] = send;
        sh->barrier();
        for ( int q = 0; q < sh->n; ++q )
            if ( bytes )
                std::memcpy( static_cast<char *>( recv ) + q * bytes, sh->ptr[q], bytes );
        sh->barrier();
    }
    void alltoallv( void const *send, std::vector<int64_t> const &send_bytes, void *recv,
                    std::vector<int64_t> const &recv_bytes ) const
    {
        sh->ptr[r] = send;
        sh->bytes[r] = &send_bytes;
        sh->barrier();
        char *out = static_cast<char *>( recv );
        for ( int q = 0; q < sh->n; ++q )
        {
            std::vector<int64_t> const &qb = *sh->bytes[q];
            int64_t off = 0;
            for ( int d = 0; d < r; ++d )
                off += qb[d];
            if ( qb[r] != recv_bytes[q] )
            {
                std::printf( "FAIL exchange sizes disagree\n" );
                std::exit( 1 );
            }
            if ( recv_bytes[q] )
                std::memcpy( out, static_cast<char const *>( sh->ptr[q] ) + off, recv_bytes[q] );
            out += recv_bytes[q];
        }
        sh->barrier();
    }
};

#ifdef DTK_FAKE_MPI
using CommT = MPI_Comm;
CommT make_comm( Shared *, int r )
{
    fake_mpi::thread_rank() = r;
    return MPI_COMM_WORLD;
}
MPI_Comm const ONE_RANK = MPI_COMM_SELF;
#else
using CommT = ThreadComm;
CommT make_comm( Shared *sh, int r ) { return ThreadComm{sh, r}; }
int const ONE_RANK = 0; // not a communicator type: one rank
#endif

struct Buf
{
    double *d = nullptr;
    std::size_t n = 0;
    explicit Buf( std::size_t n_ ) : n( n_ ) { cudaMalloc( &d, std::max<std::size_t>( 1, n ) * 8 ); }
    ~Buf() { cudaFree( d ); }
};

DeviceView<double const> points( Buf &b, std::vector<Pt> const &p )
{
    std::vector<double> h( 3 * p.size() );
    for ( std::size_t i = 0; i < p.size(); ++i )
        for ( int d = 0; d < 3; ++d )
            h[3 * i + d] = p[i][d];
    cudaMemcpy( b.d, h.data(), h.size() * 8, cudaMemcpyHostToDevice );
    DeviceView<double const> v;
    v.ptr = b.d;
    v.n0 = p.size();
    v.n1 = 3;
    v.s0 = 3;
    v.s1 = 1;
    return v;
}

DeviceView<double const> values( Buf &b, std::vector<double> const &h )
{
    cudaMemcpy( b.d, h.data(), h.size() * 8, cudaMemcpyHostToDevice );
    DeviceView<double const> v;
    v.ptr = b.d;
    v.n0 = h.size();
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

std::vector<Pt> cloud( int n, unsigned seed, double scale, double shift )
{
    std::mt19937_64 g( seed );
    std::uniform_real_distribution<double> u( 0.0, 1.0 );
    std::vector<Pt> c( n );
    for ( auto &p : c )
        p = {shift + scale * u( g ), u( g ), u( g )};
    return c;
}

double field( Pt const &p ) { return std::sin( 3 * p[0] ) + p[1] * p[2] + 0.5 * p[2]; }

template <typename Op>
void compare_with_union( CommT const &comm, int r, cudaStream_t stream, std::vector<std::vector<Pt>> const &srcs,
                         std::vector<Pt> const &tgt, MlsOptions ext, double tol )
{
    std::vector<Pt> const &src = srcs[r];
    Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
    std::vector<double> sv;
    for ( auto &p : src )
        sv.push_back( field( p ) );
    ext.stream = reinterpret_cast<dtk_stream_t>( stream );
    Op op( comm, points( bs, src ), points( bt, tgt ), ext );
    op.apply( values( bv, sv ), out( bo ) );
    auto y = host( bo );
    // the one-rank operator over the union in rank order
    std::vector<Pt> uni;
    std::vector<double> uv;
    for ( auto const &s : srcs )
        for ( auto &p : s )
        {
            uni.push_back( p );
            uv.push_back( field( p ) );
        }
    Buf us( 3 * uni.size() ), uvb( uni.size() ), uo( tgt.size() );
    Op one( ONE_RANK, points( us, uni ), points( bt, tgt ), ext );
    one.apply( values( uvb, uv ), out( uo ) );
    auto z = host( uo );
    double num = 0.0, den = 0.0;
    for ( std::size_t i = 0; i < tgt.size(); ++i )
    {
        num += ( y[i] - z[i] ) * ( y[i] - z[i] );
        den += z[i] * z[i];
    }
    CHECK( tgt.empty() || std::sqrt( num ) <= tol * std::sqrt( den ) );
}

void rank_main( Shared *sh, int r )
{
    cudaSetDevice( 0 );
    cudaStream_t stream;
    cudaStreamCreateWithFlags( &stream, cudaStreamNonBlocking );
    CommT const comm = make_comm( sh, r );
    using Quad = MovingLeastSquaresOperator<CudaDevice, Wendland<2>, MultivariatePolynomialBasis<Quadratic, 3>>;
    using Lin = MovingLeastSquaresOperator<CudaDevice, Wendland<0>, MultivariatePolynomialBasis<Linear, 3>>;
    {
        // overlapping clouds of unequal sizes; FP64 and mixed forms
        std::vector<std::vector<Pt>> srcs = {cloud( 6000, 11, 1.0, 0.0 ), cloud( 4000, 12, 1.5, 0.0 )};
        std::vector<Pt> tgt = cloud( r == 0 ? 1500 : 900, 20 + r, 1.0, 0.0 );
        MlsOptions ext;
        ext.k = 20;
        compare_with_union<Quad>( comm, r, stream, srcs, tgt, ext, 1e-13 );
        ext.precision = DTK_MIXED;
        compare_with_union<Quad>( comm, r, stream, srcs, tgt, ext, 1e-12 );
    }
    {
        // side-by-side slabs; the reference's default k (basis size)
        std::vector<std::vector<Pt>> srcs = {cloud( 5000, 31, 0.5, 0.0 ), cloud( 5000, 32, 0.5, 0.5 )};
        std::vector<Pt> tgt = cloud( 1000, 40 + r, 0.5, 0.5 * r );
        compare_with_union<Lin>( comm, r, stream, srcs, tgt, MlsOptions{}, 1e-13 );
    }
    {
        // one rank without sources, one without targets
        std::vector<std::vector<Pt>> srcs = {cloud( 3000, 51, 1.0, 0.0 ), {}};
        std::vector<Pt> tgt = r == 0 ? std::vector<Pt>{} : cloud( 700, 52, 1.0, 0.0 );
        MlsOptions ext;
        ext.k = 10;
        compare_with_union<Quad>( comm, r, stream, srcs, tgt, ext, 1e-13 );
    }
    {
        // nearest neighbour over both ranks: exactly the one-rank operator's values
        std::vector<std::vector<Pt>> srcs = {cloud( 5000, 61, 0.5, 0.0 ), cloud( 3000, 62, 0.5, 0.5 )};
        std::vector<Pt> tgt = cloud( 2000, 70 + r, 1.0, 0.0 );
        std::vector<Pt> const &src = srcs[r];
        Buf bs( 3 * src.size() ), bt( 3 * tgt.size() ), bv( src.size() ), bo( tgt.size() );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( field( p ) );
        NearestNeighborOperator<CudaDevice> nn( comm, points( bs, src ), points( bt, tgt ),
                                                reinterpret_cast<dtk_stream_t>( stream ) );
        nn.apply( values( bv, sv ), out( bo ) );
        std::vector<Pt> uni;
        std::vector<double> uv;
        for ( auto const &c : srcs )
            for ( auto &p : c )
            {
                uni.push_back( p );
                uv.push_back( field( p ) );
            }
        Buf us( 3 * uni.size() ), ub( uni.size() ), uo( tgt.size() );
        NearestNeighborOperator<CudaDevice> one( ONE_RANK, points( us, uni ), points( bt, tgt ),
                                                 reinterpret_cast<dtk_stream_t>( stream ) );
        one.apply( values( ub, uv ), out( uo ) );
        CHECK( host( bo ) == host( uo ) );
    }
    {
        // the reference's grid case across the ranks (ties at the k-th neighbour)
        std::vector<Pt> src;
        for ( int i = 0; i < 40; ++i )
            for ( int j = 0; j < 40; ++j )
                src.push_back( {double( i ), double( j ), double( r )} );
        std::vector<Pt> tgt = {{19.0, 19.0, double( r )}};
        auto f = []( Pt const &p ) { return 4 + 2 * p[0] + 3 * p[1] - 2 * p[2]; };
        Buf bs( 3 * src.size() ), bt( 3 ), bv( src.size() ), bo( 1 );
        std::vector<double> sv;
        for ( auto &p : src )
            sv.push_back( f( p ) );
        MlsOptions ext;
        ext.stream = reinterpret_cast<dtk_stream_t>( stream );
        Lin op( comm, points( bs, src ), points( bt, tgt ), ext );
        op.apply( values( bv, sv ), out( bo ) );
        CHECK( std::abs( host( bo )[0] - f( tgt[0] ) ) <= 1e-14 * std::abs( f( tgt[0] ) ) );
    }
    {
        // no sources on any rank: DTK_CHECK( !search_tree.empty() ), on every rank
        Buf bs( 1 ), bt( 3 );
        std::vector<Pt> tgt = {{0.5, 0.5, 0.5}};
        bool threw = false;
        try
        {
            MlsOptions ext;
            ext.stream = reinterpret_cast<dtk_stream_t>( stream );
            Lin op( comm, points( bs, {} ), points( bt, tgt ), ext );
        }
        catch ( DataTransferKitException const & )
        {
            threw = true;
        }
        CHECK( threw );
    }
    cudaStreamDestroy( stream );
}

int main()
{
#ifdef DTK_FAKE_MPI
    fake_mpi::init( 2 );
#endif
    Shared sh( 2 );
    std::thread a( rank_main, &sh, 0 ), b( rank_main, &sh, 1 );
    a.join();
    b.join();
    std::printf( "PASS %d\n", g_checks.load() );
    return 0;
}
