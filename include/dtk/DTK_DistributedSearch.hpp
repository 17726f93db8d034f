/*
 * Multi-rank host side of the drop-in operators: the distributed kNN search
 * and the value fetch of DataTransferKit's MPI operators, over the C ABI of
 * dtk_gb300.h and a communicator's exchange operations.
 *
 * Mirrors (paths inside the DataTransferKit project):
 *   ArborX::DistributedTree + kNN query   DTK_MovingLeastSquaresOperator_def.hpp:47-60
 *   fetch of the neighbours' coordinates  DTK_MovingLeastSquaresOperator_def.hpp:66-67
 *   fetch of the source values in apply   DTK_MovingLeastSquaresOperator_def.hpp:133-134
 *   NearestNeighborOperatorImpl::fetch    DTK_DetailsNearestNeighborOperatorImpl.hpp:47-192
 *
 * A source's global index is its rank's offset (the sources of the lower
 * ranks) plus its local index; rows are the min(k, N) nearest sources of all
 * ranks by (d2, global index), so a row equals the one-rank operator's over
 * the rank-ordered union of the clouds.  Steps: the ranks share their source
 * counts and boxes; each searches its own sources; the local k-th d2 bounds a
 * target, which is sent to the ranks whose box lies within the bound (the
 * rounded box distance never exceeds the rounded d2 of a point in the box);
 * the owners answer with their k nearest; the rows of the targets that asked
 * merge by (d2, global index).  The operator is built from the rows with the
 * values laid out as [this rank's n_loc sources | the n_remote distinct other
 * sources its rows use], and the fetch plan is exchanged once: apply copies
 * the rank's own values on the device and moves only the remote ones.
 *
 * Communicators: any type with rank(), size(), allgather(send, bytes, recv)
 * (recv holds size() blocks of `bytes`) and alltoallv(send, send_bytes,
 * recv, recv_bytes) (per-rank byte counts, blocks packed in rank order), and
 * MPI_Comm when <mpi.h> is included before this header.
 */
#ifndef DTK_GB300_DISTRIBUTED_SEARCH_HPP
#define DTK_GB300_DISTRIBUTED_SEARCH_HPP

#include "../dtk_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace DataTransferKit
{
namespace Details
{

// ---------------------------------------------------------------------------
// Communicators
// ---------------------------------------------------------------------------
template <typename Comm, typename = void>
struct CommTraits
{
    static constexpr bool exchange = false;
    static int size( Comm const & ) { return 1; }
};

template <typename Comm>
struct CommTraits<Comm, std::void_t<decltype( std::declval<Comm const &>().rank() ),
                                    decltype( std::declval<Comm const &>().size() ),
                                    decltype( std::declval<Comm const &>().allgather( nullptr, 0, nullptr ) ),
                                    decltype( std::declval<Comm const &>().alltoallv(
                                        nullptr, std::declval<std::vector<int64_t> const &>(), nullptr,
                                        std::declval<std::vector<int64_t> const &>() ) )>>
{
    static constexpr bool exchange = true;
    static int rank( Comm const &c ) { return (int)c.rank(); }
    static int size( Comm const &c ) { return (int)c.size(); }
    static void allgather( Comm const &c, void const *send, int64_t bytes, void *recv )
    {
        c.allgather( send, bytes, recv );
    }
    static void alltoallv( Comm const &c, void const *send, std::vector<int64_t> const &send_bytes, void *recv,
                           std::vector<int64_t> const &recv_bytes )
    {
        c.alltoallv( send, send_bytes, recv, recv_bytes );
    }
};

#ifdef MPI_VERSION
template <>
struct CommTraits<MPI_Comm, void>
{
    static constexpr bool exchange = true;
    static int rank( MPI_Comm c )
    {
        int r = 0;
        MPI_Comm_rank( c, &r );
        return r;
    }
    static int size( MPI_Comm c )
    {
        int s = 1;
        MPI_Comm_size( c, &s );
        return s;
    }
    // MPI counts and displacements are int: larger exchanges are refused
    static int count( int64_t v )
    {
        if ( v < 0 || v > INT_MAX )
            throw std::length_error( "DTK distributed: an exchange exceeds MPI's int byte counts" );
        return (int)v;
    }
    static void allgather( MPI_Comm c, void const *send, int64_t bytes, void *recv )
    {
        MPI_Allgather( const_cast<void *>( send ), count( bytes ), MPI_BYTE, recv, count( bytes ), MPI_BYTE, c );
    }
    static void alltoallv( MPI_Comm c, void const *send, std::vector<int64_t> const &send_bytes, void *recv,
                           std::vector<int64_t> const &recv_bytes )
    {
        int const n = (int)send_bytes.size();
        std::vector<int> sc( n ), sd( n ), rc( n ), rd( n );
        int64_t s = 0, t = 0;
        for ( int r = 0; r < n; ++r )
        {
            sc[r] = count( send_bytes[r] );
            sd[r] = count( s );
            s += sc[r];
            rc[r] = count( recv_bytes[r] );
            rd[r] = count( t );
            t += rc[r];
        }
        MPI_Alltoallv( const_cast<void *>( send ), sc.data(), sd.data(), MPI_BYTE, recv, rc.data(), rd.data(),
                       MPI_BYTE, c );
    }
};
#endif

// ---------------------------------------------------------------------------
// Device buffers on a stream (stream-ordered allocation)
// ---------------------------------------------------------------------------
inline void cuda_check( cudaError_t e, char const *what )
{
    if ( e != cudaSuccess )
        throw std::runtime_error( std::string( "DTK distributed: " ) + what + ": " + cudaGetErrorString( e ) );
}

inline void dtk_check( dtk_status s )
{
    if ( s != DTK_OK )
        throw std::runtime_error( std::string( dtk_status_string( s ) ) + ": " + dtk_last_error() );
}

template <typename T>
class DevArray
{
  public:
    DevArray() = default;
    DevArray( std::size_t n, cudaStream_t s ) { resize( n, s ); }
    DevArray( DevArray const & ) = delete;
    DevArray &operator=( DevArray const & ) = delete;
    ~DevArray() { release(); }
    void resize( std::size_t n, cudaStream_t s )
    {
        release();
        _s = s;
        _n = n;
        if ( n )
            cuda_check( cudaMallocAsync( reinterpret_cast<void **>( &_p ), n * sizeof( T ), s ), "allocation" );
    }
    void release()
    {
        if ( _p )
            cudaFreeAsync( _p, _s );
        _p = nullptr;
        _n = 0;
    }
    T *get() const { return _p; }
    std::size_t size() const { return _n; }
    void upload( T const *h, std::size_t n, std::size_t at = 0 ) const
    {
        if ( n )
            cuda_check( cudaMemcpyAsync( _p + at, h, n * sizeof( T ), cudaMemcpyHostToDevice, _s ), "upload" );
    }
    void download( T *h, std::size_t n, std::size_t at = 0 ) const
    {
        if ( n )
            cuda_check( cudaMemcpyAsync( h, _p + at, n * sizeof( T ), cudaMemcpyDeviceToHost, _s ), "download" );
    }

  private:
    T *_p = nullptr;
    std::size_t _n = 0;
    cudaStream_t _s = nullptr;
};

struct PointsArg
{
    double const *data;
    int64_t n, ps, ds;
};

// Rounded squared distance of t to the box [lo, hi] (never above the rounded
// d2 of a point inside: rounding is monotone).
inline double box_d2( double const *t, double const *box )
{
    double acc[3];
    for ( int d = 0; d < 3; ++d )
    {
        double const g = std::max( { box[d] - t[d], t[d] - box[3 + d], 0.0 } );
        acc[d] = g * g;
    }
    return ( acc[0] + acc[1] ) + acc[2];
}

// The rank's part of a distributed operator: the handle over its rows and the
// plan of the value fetch.
struct DistributedOperator
{
    std::shared_ptr<struct dtk_mls_s> handle;
    cudaStream_t stream = nullptr;
    int64_t n_loc = 0, n_remote = 0, n_tgt = 0;
    int row = 0;
    std::vector<int64_t> send_counts, recv_counts; // values a rank sends to / receives from each rank
    DevArray<int32_t> send_index;                  // this rank's values the others asked for, by asker
    DevArray<double> fetched, send_values;         // [own | remote] values; the values sent
    std::vector<double> send_host, recv_host;
    std::vector<int64_t> global_rows;              // (n_tgt x row) global source index of every entry
    DevArray<int32_t> slots;                       // the entries' positions in `fetched` (nearest neighbour)
    int64_t queries_sent = 0;
};

// The distributed setup (collective).  k: neighbours per target (<= 32).
// With `mls`, the MLS operator of the rows; without, only the rows' positions
// in the fetched values (the nearest-neighbour operator, k = 1).
template <typename Comm>
std::unique_ptr<DistributedOperator> distributed_setup( Comm const &comm, dtk_mls_options opts, PointsArg src,
                                                        PointsArg tgt, int k, cudaStream_t stream, bool mls = true )
{
    using T = CommTraits<Comm>;
    int const world = T::size( comm ), rank = T::rank( comm );
    auto op = std::make_unique<DistributedOperator>();
    op->stream = stream;
    int64_t const n_loc = src.n, n_tgt = tgt.n;
    op->n_loc = n_loc;
    op->n_tgt = n_tgt;
    dtk_stream_t const ds = reinterpret_cast<dtk_stream_t>( stream );

    // 1. counts and boxes of every rank's sources
    std::vector<int64_t> counts( world );
    T::allgather( comm, &n_loc, sizeof( int64_t ), counts.data() );
    std::vector<int64_t> first( world, 0 );
    for ( int r = 1; r < world; ++r )
        first[r] = first[r - 1] + counts[r - 1];
    int64_t const total = first[world - 1] + counts[world - 1];
    if ( total == 0 ) // DTK_CHECK( !search_tree.empty() )
        throw std::invalid_argument( "DTK_CHECK( !search_tree.empty() ): the distributed source cloud is empty" );
    int const row = (int)std::min<int64_t>( k, total );
    op->row = row;
    double box[6];
    dtk_check( dtk_points_bounds( src.data, n_loc, src.ps, src.ds, box, ds ) );
    std::vector<double> boxes( 6 * world );
    T::allgather( comm, box, sizeof( box ), boxes.data() );

    // host copies of the points (the routing, the answers' coordinates)
    auto host_points = [&]( PointsArg p ) {
        std::vector<double> h( 3 * p.n );
        if ( p.n )
        {
            DevArray<double> packed( 3 * p.n, stream );
            dtk_check( dtk_points_pack( p.data, p.n, p.ps, p.ds, packed.get(), ds ) );
            packed.download( h.data(), h.size() );
            cuda_check( cudaStreamSynchronize( stream ), "synchronize" );
        }
        return h;
    };
    std::vector<double> const src_h = host_points( src ), tgt_h = host_points( tgt );

    // 2. local rows and their bounds
    int const row_l = (int)std::min<int64_t>( row, n_loc );
    DevArray<int32_t> idx_l( n_tgt * (int64_t)row_l, stream );
    std::vector<int32_t> idx_lh( idx_l.size() );
    std::vector<double> kth( n_tgt, std::numeric_limits<double>::infinity() );
    if ( row_l > 0 && n_tgt > 0 )
    {
        DevArray<double> d2_l( idx_l.size(), stream );
        dtk_check( dtk_knn_search_d2( src.data, n_loc, src.ps, src.ds, tgt.data, n_tgt, tgt.ps, tgt.ds, row,
                                      idx_l.get(), d2_l.get(), ds ) );
        idx_l.download( idx_lh.data(), idx_lh.size() );
        if ( row_l == row )
            cuda_check( cudaMemcpy2DAsync( kth.data(), sizeof( double ), d2_l.get() + ( row_l - 1 ),
                                           row_l * sizeof( double ), sizeof( double ), n_tgt,
                                           cudaMemcpyDeviceToHost, stream ),
                        "bounds" );
        cuda_check( cudaStreamSynchronize( stream ), "synchronize" );
    }

    // 3. the queries, grouped by destination
    std::vector<std::vector<int64_t>> sel( world );
    for ( int q = 0; q < world; ++q )
    {
        if ( q == rank || counts[q] == 0 )
            continue;
        for ( int64_t t = 0; t < n_tgt; ++t )
            // a relative margin of 2^-40 covers how the host compiler may round
            // (a contracted multiply-add); a query too many costs only time
            if ( box_d2( &tgt_h[3 * t], &boxes[6 * q] ) * ( 1.0 - 0x1p-40 ) <= kth[t] )
                sel[q].push_back( t );
    }
    std::vector<int64_t> send_n( world ), recv_n( world );
    for ( int q = 0; q < world; ++q )
        send_n[q] = (int64_t)sel[q].size();
    std::vector<int64_t> eight( world, sizeof( int64_t ) );
    T::alltoallv( comm, send_n.data(), eight, recv_n.data(), eight );
    std::vector<double> queries;
    for ( int q = 0; q < world; ++q )
        for ( int64_t t : sel[q] )
            queries.insert( queries.end(), &tgt_h[3 * t], &tgt_h[3 * t + 3] );
    int64_t const n_asked = std::accumulate( recv_n.begin(), recv_n.end(), int64_t( 0 ) );
    std::vector<double> asked( 3 * n_asked );
    {
        std::vector<int64_t> sb( world ), rb( world );
        for ( int q = 0; q < world; ++q )
        {
            sb[q] = 24 * send_n[q];
            rb[q] = 24 * recv_n[q];
        }
        T::alltoallv( comm, queries.data(), sb, asked.data(), rb );
    }
    op->queries_sent = (int64_t)queries.size() / 3;

    // 4. this rank's answers: (d2, x, y, z) and the global index per entry
    int const row_o = (int)std::min<int64_t>( row, n_loc );
    std::vector<double> answer( 4 * n_asked * row_o );
    std::vector<int64_t> answer_gid( n_asked * row_o );
    if ( n_asked > 0 && row_o > 0 )
    {
        DevArray<double> asked_d( 3 * n_asked, stream ), d2_o( n_asked * row_o, stream );
        DevArray<int32_t> idx_o( n_asked * row_o, stream );
        asked_d.upload( asked.data(), asked.size() );
        dtk_check( dtk_knn_search_d2( src.data, n_loc, src.ps, src.ds, asked_d.get(), n_asked, 3, 1, row,
                                      idx_o.get(), d2_o.get(), ds ) );
        std::vector<int32_t> io( idx_o.size() );
        std::vector<double> dd( d2_o.size() );
        idx_o.download( io.data(), io.size() );
        d2_o.download( dd.data(), dd.size() );
        cuda_check( cudaStreamSynchronize( stream ), "synchronize" );
        for ( std::size_t e = 0; e < io.size(); ++e )
        {
            answer[4 * e] = dd[e];
            std::memcpy( &answer[4 * e + 1], &src_h[3 * (int64_t)io[e]], 3 * sizeof( double ) );
            answer_gid[e] = first[rank] + io[e];
        }
    }
    std::vector<int64_t> back_send( world ), back_recv( world ), per_q( world );
    for ( int q = 0; q < world; ++q )
    {
        per_q[q] = std::min<int64_t>( row, counts[q] );
        back_send[q] = recv_n[q] * row_o;
        back_recv[q] = send_n[q] * per_q[q];
    }
    int64_t const n_back = std::accumulate( back_recv.begin(), back_recv.end(), int64_t( 0 ) );
    std::vector<double> answers( 4 * n_back );
    std::vector<int64_t> answers_gid( n_back );
    {
        std::vector<int64_t> sb( world ), rb( world ), sg( world ), rg( world );
        for ( int q = 0; q < world; ++q )
        {
            sb[q] = 32 * back_send[q];
            rb[q] = 32 * back_recv[q];
            sg[q] = 8 * back_send[q];
            rg[q] = 8 * back_recv[q];
        }
        T::alltoallv( comm, answer.data(), sb, answers.data(), rb );
        T::alltoallv( comm, answer_gid.data(), sg, answers_gid.data(), rg );
    }

    // 5. merge the rows of the targets that asked: (d2, global index), first `row`
    struct Cand
    {
        double d2;
        int64_t gid;
        double x, y, z;
    };
    std::vector<std::vector<Cand>> cand( n_tgt );
    std::vector<char> touched( n_tgt, 0 );
    {
        int64_t at = 0;
        for ( int q = 0; q < world; ++q )
            for ( int64_t t : sel[q] )
            {
                touched[t] = 1;
                for ( int64_t j = 0; j < per_q[q]; ++j, ++at )
                    cand[t].push_back( {answers[4 * at], answers_gid[at], answers[4 * at + 1], answers[4 * at + 2],
                                        answers[4 * at + 3]} );
            }
    }
    if ( row_l < row )
        for ( int64_t t = 0; t < n_tgt; ++t )
            if ( !touched[t] )
                throw std::logic_error( "DTK distributed: a short row asked no other rank" );
    // the local rows of the touched targets again, with the search's own d2
    // (the search is exact, so the rows are the ones found above)
    std::vector<int64_t> tlist;
    for ( int64_t t = 0; t < n_tgt; ++t )
        if ( touched[t] )
            tlist.push_back( t );
    std::vector<int32_t> tidx( tlist.size() * row_l );
    std::vector<double> td2( tidx.size() );
    if ( row_l > 0 && !tlist.empty() )
    {
        std::vector<double> tp( 3 * tlist.size() );
        for ( std::size_t i = 0; i < tlist.size(); ++i )
            std::memcpy( &tp[3 * i], &tgt_h[3 * tlist[i]], 3 * sizeof( double ) );
        DevArray<double> tp_d( tp.size(), stream ), td2_d( td2.size(), stream );
        DevArray<int32_t> tidx_d( tidx.size(), stream );
        tp_d.upload( tp.data(), tp.size() );
        dtk_check( dtk_knn_search_d2( src.data, n_loc, src.ps, src.ds, tp_d.get(), (int64_t)tlist.size(), 3, 1, row,
                                      tidx_d.get(), td2_d.get(), ds ) );
        tidx_d.download( tidx.data(), tidx.size() );
        td2_d.download( td2.data(), td2.size() );
        cuda_check( cudaStreamSynchronize( stream ), "synchronize" );
    }
    for ( std::size_t i = 0; i < tlist.size(); ++i )
        for ( int j = 0; j < row_l; ++j )
        {
            int64_t const li = tidx[i * row_l + j];
            double const *p = &src_h[3 * li];
            cand[tlist[i]].push_back( {td2[i * row_l + j], first[rank] + li, p[0], p[1], p[2]} );
        }
    std::vector<int64_t> grows( n_tgt * (int64_t)row ); // global index of every entry
    std::vector<double> gxyz;                           // coordinates of the touched rows' remote entries
    for ( int64_t t = 0; t < n_tgt; ++t )
    {
        if ( !touched[t] )
        {
            for ( int j = 0; j < row; ++j )
                grows[t * row + j] = first[rank] + idx_lh[t * row_l + j];
            continue;
        }
        auto &c = cand[t];
        std::sort( c.begin(), c.end(), []( Cand const &u, Cand const &v ) {
            return u.d2 < v.d2 || ( u.d2 == v.d2 && u.gid < v.gid );
        } );
        if ( (int64_t)c.size() < row )
            throw std::logic_error( "DTK distributed: a row came back short" );
        for ( int j = 0; j < row; ++j )
            grows[t * row + j] = c[j].gid;
    }
    // the distinct remote sources, ascending (so grouped by owner), and their coordinates
    std::vector<int64_t> remote;
    for ( int64_t g : grows )
        if ( g < first[rank] || g >= first[rank] + n_loc )
            remote.push_back( g );
    std::sort( remote.begin(), remote.end() );
    remote.erase( std::unique( remote.begin(), remote.end() ), remote.end() );
    op->n_remote = (int64_t)remote.size();
    std::vector<double> remote_xyz( 3 * remote.size() );
    for ( int64_t t = 0; t < n_tgt; ++t )
        if ( touched[t] )
            for ( int j = 0; j < row; ++j )
            {
                Cand const &c = cand[t][j];
                if ( c.gid < first[rank] || c.gid >= first[rank] + n_loc )
                {
                    auto const slot = std::lower_bound( remote.begin(), remote.end(), c.gid ) - remote.begin();
                    remote_xyz[3 * slot] = c.x;
                    remote_xyz[3 * slot + 1] = c.y;
                    remote_xyz[3 * slot + 2] = c.z;
                }
            }
    // entries as positions in the fetched values [own | remote]
    std::vector<int32_t> slots( grows.size() );
    for ( std::size_t e = 0; e < grows.size(); ++e )
    {
        int64_t const g = grows[e];
        slots[e] = ( g >= first[rank] && g < first[rank] + n_loc )
                       ? (int32_t)( g - first[rank] )
                       : (int32_t)( n_loc + ( std::lower_bound( remote.begin(), remote.end(), g ) - remote.begin() ) );
    }
    op->global_rows = std::move( grows );

    // 6. the operator of the rows
    int64_t const nnz = (int64_t)slots.size();
    op->slots.resize( nnz, stream );
    op->slots.upload( slots.data(), slots.size() );
    if ( mls )
    {
        DevArray<double> extra_d( remote_xyz.size(), stream ), nb_d( 3 * nnz, stream );
        extra_d.upload( remote_xyz.data(), remote_xyz.size() );
        dtk_check( dtk_gather_points( src.data, n_loc, src.ps, src.ds, extra_d.get(), op->n_remote,
                                      op->slots.get(), nnz, nb_d.get(), ds ) );
        opts.comm_size = 1;
        dtk_mls_handle h = nullptr;
        dtk_check( dtk_mls_create_from_neighbors( &opts, tgt.data, n_tgt, tgt.ps, tgt.ds, row, nb_d.get(),
                                                  op->slots.get(), n_loc + op->n_remote, ds, &h ) );
        op->handle.reset( h, []( dtk_mls_handle p ) { dtk_mls_destroy( p ); } );
    }

    // 7. the fetch plan: each owner learns which of its values to send, in
    //    the order asked (remote is ascending, so grouped by owner)
    op->recv_counts.assign( world, 0 );
    std::vector<int32_t> want;
    for ( int64_t g : remote )
    {
        // the last rank whose first index is <= g (an empty rank shares its
        // first index with the next one, so it is never the last)
        int const q = (int)( std::upper_bound( first.begin(), first.end(), g ) - first.begin() ) - 1;
        ++op->recv_counts[q];
        want.push_back( (int32_t)( g - first[q] ) );
    }
    op->send_counts.assign( world, 0 );
    T::alltoallv( comm, op->recv_counts.data(), eight, op->send_counts.data(), eight );
    int64_t const n_send = std::accumulate( op->send_counts.begin(), op->send_counts.end(), int64_t( 0 ) );
    std::vector<int32_t> send_index( n_send );
    {
        std::vector<int64_t> sb( world ), rb( world );
        for ( int q = 0; q < world; ++q )
        {
            sb[q] = 4 * op->recv_counts[q];
            rb[q] = 4 * op->send_counts[q];
        }
        T::alltoallv( comm, want.data(), sb, send_index.data(), rb );
    }
    op->send_index.resize( n_send, stream );
    op->send_index.upload( send_index.data(), send_index.size() );
    op->fetched.resize( n_loc + op->n_remote, stream );
    op->send_values.resize( n_send, stream );
    op->send_host.resize( n_send );
    op->recv_host.resize( op->n_remote );
    cuda_check( cudaStreamSynchronize( stream ), "synchronize" );
    return op;
}

// The value fetch (collective): op.fetched = [this rank's values | the
// remote values its rows use]; this rank's values stay on the device.
template <typename Comm>
void distributed_fetch( Comm const &comm, DistributedOperator &op, double const *source_values )
{
    using T = CommTraits<Comm>;
    int const world = T::size( comm );
    dtk_stream_t const ds = reinterpret_cast<dtk_stream_t>( op.stream );
    if ( op.n_loc )
        cuda_check( cudaMemcpyAsync( op.fetched.get(), source_values, op.n_loc * sizeof( double ),
                                     cudaMemcpyDeviceToDevice, op.stream ),
                    "own values" );
    if ( op.send_index.size() )
    {
        dtk_check( dtk_gather_values( source_values, op.n_loc, op.send_index.get(), (int64_t)op.send_index.size(),
                                      op.send_values.get(), ds ) );
        op.send_values.download( op.send_host.data(), op.send_host.size() );
    }
    cuda_check( cudaStreamSynchronize( op.stream ), "synchronize" );
    std::vector<int64_t> sb( world ), rb( world );
    for ( int q = 0; q < world; ++q )
    {
        sb[q] = 8 * op.send_counts[q];
        rb[q] = 8 * op.recv_counts[q];
    }
    T::alltoallv( comm, op.send_host.data(), sb, op.recv_host.data(), rb );
    op.fetched.upload( op.recv_host.data(), op.recv_host.size(), op.n_loc );
}

// The distributed MLS apply (collective): target_values = the rows'
// transfer of all ranks' source values.
template <typename Comm>
void distributed_apply( Comm const &comm, DistributedOperator &op, double const *source_values,
                        double *target_values )
{
    distributed_fetch( comm, op, source_values );
    dtk_check( dtk_mls_apply( op.handle.get(), op.fetched.get(), op.n_loc + op.n_remote, target_values, op.n_tgt,
                              reinterpret_cast<dtk_stream_t>( op.stream ) ) );
}

// The distributed nearest-neighbour apply (collective): every target takes
// the value of its nearest source on any rank.
template <typename Comm>
void distributed_apply_nearest( Comm const &comm, DistributedOperator &op, double const *source_values,
                                double *target_values )
{
    distributed_fetch( comm, op, source_values );
    dtk_check( dtk_gather_values( op.fetched.get(), op.n_loc + op.n_remote, op.slots.get(), op.n_tgt,
                                  target_values, reinterpret_cast<dtk_stream_t>( op.stream ) ) );
}

} // namespace Details
} // namespace DataTransferKit

#endif
