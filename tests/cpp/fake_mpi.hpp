// A stand-in for the few MPI calls the drop-in's MPI_Comm path makes
// (MPI_Comm_rank, MPI_Comm_size, MPI_Allgather, MPI_Alltoallv on MPI_BYTE),
// for testing that path without an MPI library: the ranks are host threads
// of one process, MPI_COMM_WORLD spans them and MPI_COMM_SELF is each one
// alone.  Test code only; include before the drop-in headers.
#ifndef DTK_TEST_FAKE_MPI_HPP
#define DTK_TEST_FAKE_MPI_HPP

#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#define MPI_VERSION 3
typedef int MPI_Comm;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 91
#define MPI_COMM_SELF 92
#define MPI_BYTE 1

namespace fake_mpi
{
struct World
{
    int n = 1;
    std::mutex m;
    std::condition_variable cv;
    int arrived = 0;
    long generation = 0;
    std::vector<void const *> ptr;
    std::vector<int const *> counts, displs;
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
inline World &world()
{
    static World w;
    return w;
}
inline int &thread_rank()
{
    thread_local int r = 0;
    return r;
}
inline void init( int n )
{
    World &w = world();
    w.n = n;
    w.ptr.assign( n, nullptr );
    w.counts.assign( n, nullptr );
    w.displs.assign( n, nullptr );
}
} // namespace fake_mpi

inline int MPI_Comm_rank( MPI_Comm c, int *r )
{
    *r = c == MPI_COMM_SELF ? 0 : fake_mpi::thread_rank();
    return 0;
}
inline int MPI_Comm_size( MPI_Comm c, int *s )
{
    *s = c == MPI_COMM_SELF ? 1 : fake_mpi::world().n;
    return 0;
}
inline int MPI_Allgather( void *send, int sc, MPI_Datatype, void *recv, int rc, MPI_Datatype, MPI_Comm c )
{
    if ( c == MPI_COMM_SELF )
    {
        std::memcpy( recv, send, sc );
        return 0;
    }
    fake_mpi::World &w = fake_mpi::world();
    int const r = fake_mpi::thread_rank();
    w.ptr[r] = send;
    w.barrier();
    for ( int q = 0; q < w.n; ++q )
        if ( rc )
            std::memcpy( static_cast<char *>( recv ) + (std::size_t)q * rc, w.ptr[q], rc );
    w.barrier();
    return 0;
}
inline int MPI_Alltoallv( void *send, int const *sc, int const *sd, MPI_Datatype, void *recv, int const *rc,
                          int const *rd, MPI_Datatype, MPI_Comm c )
{
    fake_mpi::World &w = fake_mpi::world();
    if ( c == MPI_COMM_SELF )
    {
        std::memcpy( static_cast<char *>( recv ) + rd[0], static_cast<char *>( send ) + sd[0], sc[0] );
        return 0;
    }
    int const r = fake_mpi::thread_rank();
    w.ptr[r] = send;
    w.counts[r] = sc;
    w.displs[r] = sd;
    w.barrier();
    for ( int q = 0; q < w.n; ++q )
        if ( rc[q] )
            std::memcpy( static_cast<char *>( recv ) + rd[q], static_cast<char const *>( w.ptr[q] ) + w.displs[q][r],
                         rc[q] );
    w.barrier();
    return 0;
}

#endif
