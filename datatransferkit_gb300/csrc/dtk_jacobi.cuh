// Symmetric Jacobi eigen-solver pieces shared by the mixed setup and the
// adjoint kernels (one thread per matrix, state behind accessors so that it
// can live in shared memory or registers).
#pragma once

#include "dtk_common.cuh"

namespace dtk
{

template <int M>
__host__ __device__ constexpr int ut( int i, int j )
{
    // upper-triangle index of (min(i,j), max(i,j)), row-major
    return i <= j ? i * M - i * ( i - 1 ) / 2 + ( j - i ) : j * M - j * ( j - 1 ) / 2 + ( i - j );
}

// Round-robin ("parallel") ordering of the M(M-1)/2 pairs: with n = M (M
// even) or M + 1 (odd, one dummy player), n - 1 rounds; in round r player
// n - 1 meets r and player (r + i) mod (n - 1) meets (r - i) mod (n - 1) for
// i = 1 .. n/2 - 1.  Every pair meets once per sweep; the pairs of a round
// are disjoint.
template <int M>
struct RoundRobin
{
    static constexpr int N = M % 2 ? M + 1 : M;
    static constexpr int R = N - 1;      // rounds
    static constexpr int P = M / 2;      // real pairs per round
    // pair i of round r (i = 0 .. N/2 - 1), ordered a < b; the dummy
    // player (index M when M is odd) marks a pair to skip
    __device__ __forceinline__ static void pair( int r, int i, int &a, int &b )
    {
        int x = i == 0 ? N - 1 : ( r + i ) % ( N - 1 );
        int y = i == 0 ? r : ( r - i + N - 1 ) % ( N - 1 );
        a = x < y ? x : y;
        b = x < y ? y : x;
    }
};

// Rutishauser rotation parameters for one pair: t = tan(theta) (smaller
// root), c = cos, s = sin.
template <class T>
__device__ __forceinline__ void rotation( T app, T aqq, T apq, T &c, T &s, T &t )
{
    T const d = aqq - app;
    T const h = T( 0.5 ) * fabs( d );
    T tt = apq / ( h + sqrt( fma( h, h, apq * apq ) ) );
    t = d < T( 0 ) ? -tt : tt;
    c = T( 1 ) / sqrt( fma( t, t, T( 1 ) ) );
    s = t * c;
}

template <int M, class T, class AAcc, class VAcc>
__device__ int jacobi_sweep_rr( AAcc &a, VAcc &v, T skip );

// One parallel-ordered sweep of the symmetric Jacobi method on the upper
// triangle A (accessor a(u)), accumulating the eigenvectors in V (accessor
// v(r, c)).  Each round computes the M/2 rotation parameters independently
// (their dependent chains overlap) and applies A <- J^T A J for the
// block-diagonal J of the round, block by block, then V <- V J.
// Returns the number of rotations performed.
template <int M, class T, class AAcc, class VAcc>
__device__ int jacobi_sweep( AAcc &&a, VAcc &&v, T skip )
{
    if constexpr ( M < 2 )
        return 0;
    else
        return jacobi_sweep_rr<M, T>( a, v, skip );
}

template <int M, class T, class AAcc, class VAcc>
__device__ int jacobi_sweep_rr( AAcc &a, VAcc &v, T skip )
{
    using RR = RoundRobin<M>;
    constexpr int NP = RR::P;
    int done = 0;
    for ( int r = 0; r < RR::R; ++r )
    {
        int P[NP], Q[NP];
        T C[NP], S[NP], Tn[NP];
        bool on[NP];
        {
            // the real pairs of round r (odd M: the one with the dummy is dropped)
            int k = 0;
#pragma unroll
            for ( int i = 0; i < RR::N / 2; ++i )
            {
                int x, y;
                RR::pair( r, i, x, y );
                if ( y < M && k < NP )
                {
                    P[k] = x;
                    Q[k] = y;
                    ++k;
                }
            }
        }
#pragma unroll
        for ( int k = 0; k < NP; ++k )
        {
            T const app = a( ut<M>( P[k], P[k] ) ), aqq = a( ut<M>( Q[k], Q[k] ) );
            T const apq = a( ut<M>( P[k], Q[k] ) );
            // a pair already negligible (a_pq^2 <= skip^2 |a_pp a_qq|) is
            // not rotated; the branch skips its parameter chain whenever no
            // lane of the warp needs it
            on[k] = !( apq * apq <= skip * skip * fabs( app * aqq ) );
            C[k] = T( 1 );
            S[k] = T( 0 );
            Tn[k] = T( 0 );
            if ( on[k] )
                rotation<T>( app, aqq, apq, C[k], S[k], Tn[k] );
            done += on[k];
        }
        // off-diagonal 2x2 blocks between pairs k < l
#pragma unroll
        for ( int k = 0; k < NP; ++k )
#pragma unroll
            for ( int l = k + 1; l < NP; ++l )
            {
                if ( !( on[k] || on[l] ) )
                    continue;
                T const a11 = a( ut<M>( P[k], P[l] ) ), a12 = a( ut<M>( P[k], Q[l] ) );
                T const a21 = a( ut<M>( Q[k], P[l] ) ), a22 = a( ut<M>( Q[k], Q[l] ) );
                // rows p_k, q_k by J_k^T
                T const b11 = C[k] * a11 - S[k] * a21, b21 = S[k] * a11 + C[k] * a21;
                T const b12 = C[k] * a12 - S[k] * a22, b22 = S[k] * a12 + C[k] * a22;
                // columns p_l, q_l by J_l
                a( ut<M>( P[k], P[l] ) ) = C[l] * b11 - S[l] * b12;
                a( ut<M>( P[k], Q[l] ) ) = S[l] * b11 + C[l] * b12;
                a( ut<M>( Q[k], P[l] ) ) = C[l] * b21 - S[l] * b22;
                a( ut<M>( Q[k], Q[l] ) ) = S[l] * b21 + C[l] * b22;
            }
        // diagonal blocks (Rutishauser) and eigenvectors
#pragma unroll
        for ( int k = 0; k < NP; ++k )
        {
            if ( !on[k] )
                continue;
            T const apq = a( ut<M>( P[k], Q[k] ) );
            a( ut<M>( P[k], P[k] ) ) = a( ut<M>( P[k], P[k] ) ) - Tn[k] * apq;
            a( ut<M>( Q[k], Q[k] ) ) = a( ut<M>( Q[k], Q[k] ) ) + Tn[k] * apq;
            a( ut<M>( P[k], Q[k] ) ) = T( 0 );
#pragma unroll
            for ( int i = 0; i < M; ++i )
            {
                T const vp = v( i, P[k] ), vq = v( i, Q[k] );
                v( i, P[k] ) = C[k] * vp - S[k] * vq;
                v( i, Q[k] ) = S[k] * vp + C[k] * vq;
            }
        }
        if constexpr ( M % 2 )
        {
            // odd M: one index idles each round; its row/column with the
            // rotated pairs still needs the one-sided updates
            int idle = 0;
            {
                unsigned used = 0;
#pragma unroll
                for ( int k = 0; k < NP; ++k )
                    used |= ( 1u << P[k] ) | ( 1u << Q[k] );
                while ( used & ( 1u << idle ) )
                    ++idle;
            }
#pragma unroll
            for ( int k = 0; k < NP; ++k )
            {
                if ( !on[k] )
                    continue;
                T const x = a( ut<M>( idle, P[k] ) ), y = a( ut<M>( idle, Q[k] ) );
                a( ut<M>( idle, P[k] ) ) = C[k] * x - S[k] * y;
                a( ut<M>( idle, Q[k] ) ) = S[k] * x + C[k] * y;
            }
        }
    }
    return done;
}


} // namespace dtk
