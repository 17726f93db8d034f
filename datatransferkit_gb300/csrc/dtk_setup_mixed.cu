// Fused MLS setup, mixed FP32/FP64 form (sm_103a).
//
// Same stages as the FP64 form (DTK_DetailsMovingLeastSquaresOperatorImpl.hpp
// :72-336 after the search), one thread per target, but:
//   * centring and scaling by the support radius: x^ = (s - t) / r, formed
//     in FP64 and rounded once to FP32, so the basis and the weights see
//     O(1) arguments (P(x) / r^deg = P(x^), and rbf(|x| / r) = rbf(|x^|));
//   * FP32 weights, basis and moment assembly, the 55 upper-triangle sums
//     Kahan-compensated (plain FP32 sums lose ~2e-6 at k = 32);
//   * the eigen-decomposition of the scaled moments A^ = V L V^T as a
//     symmetric Jacobi method in round-robin (parallel) order -- each round's
//     M/2 disjoint rotations have independent parameter chains, which hides
//     the FP64 latency -- run to FP32 convergence, then
//     finished in FP64: B = V32^T A^ V32 (A^ with its compensation terms,
//     exactly in FP64) is nearly diagonal and one FP64 sweep (pairs below
//     1e-15 relative are skipped) converges it quadratically, accumulating
//     W = V32 V64;
//   * FP64 truncation relative to the scaled spectrum: lambda_k <= 2^-20
//     lambda_max is dropped (the scaled moments are well conditioned, cond
//     ~1e3-1e4 at the benchmark densities, so only geometric rank deficiency
//     falls below it);
//   * one FP64 iterative-refinement step of row 0 of the pseudo-inverse
//     against the exact residual e0 - sum_j phi_j P_j (P_j . a) (the basis
//     of FP32 coordinates is exact in FP64), which removes the FP32
//     assembly error (the step contracts it by ~cond(A^) * 2^-24);
//   * coefficients c_j = phi_j (P(x^_j) . a), stored in FP32.
// Row 0 of the pseudo-inverse is applied without forming it:
//   A^+ v = W L^+ W^T v.
// GB300 issues one FP64 warp instruction per 64 cycles per SM sub-partition,
// so all Jacobi state lives in shared memory (thread-interleaved, 1640 B per
// thread at M = 10: four warps per SM, one per sub-partition) and the FP64
// work is what sets the time: ~11k FP64 operations per target against ~57k
// for the FP64 form's reference Jacobi.
#include "dtk_common.cuh"

namespace dtk
{
namespace
{

constexpr int MB = 32;      // threads per block (one warp)
constexpr unsigned FULL = 0xffffffffu;

// FP32 weight of a scaled neighbour.  The Buhmann functions are expanded
// polynomials whose terms cancel (coefficients up to ~400 for values ~0.1),
// so they are evaluated in FP64 and rounded once; the Wendland and Wu
// functions are products (1 - x)^n p(x) and stay accurate in FP32.
__device__ __forceinline__ float weight32( int rbf, float x, float y, float z )
{
    if ( rbf >= DTK_BUHMANN2 )
    {
        double const dx = x, dy = y, dz = z;
        return (float)rbf_eval<double>( rbf, sqrt( dx * dx + dy * dy + dz * dz ) );
    }
    return rbf_eval<float>( rbf, sqrtf( x * x + y * y + z * z ) );
}

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

template <int M>
__global__ void __launch_bounds__( MB )
    k_setup_mixed( PointsView src, PointsView tgt, int32_t const *offset, int32_t const *idx,
                   uint32_t const *order, int64_t n_tgt, int rbf, bool rows_sorted,
                   float *coeff, unsigned long long *under_count,
                   unsigned long long *rot_count, unsigned long long *rot32_count,
                   unsigned *status )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    extern __shared__ unsigned char smem_raw[];
    // Per-thread regions, thread-interleaved (conflict-free):
    //   R1: M*M doubles  -- A64 (compensated moments), later W = V32 V64
    //   R3: NU doubles   -- A32 (FP32 copy, first half), later B
    //   R2: M*M floats   -- V32
    double *r1 = reinterpret_cast<double *>( smem_raw );
    double *r3 = r1 + M * M * MB;
    float *r2 = reinterpret_cast<float *>( r3 + NU * MB );
    int const t = threadIdx.x;
    auto A64 = [&]( int u ) -> double & { return r1[u * MB + t]; };
    auto W = [&]( int r, int c ) -> double & { return r1[( r * M + c ) * MB + t]; };
    auto A32 = [&]( int u ) -> float & { return reinterpret_cast<float *>( r3 )[u * MB + t]; };
    auto B = [&]( int u ) -> double & { return r3[u * MB + t]; };
    auto V32 = [&]( int r, int c ) -> float & { return r2[( r * M + c ) * MB + t]; };

    int64_t const g = blockIdx.x * (int64_t)MB + threadIdx.x;
    unsigned rotations = 0, rotations32 = 0;
    int dropped = 0;
    if ( g < n_tgt )
    {
        int64_t const i = order ? (int64_t)order[g] : g;
        int64_t const b = offset[i];
        int len = offset[i + 1] - (int)b;
        for ( int j = 0; j < len; ++j )
            if ( (uint32_t)idx[b + j] >= (uint64_t)src.n )
            {
                atomicOr( status, DEV_BAD_INDEX );
                len = 0;
            }
        double const tx = tgt( i, 0 ), ty = tgt( i, 1 ), tz = tgt( i, 2 );

        // support radius (FP64, as the reference: 1.1 * max(10 eps, max |x|))
        double d2max = 0.0;
        for ( int j = rows_sorted ? max( 0, len - 1 ) : 0; j < len; ++j )
        {
            int64_t const sj = idx[b + j];
            d2max = fmax( d2max, dist2_rn( src( sj, 0 ), src( sj, 1 ), src( sj, 2 ), tx, ty, tz ) );
        }
        double distance = 10. * DBL_EPSILON;
        double const dmax = __dsqrt_rn( d2max );
        if ( dmax > distance )
            distance = dmax;
        double const inv_r = 1.0 / ( 1.1 * distance );
        // centred, scaled neighbour coordinates: FP64 difference, one rounding
        auto scaled = [&]( int j, float &x, float &y, float &z ) {
            int64_t const sj = idx[b + j];
            x = (float)( ( src( sj, 0 ) - tx ) * inv_r );
            y = (float)( ( src( sj, 1 ) - ty ) * inv_r );
            z = (float)( ( src( sj, 2 ) - tz ) * inv_r );
        };

        // FP32 moments with Kahan compensation (registers)
        {
            float A[NU], C[NU];
#pragma unroll
            for ( int u = 0; u < NU; ++u )
            {
                A[u] = 0.f;
                C[u] = 0.f;
            }
            for ( int j = 0; j < len; ++j )
            {
                float x, y, z;
                scaled( j, x, y, z );
                float P[M];
                basis_eval<M, float>( x, y, z, P );
                float const phi = weight32( rbf, x, y, z );
#pragma unroll
                for ( int a = 0; a < M; ++a )
                {
                    float const pa = P[a] * phi;
#pragma unroll
                    for ( int c = a; c < M; ++c )
                    {
                        int const u = ut<M>( a, c );
                        float const term = __fmul_rn( pa, P[c] );
                        float const yv = __fsub_rn( term, C[u] );
                        float const tt = __fadd_rn( A[u], yv );
                        C[u] = __fsub_rn( __fsub_rn( tt, A[u] ), yv );
                        A[u] = tt;
                    }
                }
            }
#pragma unroll
            for ( int u = 0; u < NU; ++u )
            {
                double const v = (double)A[u] - (double)C[u]; // exact in FP64
                A64( u ) = v;
                A32( u ) = (float)v;
            }
        }

        // FP32 cyclic Jacobi to FP32 convergence
#pragma unroll
        for ( int r = 0; r < M; ++r )
#pragma unroll
            for ( int c = 0; c < M; ++c )
                V32( r, c ) = r == c ? 1.f : 0.f;
        for ( int sweep = 0; sweep < 12; ++sweep )
        {
            int const n = jacobi_sweep<M, float>( A32, V32, 1e-7f );
            rotations32 += n;
            if ( n == 0 )
                break;
        }

        // B = V32^T A64 V32 (upper triangle, FP64), written over A32
        for ( int k = 0; k < M; ++k )
        {
            double ck[M];
#pragma unroll
            for ( int r = 0; r < M; ++r )
            {
                double acc = 0.0;
#pragma unroll
                for ( int c = 0; c < M; ++c )
                    acc = fma( A64( ut<M>( r, c ) ), (double)V32( c, k ), acc );
                ck[r] = acc;
            }
            for ( int jj = 0; jj <= k; ++jj )
            {
                double acc = 0.0;
#pragma unroll
                for ( int r = 0; r < M; ++r )
                    acc = fma( (double)V32( r, jj ), ck[r], acc );
                B( ut<M>( jj, k ) ) = acc;
            }
        }
        // W = V32 in FP64 (over A64), then FP64 sweeps on the nearly
        // diagonal B until no pair is above 1e-15 relative
#pragma unroll
        for ( int r = 0; r < M; ++r )
#pragma unroll
            for ( int c = 0; c < M; ++c )
                W( r, c ) = (double)V32( r, c );
        // one FP64 sweep: B is FP32-converged (off-diagonal ~1e-7
        // relative), so one quadratically convergent sweep takes it to
        // ~1e-14; the refinement step below absorbs what is left
        rotations += jacobi_sweep<M, double>( B, W, 1e-15 );

        // truncation relative to the scaled spectrum: keep 1/lambda_k (or 0)
        // on the diagonal of B for the pseudo-inverse A^+ = W L^+ W^T
        double lmax = 0.0;
        for ( int k = 0; k < M; ++k )
            lmax = fmax( lmax, fabs( B( ut<M>( k, k ) ) ) );
        double const cut = lmax * 9.5367431640625e-07; // 2^-20
        for ( int k = 0; k < M; ++k )
        {
            double const lk = B( ut<M>( k, k ) );
            if ( fabs( lk ) > cut && lk != 0.0 )
                B( ut<M>( k, k ) ) = 1.0 / lk;
            else
            {
                B( ut<M>( k, k ) ) = 0.0;
                dropped = 1;
            }
        }
        // y += A^+ v (FP64), one eigen-direction at a time
        auto pinv_add = [&]( double const *v, double *y ) {
            for ( int k = 0; k < M; ++k )
            {
                double acc = 0.0;
#pragma unroll
                for ( int r = 0; r < M; ++r )
                    acc = fma( W( r, k ), v[r], acc );
                acc *= B( ut<M>( k, k ) );
#pragma unroll
                for ( int r = 0; r < M; ++r )
                    y[r] = fma( W( r, k ), acc, y[r] );
            }
        };
        double a[M];
#pragma unroll
        for ( int r = 0; r < M; ++r )
            a[r] = 0.0;
        for ( int k = 0; k < M; ++k )
        {
            double const g = W( 0, k ) * B( ut<M>( k, k ) );
#pragma unroll
            for ( int r = 0; r < M; ++r )
                a[r] = fma( W( r, k ), g, a[r] );
        }

        // One FP64 refinement step of row 0: the FP32 moments carry
        // ~cond * 6e-8 relative error; the residual r = e0 - sum_j phi_j
        // P_j (P_j . a) is exact up to FP64 rounding (P of the FP32
        // coordinates is exact in FP64, phi_j is the FP32 weight), and
        // a += A32^+ r contracts the error by ~cond(A^) * 2^-24.
        {
            double r[M];
#pragma unroll
            for ( int q = 0; q < M; ++q )
                r[q] = q == 0 ? 1.0 : 0.0;
            for ( int j = 0; j < len; ++j )
            {
                float x, y, z;
                scaled( j, x, y, z );
                double P[M];
                basis_eval<M, double>( (double)x, (double)y, (double)z, P );
                double const phi = (double)weight32( rbf, x, y, z );
                double dot = 0.0;
#pragma unroll
                for ( int q = 0; q < M; ++q )
                    dot = fma( P[q], a[q], dot );
                double const w = phi * dot;
#pragma unroll
                for ( int q = 0; q < M; ++q )
                    r[q] = fma( -w, P[q], r[q] );
            }
            pinv_add( r, a );
        }

        // coefficients c_j = phi_j (P_j . a): FP64 dot of exact FP64 basis
        // values of the FP32 coordinates, stored in FP32
        for ( int j = 0; j < len; ++j )
        {
            float x, y, z;
            scaled( j, x, y, z );
            double P[M];
            basis_eval<M, double>( (double)x, (double)y, (double)z, P );
            float const phi = weight32( rbf, x, y, z );
            double dot = 0.0;
#pragma unroll
            for ( int q = 0; q < M; ++q )
                dot = fma( P[q], a[q], dot );
            coeff[b + j] = (float)( dot * (double)phi );
        }
    }
    unsigned long long it64 = rotations, it32 = rotations32, dr64 = dropped;
    for ( int o = 16; o; o >>= 1 )
    {
        it64 += __shfl_xor_sync( FULL, it64, o );
        it32 += __shfl_xor_sync( FULL, it32, o );
        dr64 += __shfl_xor_sync( FULL, dr64, o );
    }
    if ( threadIdx.x == 0 )
    {
        if ( it64 )
            atomicAdd( rot_count, it64 );
        if ( it32 )
            atomicAdd( rot32_count, it32 );
        if ( dr64 )
            atomicAdd( under_count, dr64 );
    }
}

template <int M>
void launch_mixed( SetupArgs const &a, cudaStream_t s )
{
    size_t const smem = ( (size_t)M * M * sizeof( double ) + (size_t)M * ( M + 1 ) / 2 * sizeof( double ) +
                          (size_t)M * M * sizeof( float ) ) * MB;
    static bool configured = false;
    if ( !configured )
    {
        DTK_CUDA_OR_THROW( cudaFuncSetAttribute( k_setup_mixed<M>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem ) );
        configured = true;
    }
    unsigned const blocks = (unsigned)( ( a.n_tgt + MB - 1 ) / MB );
    k_setup_mixed<M><<<blocks, MB, smem, s>>>( a.src, a.tgt, a.offset, a.idx, a.order, a.n_tgt,
                                                a.rbf, a.rows_sorted, a.coeff32, a.underdetermined,
                                                a.rotations, a.rotations32, a.status );
    check_launch( "k_setup_mixed" );
}

} // namespace

void setup_mixed( SetupArgs const &a, cudaStream_t s )
{
    if ( a.n_tgt == 0 )
        return;
    switch ( a.basis )
    {
    case DTK_CONSTANT3:
        launch_mixed<1>( a, s );
        break;
    case DTK_LINEAR3:
        launch_mixed<4>( a, s );
        break;
    default:
        launch_mixed<10>( a, s );
        break;
    }
}

} // namespace dtk
