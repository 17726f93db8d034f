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
#include "dtk_jacobi.cuh"

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
