// Fused MLS setup, mixed FP32/FP64 form (sm_103a).
//
// Same stages as the FP64 form (DTK_DetailsMovingLeastSquaresOperatorImpl.hpp
// :72-336 after the search), one thread per target, but:
//   * centring and scaling by the support radius, x^ = (s - t) (1/r) with
//     the difference rounded to FP32 (from double-float splits of s and t
//     in the fast path, in FP64 in the Jacobi path) and an FP32 scale, so the
//     basis and the weights see O(1) arguments (P(x) / r^deg = P(x^), and
//     rbf(|x| / r) = rbf(|x^|));
//   * FP32 weights, basis and moment assembly (registers);
//   * an FP32 inverse M of the scaled moments A^ as the preconditioner of
//     iterative refinement for row 0 of the pseudo-inverse, a = M e0,
//     a += M (e0 - A a), the residual summed over the neighbours themselves
//     (not from the FP32 moments): in double-float arithmetic on the FP32
//     pipe in the fast path, in FP64 in the Jacobi path.  The basis of FP32
//     coordinates is exact there and phi_j is the FP32 weight.  A step
//     contracts the FP32 error by ~cond(A^) 2^-24, which leaves the FP32
//     rounding of the coordinates as the only error (~2.5e-8 rel L2 on the
//     8M-point workload; an FP64 eigen-solve, or Kahan-compensated moments,
//     give the same error);
//   * coefficients c_j = phi_j (P(x^_j) . a) as compensated dots, stored in
//     FP32.
// The preconditioner M:
//   * fast path (k_setup_mixed): Cholesky A^ = R^T R in FP32 registers,
//     S = R^-1, M = S S^T.  It is taken when the factorization succeeds and
//     trace(A^) ||S||_F^2 <= 2^20: since lambda_max <= trace and
//     1/lambda_min = ||S||_2^2 <= ||S||_F^2, that bounds cond(A^) by 2^20, so
//     the truncation below would drop nothing and M ~ A^-1 = A^+.  Above
//     2^16 a second refinement step is taken.
//   * otherwise (k_setup_mixed_eig, the targets the fast path lists): the
//     symmetric Jacobi method in round-robin order, in FP32 to FP32
//     convergence, truncation lambda_k <= 2^-20 lambda_max (geometric rank
//     deficiency), M = V L^+ V^T.
// GB300 issues one FP64 warp instruction per 64 cycles per SM sub-partition;
// the FP64 work left in the fast path is the support radius (one FP64
// distance per target for sorted rows).  The fast path stages each warp's
// rows in shared memory (12.4 KB per warp) and keeps the rest in registers;
// the Jacobi path keeps A^ and V (FP32) thread-interleaved in shared memory,
// 620 B per thread at M = 10.
#include "dtk_common.cuh"
#include "dtk_jacobi.cuh"

#include <algorithm>

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

// ---------------------------------------------------------------------------
// Double-float arithmetic on the FP32 pipe (GB300's FP64 rate is 1/58 of its
// FP32 rate): a value is an unevaluated sum hi + lo of two floats.  TwoSum
// (Knuth) and TwoProd (with an FMA) are error-free; the dot products follow
// the compensated "Dot2" scheme of Ogita, Rump and Oishi (2005): the rounding
// errors of every product and partial sum are collected in a second float,
// which gives the result as if computed in twice the working precision.
// The explicit _rn intrinsics keep the compiler from contracting the
// error-free steps into FMAs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum( float a, float b, float &s, float &e )
{
    s = __fadd_rn( a, b );
    float const bb = __fsub_rn( s, a );
    e = __fadd_rn( __fsub_rn( a, __fsub_rn( s, bb ) ), __fsub_rn( b, bb ) );
}

__device__ __forceinline__ void two_prod( float a, float b, float &p, float &e )
{
    p = __fmul_rn( a, b );
    e = __fmaf_rn( a, b, -p );
}

// Basis values of FP32 coordinates as double-floats (exact: the quadratic
// products are TwoProds).
template <int M>
__device__ __forceinline__ void basis_df( float x, float y, float z, float *ph, float *pl )
{
    ph[0] = 1.f;
    pl[0] = 0.f;
    if constexpr ( M >= 4 )
    {
        ph[1] = x;
        ph[2] = y;
        ph[3] = z;
        pl[1] = pl[2] = pl[3] = 0.f;
    }
    if constexpr ( M == 10 )
    {
        two_prod( x, x, ph[4], pl[4] );
        two_prod( x, y, ph[5], pl[5] );
        two_prod( x, z, ph[6], pl[6] );
        two_prod( y, y, ph[7], pl[7] );
        two_prod( y, z, ph[8], pl[8] );
        two_prod( z, z, ph[9], pl[9] );
    }
}

// P . a as (s, c) with s + c the compensated dot, a = ah + al
template <int M>
__device__ __forceinline__ void dot_df( float const *ph, float const *pl, float const *ah, float const *al,
                                        float &s, float &c )
{
    s = 0.f;
    c = 0.f;
#pragma unroll
    for ( int q = 0; q < M; ++q )
    {
        float p, e, t, f;
        two_prod( ph[q], ah[q], p, e );
        two_sum( s, p, t, f );
        s = t;
        c = __fadd_rn( c, __fadd_rn( e, f ) );
        c = __fmaf_rn( ph[q], al[q], c );
        c = __fmaf_rn( pl[q], ah[q], c );
    }
}

// Refinement and coefficients of the fast path in double-float: a = ah + al
// on entry (the FP32 solve, al = 0); r = e0 - sum_j phi_j P_j (P_j . a)
// accumulated per component as rh + rl; a += M r; c_j = phi_j (P_j . a)
// rounded once to FP32 and handed to store(j, c_j).
template <int M, class Scaled, class Pinv, class Store>
__device__ __forceinline__ void refine_and_store_df( int len, int rbf, int steps, Scaled const &scaled,
                                                     Pinv const &pinv32, float *ah, float *al,
                                                     Store const &store )
{
    for ( int step = 0; step < steps; ++step )
    {
        float rh[M], rl[M];
#pragma unroll
        for ( int q = 0; q < M; ++q )
        {
            rh[q] = q == 0 ? 1.f : 0.f;
            rl[q] = 0.f;
        }
        for ( int j = 0; j < len; ++j )
        {
            float x, y, z;
            scaled( j, x, y, z );
            float ph[M], pl[M];
            basis_df<M>( x, y, z, ph, pl );
            float const phi = weight32( rbf, x, y, z );
            float s, c;
            dot_df<M>( ph, pl, ah, al, s, c );
            float wh, wl;
            two_prod( phi, s, wh, wl );
            wl = __fmaf_rn( phi, c, wl );
#pragma unroll
            for ( int q = 0; q < M; ++q )
            {
                float p, e, t, f;
                two_prod( wh, ph[q], p, e );
                e = __fmaf_rn( wh, pl[q], e );
                e = __fmaf_rn( wl, ph[q], e );
                two_sum( rh[q], -p, t, f );
                rh[q] = t;
                rl[q] = __fadd_rn( rl[q], __fsub_rn( f, e ) );
            }
        }
        float rf[M], d[M];
#pragma unroll
        for ( int q = 0; q < M; ++q )
            rf[q] = __fadd_rn( rh[q], rl[q] );
        pinv32( rf, d );
#pragma unroll
        for ( int q = 0; q < M; ++q )
        {
            float t, f;
            two_sum( ah[q], d[q], t, f );
            ah[q] = t;
            al[q] = __fadd_rn( al[q], f );
        }
    }
    for ( int j = 0; j < len; ++j )
    {
        float x, y, z;
        scaled( j, x, y, z );
        float ph[M], pl[M];
        basis_df<M>( x, y, z, ph, pl );
        float const phi = weight32( rbf, x, y, z );
        float s, c;
        dot_df<M>( ph, pl, ah, al, s, c );
        float wh, wl;
        two_prod( phi, s, wh, wl );
        store( j, __fadd_rn( wh, __fmaf_rn( phi, c, wl ) ) );
    }
}

// Sources as double-floats: hi = fl32(v), lo = fl32(v - hi), (hi, lo) per
// coordinate, 3 float2 per point: in the tree's sorted order (s2 set: the
// neighbours are then addressed by sorted position) or in the caller's.
__global__ void k_split_points( PointsView p, double2 const *s2, float2 *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= p.n )
        return;
    double v[3];
    if ( s2 )
    {
        double2 const a = s2[2 * i], b = s2[2 * i + 1];
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
    }
    else
        for ( int d = 0; d < 3; ++d )
            v[d] = p( i, d );
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        float const hi = __double2float_rn( v[d] );
        out[3 * i + d] = make_float2( hi, __double2float_rn( v[d] - (double)hi ) );
    }
}

// Fast path: FP32 Cholesky preconditioner in registers; targets it cannot
// take (factorization fails, or the condition bound exceeds 2^20) are
// appended to `list` for k_setup_mixed_eig.  A warp first stages the
// neighbours of its 32 targets in shared memory, one row at a time with one
// lane per neighbour (coalesced index loads, 32 independent gathers in
// flight), as centred FP32 coordinates (sh - th) + (sl - tl); the three
// per-target passes (moments, residual, coefficients) then read them from
// there, and the coefficients go back out row by row.
constexpr int SMX = 32;       // threads per block of the fast kernel (one warp: 3% faster than two)
constexpr int ROW_PITCH = 33; // staged rows: [axis][neighbour][target lane], 33 floats a neighbour

template <int M>
__global__ void __launch_bounds__( SMX, 16 )
    k_setup_mixed( Neighbours nb, float2 const *__restrict__ split, PointsView tgt, int32_t const *offset,
                   uint32_t const *order, int64_t n_tgt, int rbf, bool rows_sorted,
                   float *coeff, int32_t *list, unsigned *count, unsigned *status )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    static_assert( FUSED_MAX_ROW <= 32, "one lane per neighbour when staging a row" );
    // pitch 33: the row-wise fill (lanes = neighbours) and the per-target
    // reads (lanes = targets) both touch 32 distinct banks; after the last
    // pass the x plane holds the coefficients
    __shared__ float s_nb[SMX / 32][3][32 * ROW_PITCH];
    int const lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int64_t const g = blockIdx.x * (int64_t)SMX + threadIdx.x;
    if ( g - lane >= n_tgt )
        return; // the whole warp is past the end; below, all 32 lanes take part
    bool const active = g < n_tgt;
    int64_t const i = active ? ( order ? (int64_t)order[g] : g ) : 0;
    int64_t const b = active ? offset[i] : 0;
    int len = active ? offset[i + 1] - (int)b : 0;
    if ( len > FUSED_MAX_ROW || len < 0 )
    {
        atomicOr( status, DEV_BAD_INDEX );
        len = 0;
    }
    double const tx = active ? tgt( i, 0 ) : 0.0, ty = active ? tgt( i, 1 ) : 0.0,
                 tz = active ? tgt( i, 2 ) : 0.0;
    float *const sx = s_nb[wib][0], *const sy = s_nb[wib][1], *const sz = s_nb[wib][2];
    // sorted rows: the farthest neighbour (the last) sets the support radius;
    // its FP64 coordinates are fetched now, to arrive during the staging
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if ( rows_sorted && len > 0 && (uint32_t)nb.ref( b + len - 1 ) < (uint64_t)nb.src.n )
        nb.xyz( b + len - 1, fx, fy, fz );
    {
        // the target as double-floats; (sh - th) is exact for nearby points
        // (Sterbenz)
        float th[3], tl[3];
        double const t3[3] = {tx, ty, tz};
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            th[d] = __double2float_rn( t3[d] );
            tl[d] = __double2float_rn( t3[d] - (double)th[d] );
        }
        unsigned bad_rows = 0;
#pragma unroll 2
        for ( int t = 0; t < 32; ++t )
        {
            int const lt = __shfl_sync( FULL, len, t );
            if ( lt == 0 )
                continue; // warp-uniform
            int64_t const bt = __shfl_sync( FULL, b, t );
            float const hx = __shfl_sync( FULL, th[0], t ), hy = __shfl_sync( FULL, th[1], t ),
                        hz = __shfl_sync( FULL, th[2], t );
            float const lx = __shfl_sync( FULL, tl[0], t ), ly = __shfl_sync( FULL, tl[1], t ),
                        lz = __shfl_sync( FULL, tl[2], t );
            bool bad = false;
            if ( lane < lt )
            {
                uint32_t const sj = (uint32_t)nb.ref( bt + lane );
                if ( sj >= (uint64_t)nb.src.n )
                    bad = true;
                else
                {
                    float2 const a0 = __ldg( split + 3 * (int64_t)sj ), a1 = __ldg( split + 3 * (int64_t)sj + 1 ),
                                 a2 = __ldg( split + 3 * (int64_t)sj + 2 );
                    sx[lane * ROW_PITCH + t] = __fadd_rn( __fsub_rn( a0.x, hx ), __fsub_rn( a0.y, lx ) );
                    sy[lane * ROW_PITCH + t] = __fadd_rn( __fsub_rn( a1.x, hy ), __fsub_rn( a1.y, ly ) );
                    sz[lane * ROW_PITCH + t] = __fadd_rn( __fsub_rn( a2.x, hz ), __fsub_rn( a2.y, lz ) );
                }
            }
            if ( __any_sync( FULL, bad ) )
                bad_rows |= 1u << t;
        }
        __syncwarp();
        if ( ( bad_rows >> lane ) & 1u )
        {
            atomicOr( status, DEV_BAD_INDEX );
            len = 0;
        }
    }
    bool fast = false;
    if ( active )
    {
        double d2max = rows_sorted && len > 0 ? dist2_rn( fx, fy, fz, tx, ty, tz ) : 0.0;
        for ( int j = 0; !rows_sorted && j < len; ++j )
        {
            double sx, sy, sz;
            nb.xyz( b + j, sx, sy, sz );
            d2max = fmax( d2max, dist2_rn( sx, sy, sz, tx, ty, tz ) );
        }
        double distance = 10. * DBL_EPSILON;
        double const dmax = __dsqrt_rn( d2max );
        if ( dmax > distance )
            distance = dmax;
        float const inv_r = (float)( 1.0 / ( 1.1 * distance ) );
        auto scaled = [&]( int j, float &x, float &y, float &z ) {
            x = __fmul_rn( sx[j * ROW_PITCH + lane], inv_r );
            y = __fmul_rn( sy[j * ROW_PITCH + lane], inv_r );
            z = __fmul_rn( sz[j * ROW_PITCH + lane], inv_r );
        };

        // FP32 moments, upper triangle R(a, c) = A[ut(a, c)], a <= c
        float A[NU];
#pragma unroll
        for ( int u = 0; u < NU; ++u )
            A[u] = 0.f;
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
                    A[ut<M>( a, c )] = fmaf( pa, P[c], A[ut<M>( a, c )] );
            }
        }
        float trace = 0.f;
#pragma unroll
        for ( int k = 0; k < M; ++k )
            trace += A[ut<M>( k, k )];

        // Cholesky A = R^T R in place (R upper triangular, row-major packed)
        bool ok = trace > 0.f;
        float rinv[M];
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
            float d = A[ut<M>( j, j )];
#pragma unroll
            for ( int k = 0; k < j; ++k )
                d = fmaf( -A[ut<M>( k, j )], A[ut<M>( k, j )], d );
            ok = ok && d > 0.f;
            float const inv = d > 0.f ? rsqrtf( d ) : 0.f;
            rinv[j] = inv;
            A[ut<M>( j, j )] = d * inv; // sqrt(d)
#pragma unroll
            for ( int c = j + 1; c < M; ++c )
            {
                float v = A[ut<M>( j, c )];
#pragma unroll
                for ( int k = 0; k < j; ++k )
                    v = fmaf( -A[ut<M>( k, j )], A[ut<M>( k, c )], v );
                A[ut<M>( j, c )] = v * inv;
            }
        }
        // S = R^-1 in place, column by column: S(j,j) = 1/R(j,j),
        // S(r,j) = -(sum_{k=r}^{j-1} S(r,k) R(k,j)) / R(j,j), r ascending
        float fro = 0.f;
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
#pragma unroll
            for ( int r = 0; r < j; ++r )
            {
                float v = 0.f;
#pragma unroll
                for ( int k = r; k < j; ++k )
                    v = fmaf( k == r ? A[ut<M>( r, r )] : A[ut<M>( r, k )], A[ut<M>( k, j )], v );
                // S(r, r) is already stored at (r, r); S(r, k) for k < j too
                A[ut<M>( r, j )] = -v * rinv[j];
            }
            A[ut<M>( j, j )] = rinv[j];
        }
#pragma unroll
        for ( int u = 0; u < NU; ++u )
            fro = fmaf( A[u], A[u], fro );
        float const crit = trace * fro;
        if ( !ok || !( crit <= 1048576.f ) ) // 2^20; false for NaN
        {
            unsigned const slot = atomicAdd( count, 1u );
            list[slot] = (int32_t)i;
        }
        else
        {
            fast = true;
            // M v = S (S^T v)
            auto pinv32 = [&]( float const *v, float *y ) {
                float w[M];
#pragma unroll
                for ( int k = 0; k < M; ++k )
                {
                    float acc = 0.f;
#pragma unroll
                    for ( int r = 0; r <= k; ++r )
                        acc = fmaf( A[ut<M>( r, k )], v[r], acc );
                    w[k] = acc;
                }
#pragma unroll
                for ( int r = 0; r < M; ++r )
                {
                    float acc = 0.f;
#pragma unroll
                    for ( int k = r; k < M; ++k )
                        acc = fmaf( A[ut<M>( r, k )], w[k], acc );
                    y[r] = acc;
                }
            };
            float ah[M], al[M];
            {
                float e0[M];
#pragma unroll
                for ( int r = 0; r < M; ++r )
                {
                    e0[r] = r == 0 ? 1.f : 0.f;
                    al[r] = 0.f;
                }
                pinv32( e0, ah );
            }
            refine_and_store_df<M>( len, rbf, crit <= 65536.f ? 1 : 2, scaled, pinv32, ah, al,
                                    [&]( int j, float c ) { sx[j * ROW_PITCH + lane] = c; } );
        }
    }
    // the coefficients of the fast rows, row by row (one lane per entry)
    int const out_len = fast ? len : 0;
    __syncwarp();
    for ( int t = 0; t < 32; ++t )
    {
        int const lt = __shfl_sync( FULL, out_len, t );
        if ( lt == 0 )
            continue; // warp-uniform
        int64_t const bt = __shfl_sync( FULL, b, t );
        if ( lane < lt )
            coeff[bt + lane] = sx[lane * ROW_PITCH + t];
    }
}

// Jacobi path over the targets the fast path listed: list[0 .. *count),
// persistent blocks striding over the list.
template <int M>
__global__ void __launch_bounds__( MB, 8 )
    k_setup_mixed_eig( PointsView src, PointsView tgt, int32_t const *offset, int32_t const *idx,
                       int32_t const *list, unsigned const *count, int rbf, bool rows_sorted,
                       float *coeff, unsigned long long *under_count,
                       unsigned long long *rot32_count, unsigned *status )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    extern __shared__ float smem_f[];
    // Per-thread regions, thread-interleaved (conflict-free):
    //   R1: NU floats  -- A^ (upper triangle); after the Jacobi its diagonal
    //                     holds 1 / lambda_k (0 where truncated)
    //   R2: M*M floats -- V
    float *r1 = smem_f;
    float *r2 = r1 + NU * MB;
    int const t = threadIdx.x;
    auto A32 = [&]( int u ) -> float & { return r1[u * MB + t]; };
    auto V32 = [&]( int r, int c ) -> float & { return r2[( r * M + c ) * MB + t]; };

    int64_t const n_list = *count;
    unsigned rotations32 = 0;
    int dropped = 0;
    for ( int64_t g = blockIdx.x * (int64_t)MB + threadIdx.x; g - threadIdx.x < n_list;
          g += (int64_t)gridDim.x * MB )
    {
        if ( g >= n_list )
            continue;
        int64_t const i = list[g];
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
        float const inv_r = (float)( 1.0 / ( 1.1 * distance ) );
        // centred, scaled neighbour coordinates: FP64 difference, FP32 scale
        auto scaled = [&]( int j, float &x, float &y, float &z ) {
            int64_t const sj = idx[b + j];
            x = __fmul_rn( (float)( src( sj, 0 ) - tx ), inv_r );
            y = __fmul_rn( (float)( src( sj, 1 ) - ty ), inv_r );
            z = __fmul_rn( (float)( src( sj, 2 ) - tz ), inv_r );
        };

        // FP32 moments (registers)
        {
            float A[NU];
#pragma unroll
            for ( int u = 0; u < NU; ++u )
                A[u] = 0.f;
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
                        A[ut<M>( a, c )] = fmaf( pa, P[c], A[ut<M>( a, c )] );
                }
            }
#pragma unroll
            for ( int u = 0; u < NU; ++u )
                A32( u ) = A[u];
        }

        // FP32 round-robin Jacobi to FP32 convergence
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

        // truncation relative to the scaled spectrum: 1/lambda_k or 0 on the diagonal
        float lmax = 0.f;
        for ( int k = 0; k < M; ++k )
            lmax = fmaxf( lmax, fabsf( A32( ut<M>( k, k ) ) ) );
        float const cut = lmax * 9.5367431640625e-07f; // 2^-20
        int dropped_here = 0;
        for ( int k = 0; k < M; ++k )
        {
            float const lk = A32( ut<M>( k, k ) );
            if ( fabsf( lk ) > cut && lk != 0.f )
                A32( ut<M>( k, k ) ) = 1.f / lk;
            else
            {
                A32( ut<M>( k, k ) ) = 0.f;
                dropped_here = 1;
            }
        }
        dropped += dropped_here;
        // y = M v = V L^+ V^T v (FP32), one eigen-direction at a time
        auto pinv32 = [&]( float const *v, float *y ) {
#pragma unroll
            for ( int r = 0; r < M; ++r )
                y[r] = 0.f;
            for ( int k = 0; k < M; ++k )
            {
                float acc = 0.f;
#pragma unroll
                for ( int r = 0; r < M; ++r )
                    acc = fmaf( V32( r, k ), v[r], acc );
                acc *= A32( ut<M>( k, k ) );
#pragma unroll
                for ( int r = 0; r < M; ++r )
                    y[r] = fmaf( V32( r, k ), acc, y[r] );
            }
        };
        double a[M];
        {
            float e0[M], y[M];
#pragma unroll
            for ( int r = 0; r < M; ++r )
                e0[r] = r == 0 ? 1.f : 0.f;
            pinv32( e0, y );
#pragma unroll
            for ( int r = 0; r < M; ++r )
                a[r] = (double)y[r];
        }

        // One refinement step of row 0: r = e0 - sum_j phi_j P_j (P_j . a) in
        // FP64 (P of the FP32 coordinates is exact in FP64, phi_j is the FP32
        // weight), a += M r.
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
            float rf[M], d[M];
#pragma unroll
            for ( int q = 0; q < M; ++q )
                rf[q] = (float)r[q];
            pinv32( rf, d );
#pragma unroll
            for ( int q = 0; q < M; ++q )
                a[q] += (double)d[q];
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
    unsigned long long it32 = rotations32, dr64 = dropped;
    for ( int o = 16; o; o >>= 1 )
    {
        it32 += __shfl_xor_sync( FULL, it32, o );
        dr64 += __shfl_xor_sync( FULL, dr64, o );
    }
    if ( threadIdx.x == 0 )
    {
        if ( it32 )
            atomicAdd( rot32_count, it32 );
        if ( dr64 )
            atomicAdd( under_count, dr64 );
    }
}

template <int M>
void launch_mixed( SetupArgs const &a, cudaStream_t s )
{
    DeviceBuffer<int32_t> list( a.n_tgt, s );
    DeviceBuffer<unsigned> count( 1, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( count.get(), 0, sizeof( unsigned ), s ) );
    DeviceBuffer<float2> split( 3 * a.src.n, s );
    k_split_points<<<(unsigned)( ( a.src.n + 255 ) / 256 ), 256, 0, s>>>( a.src, a.pos ? a.s2 : nullptr,
                                                                          split.get() );
    check_launch( "k_split_points" );
    Neighbours const nb{a.src, a.idx, a.pos, a.s2};
    k_setup_mixed<M><<<(unsigned)( ( a.n_tgt + SMX - 1 ) / SMX ), SMX, 0, s>>>(
        nb, split.get(), a.tgt, a.offset, a.order, a.n_tgt, a.rbf, a.rows_sorted, a.coeff32,
        list.get(), count.get(), a.status );
    check_launch( "k_setup_mixed" );
    // the listed targets (count known only on the device): persistent blocks
    size_t const smem = ( (size_t)M * ( M + 1 ) / 2 + (size_t)M * M ) * sizeof( float ) * MB;
    ensure_dynamic_smem( k_setup_mixed_eig<M>, smem );
    int64_t const want = ( a.n_tgt + MB - 1 ) / MB;
    unsigned const blocks = (unsigned)std::max<int64_t>( 1, std::min<int64_t>( want, 8 * num_sms() ) );
    k_setup_mixed_eig<M><<<blocks, MB, smem, s>>>( a.src, a.tgt, a.offset, a.idx, list.get(), count.get(),
                                                    a.rbf, a.rows_sorted, a.coeff32, a.underdetermined,
                                                    a.rotations32, a.status );
    check_launch( "k_setup_mixed_eig" );
}

} // namespace

void setup_mixed( SetupArgs const &a, cudaStream_t s )
{
    NvtxRange const nvtx_range( "DTK_compute_polynomial_coeffs" );
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
