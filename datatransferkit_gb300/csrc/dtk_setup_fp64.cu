// Fused MLS setup, FP64 form (sm_103a).
//
// One thread per target (targets in Morton order) runs every stage of the
// reference constructor after the search, fused, with nothing but the
// coefficients written to HBM:
//   gather + transformSourceCoordinates  Impl.hpp:72-99
//   computeVandermonde                   Impl.hpp:171-190
//   computeRadius (1.1 * max(10 eps, max |x|))   Impl.hpp:101-138
//   computeWeights                       Impl.hpp:143-169
//   computeMoments (symmetric, registers)        Impl.hpp:213-258
//   invertMoments -> SVDFunctor          SVDImpl.hpp:197-302
//   computePolynomialCoefficients        Impl.hpp:293-336
// (Impl.hpp = packages/Meshfree/src/DTK_DetailsMovingLeastSquaresOperatorImpl.hpp,
//  SVDImpl.hpp = packages/Meshfree/src/DTK_DetailsSVDImpl.hpp)
//
// The pseudo-inverse keeps DTK's algorithm exactly: two-sided Jacobi with the
// largest off-diagonal pivot (first in row-major order on ties), p<q swap,
// the explicit 2x2 SVD (atan2 half angles, copysign correction, the sr sign
// rule), the absolute DBL_EPSILON stop on the off-diagonal Frobenius norm and
// the absolute DBL_EPSILON truncation.  Its results carry a deterministic
// deviation from the exact pseudo-inverse at fine point spacing (the stop is
// absolute on unscaled moments), so matching the reference to 1e-12 needs the
// same pivots, rotations and stops, not merely any accurate pseudo-inverse.
//
// Thread-per-target, not warp-per-target: GB300's FP64 pipe issues one warp
// instruction per 64 cycles per SM sub-partition, so every FP64 instruction
// must carry 32 useful lanes; the 2x2 SVD is scalar work.  Iteration counts
// are tight (about 114 +- 13 for the quadratic basis), so divergence costs
// little.  E (m x m) and column 0 of V live in shared memory, interleaved
// by thread so that dynamic (p, q) accesses are conflict-free: 880 B a
// thread at m = 10, 8 warps an SM, two per FP64 pipe.  U is never updated
// rotation by rotation: the rotations go to a log in a global work area per
// resident thread (L2-resident, interleaved the same way), and row 0 of the
// pseudo-inverse is the log applied in reverse to one vector (8M targets:
// 432 -> 366 ms against U's explicit updates).
// The kernels are persistent: a thread takes targets g, g + T, ...
// The argmax runs on the integer pipe over the IEEE bits of |E_ij|; the stop
// test too, from exponent bounds, except within a factor of four of the
// threshold where it sums the squares in FP64; the 2x2 rotation angles use
// half-angle identities rather than atan2 and sincos, and the 2x2 SVD's
// compares and sign logic run on the integer pipe too (dtk_ieee.cuh, exactly
// the IEEE results; 8M targets: 366 -> 343 ms).
#include "dtk_common.cuh"
#include "dtk_ieee.cuh"

#include <algorithm>

namespace dtk
{
namespace
{

constexpr int FP64_THREADS = 256; // threads per block of the Jacobi kernels (E, V(:, 0) in shared memory)
constexpr unsigned FULL = 0xffffffffu;

// cos and sin of phi = atan2(y, x) / 2, phi in (-pi/2, pi/2], from the
// half-angle identities (cos phi >= 0, sin phi has the sign of y):
//   x >= 0: cos = (r + x) / sqrt(2r(r + x)),  sin = y / sqrt(2r(r + x))
//   x <  0: |sin| = (r - x) / sqrt(2r(r - x)), cos = |y| / sqrt(2r(r - x))
// with r = |(x, y)|: one sqrt and one reciprocal square root instead of
// atan2 and sincos.  (x, y) is rescaled by a power of two when r^2 would
// leave [1e-280, 1e280] (atan2 is scale-invariant); r^2 >= 0 or NaN, whose
// bits order like its values.
__device__ __forceinline__ void half_angle( double y, double x, double &c, double &s )
{
    double r2 = fma( x, x, y * y );
    unsigned long long b2 = bits_of( r2 );
    if ( !r2_in_range( b2 ) && !( zero_bits( bits_of( x ) ) && zero_bits( bits_of( y ) ) ) )
    {
        int const e = ilogb( fmax( fabs( x ), fabs( y ) ) );
        x = scalbn( x, -e );
        y = scalbn( y, -e );
        r2 = fma( x, x, y * y );
        b2 = bits_of( r2 );
    }
    if ( zero_bits( b2 ) )
    {
        c = 1.0;
        s = y; // atan2(+-0, +0) = +-0
        return;
    }
    double const r = sqrt( r2 );
    double const w = r + fabs( x );
    // 2 r by its exponent: a finite r is normal here (r^2 lies in
    // [1e-280, 1e280], or in [1, 8) after the rescaling)
    double const t = rsqrt( twice_normal( r ) * w );
    if ( ieee_nonneg( x ) )
    {
        c = w * t;
        s = y * t;
    }
    else
    {
        s = copysign( w * t, y );
        c = fabs( y ) * t;
    }
}

// The rotation pair (c a - s b, s a + c b) with the multiply-adds spelled
// out, so that every kernel that runs the Jacobi rounds alike (the compiler
// is free to contract a*b - c*d either way, and may choose differently in
// different kernels).
__device__ __forceinline__ double rot_minus( double c, double s, double a, double b )
{
    return __fma_rn( c, a, -__dmul_rn( s, b ) );
}
__device__ __forceinline__ double rot_plus( double c, double s, double a, double b )
{
    return __fma_rn( s, a, __dmul_rn( c, b ) );
}
// x0 y0 + x1 y1 with the same spelled-out rounding
__device__ __forceinline__ double dot2( double x0, double y0, double x1, double y1 )
{
    return __fma_rn( x0, y0, __dmul_rn( x1, y1 ) );
}

// 2x2 SVD rotations of DTK_DetailsSVDImpl.hpp:119-162 and the sr sign rule
// of :260-263.
__device__ __forceinline__ void svd_2x2( double a, double b, double c, double d, double &cl,
                                         double &sl, double &cr, double &sr )
{
    // A A^T and A^T A in the element order of SVDImpl.hpp:109-117,123-126
    double const p00 = dot2( a, a, b, b ), p01 = dot2( a, c, b, d ), p10 = dot2( c, a, d, b ),
                 p11 = dot2( c, c, d, d );
    double const q00 = dot2( a, a, c, c ), q01 = dot2( a, b, c, d ), q10 = dot2( b, a, d, c ),
                 q11 = dot2( b, b, d, d );
    double sphi, cphi, sth, cth;
    half_angle( p01 + p10, p00 - p11, cphi, sphi );
    half_angle( q01 + q10, q00 - q11, cth, sth );
    // S = U^T A W diagonal signs (SVDImpl.hpp:149-159)
    double const aw00 = dot2( a, cth, b, sth ), aw01 = dot2( a, -sth, b, cth );
    double const aw10 = dot2( c, cth, d, sth ), aw11 = dot2( c, -sth, d, cth );
    double const s00 = dot2( cphi, aw00, sphi, aw10 );
    double const s11 = dot2( -sphi, aw01, cphi, aw11 );
    // V = W diag(c0, c1), c0 = copysign(1, s00), c1 = copysign(1, s11)
    double const v00 = times_sign_of( cth, s00 ), v01 = times_sign_of( ieee_neg( sth ), s11 ),
                 v10 = times_sign_of( sth, s00 );
    cl = cphi;
    sl = ieee_neg( sphi );
    cr = v00;
    sr = ieee_sign( v01 ) == ieee_sign( v10 ) ? ieee_neg( v01 ) : v01;
}

// svd_2x2 of a symmetric block [[a, b], [b, d]]: A A^T and A^T A are then
// formed by the same operations, so the two half-angles are one, and the
// rotations come out bit for bit as svd_2x2( a, b, b, d ) gives them.
__device__ __forceinline__ void svd_2x2_sym( double a, double b, double d, double &cl, double &sl,
                                             double &cr, double &sr )
{
    // q10 = dot2( b, a, d, b ) is q01 bit for bit (IEEE products commute)
    double const q00 = dot2( a, a, b, b ), q01 = dot2( a, b, b, d ), q11 = dot2( b, b, d, d );
    double sth, cth;
    half_angle( q01 + q01, q00 - q11, cth, sth );
    double const aw00 = dot2( a, cth, b, sth ), aw01 = dot2( a, -sth, b, cth );
    double const aw10 = dot2( b, cth, d, sth ), aw11 = dot2( b, -sth, d, cth );
    double const s00 = dot2( cth, aw00, sth, aw10 );
    double const s11 = dot2( -sth, aw01, cth, aw11 );
    double const v00 = times_sign_of( cth, s00 ), v01 = times_sign_of( ieee_neg( sth ), s11 ),
                 v10 = times_sign_of( sth, s00 );
    cl = cth;
    sl = ieee_neg( sth );
    cr = v00;
    sr = ieee_sign( v01 ) == ieee_sign( v10 ) ? ieee_neg( v01 ) : v01;
}

// |x| as an ordered integer (non-negative doubles order like their bits).
__device__ __forceinline__ long long abs_bits( double x )
{
    return __double_as_longlong( x ) & 0x7fffffffffffffffll;
}

template <int M>
struct Smem
{
    // E and V(:, 0) in shared memory, interleaved by thread (stride es, the
    // thread's column t); the global work area W (the rotation log, then U)
    // interleaved by thread too (stride us, column ut).  Every part starts
    // at an offset that does not depend on M, so that threads working on
    // different M at once (the batched setup) never share a slot.
    double *E, *W, *V0;
    int t, es;
    int64_t ut, us;
    __device__ double &e( int i, int j ) const { return E[( i * M + j ) * es + t]; }
    __device__ double &u( int i, int j ) const { return W[( JACOBI_U0 + i * M + j ) * us + ut]; }
    __device__ double &v( int i ) const { return V0[i * es + t]; }
    // rotation r of the log: (cos, sin) of U's right rotation and p * 16 + q
    __device__ double2 &rot( int r ) const { return reinterpret_cast<double2 *>( W )[r * us + ut]; }
    __device__ uint8_t &pivot( int r ) const
    {
        return reinterpret_cast<uint8_t *>( W + 2 * JACOBI_LOG * us )[r * us + ut];
    }
};

// U = G_0 G_1 ... G_{n-1} formed explicitly from the first n logged
// rotations (the updates the reference makes, in its order): for a target
// whose rotations outrun the log, which then updates U as it goes.
template <int M>
__device__ __noinline__ void form_u( Smem<M> const &s, int n )
{
#pragma unroll
    for ( int i = 0; i < M; ++i )
#pragma unroll
        for ( int j = 0; j < M; ++j )
            s.u( i, j ) = i == j ? 1.0 : 0.0;
    for ( int r = 0; r < n; ++r )
    {
        double2 const cs = s.rot( r );
        int const pq = s.pivot( r ), p = pq >> 4, q = pq & 15;
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
            double const a = s.u( j, p ), b = s.u( j, q );
            s.u( j, p ) = rot_minus( cs.x, cs.y, a, b );
            s.u( j, q ) = rot_plus( cs.x, cs.y, a, b );
        }
    }
}

// Grid of the persistent Jacobi kernels: blocks of FP64_THREADS (8 warps an
// SM, one block each) when the targets fill the GPU; otherwise blocks of one
// warp, one target a thread, spread over as many SMs as there are warps.
struct JacobiGrid
{
    unsigned blocks;
    int threads;
    size_t smem;
};
template <int M>
JacobiGrid jacobi_grid( int64_t n )
{
    int64_t const sms = num_sms();
    int const threads = n >= sms * FP64_THREADS ? FP64_THREADS : 32;
    int64_t const want = ( n + threads - 1 ) / threads;
    int64_t const cap = threads == FP64_THREADS ? sms : want;
    return JacobiGrid{(unsigned)std::max<int64_t>( 1, std::min( want, cap ) ), threads,
                      ( M * M + M ) * threads * sizeof( double )};
}

// Runs DTK's Jacobi on the thread's E; on return row0 holds row 0 of the
// pseudo-inverse.  Returns 1 if a singular value was truncated.
//
// U is not updated as the reference does (40 FP64 operations and 20 loads
// and stores a rotation at M = 10): the rotations go to a log, and row 0 of
// the pseudo-inverse, U w with w_k = V(0, k) / E(k, k) (0 where truncated),
// is G_0 (G_1 (... (G_{n-1} w))), the logged rotations applied to w in
// reverse, 4 operations each.  The pivots, rotations and stop are the
// reference's; only the final product is associated differently (a
// rounding-level difference).  A target whose rotations outrun the log forms
// U from it and continues with the reference's updates.
//
// E enters exactly symmetric (the moments fill both triangles from one sum).
// For a non-degenerate E (no zero on the diagonal), while the rotations keep
// it so -- the pivot block is then symmetric, the
// left and right rotations of its 2x2 SVD come out equal (a positive
// semi-definite block), and the right rotation of the off-block entries of
// columns p and q computes the left rotation's values of rows p and q --
// the columns are copied from the rows instead of recomputed, the 2x2 SVD
// solves one half-angle instead of two (their inputs are equal), the scan
// reads the upper triangle (the first largest |E_ij| in row-major order is
// there), and the block's off-diagonal pair, which the two rotations leave
// as two different residuals of the same zero, takes the upper one's value.
// That last step is the only departure from the reference's arithmetic (a
// rounding residual); at the first rotation whose left and right parts
// differ (an indefinite block, as negative Buhmann weights give) the loop
// falls back to the reference's full row and column updates.
template <int M>
__device__ int jacobi_row0( Smem<M> const &s, double *row0, unsigned &iters, unsigned cap, int log_cap,
                            unsigned *status )
{
    double const tol = DBL_EPSILON;
    unsigned it = 0;
    int nlog = 0;        // rotations in the log
    bool formed = false; // U formed: updated explicitly from here on
    // a basis function that vanishes on every neighbour (collinear or
    // coplanar rows) leaves a zero on the diagonal: such degenerate systems
    // keep the reference's updates throughout, since their truncation
    // decisions rest on rounding residuals
    bool sym = true;
#pragma unroll
    for ( int k = 0; k < M; ++k )
        sym = sym && s.e( k, k ) != 0.0;
    while ( true )
    {
        // Fused scan: first largest |E_ij| (integer compare of |bits|) and
        // FP32 bounds on the off-diagonal sum of squares from the exponents
        // alone: 4^e <= x^2 < 4^(e+1) for x in [2^e, 2^(e+1)).  Rows loop
        // (not unrolled) to keep the kernel's code small.  A symmetric E
        // counts its upper triangle twice.
        float lower = 0.f, upper = 0.f;
        bool huge = false, special = false;
        long long best = -1;
        int p = 0, q = 1;
        auto visit = [&]( int i, int j ) {
            long long const ab = abs_bits( s.e( i, j ) );
            if ( ab > best )
            {
                best = ab;
                p = i;
                q = j;
            }
            int const e = (int)( ab >> 52 ) - 1023; // -1023 for zero/subnormal
            special |= e == 1024;                   // Inf/NaN: decide exactly
            huge |= e > 62 && e < 1024;
            bool const mid = e >= -62 && e <= 62;
            lower += mid ? __int_as_float( ( 2 * e + 127 ) << 23 ) : 0.f;
            upper += mid ? __int_as_float( ( 2 * e + 129 ) << 23 )
                         : ( e < -62 ? 4.70197740328915e-38f : 0.f ); // 2^-124
        };
        if ( sym )
        {
            // the upper triangle in row-major order, unrolled
#pragma unroll
            for ( int i = 0; i < M; ++i )
#pragma unroll
                for ( int j = i + 1; j < M; ++j )
                    visit( i, j );
            lower *= 2.f;
            upper *= 2.f;
        }
        else
        {
#pragma unroll 1
            for ( int i = 0; i < M; ++i )
            {
#pragma unroll
                for ( int j = 0; j < M; ++j )
                    if ( j != i )
                        visit( i, j );
            }
        }
        // Stop test of the reference, sqrt(sum) > DBL_EPSILON, decided by the
        // bounds unless they straddle DBL_EPSILON^2 = 2^-104; then the FP64
        // row-major sum of squares as the reference forms it (twice the upper
        // triangle's for a symmetric E).
        constexpr float tol2 = 4.930380657631324e-32f; // 2^-104 exactly
        bool go;
        if ( !special && ( huge || lower > tol2 * 1.0009765625f ) )
            go = true;
        else if ( !special && upper < tol2 * 0.9990234375f )
            go = false;
        else
        {
            double acc = 0.0;
#pragma unroll
            for ( int i = 0; i < M; ++i )
#pragma unroll
                for ( int j = 0; j < M; ++j )
                    if ( i != j && !( sym && j < i ) )
                        acc = fma( s.e( i, j ), s.e( i, j ), acc );
            if ( sym )
                acc *= 2.0;
            go = sqrt( acc ) > tol;
        }
        if ( !go )
            break;
        if ( ++it > cap )
        {
            atomicOr( status, DEV_TIMEOUT );
            break;
        }
        if ( p > q )
        {
            int const tmp = p;
            p = q;
            q = tmp;
        }
        if ( !formed && nlog == log_cap )
        {
            form_u<M>( s, nlog );
            formed = true;
        }
        // a formed U's columns p and q are read before the 2x2 SVD and the E
        // updates, so that their loads (L2) are in flight during the FP64 work
        double up[M], uq[M];
        if ( formed )
        {
#pragma unroll
            for ( int j = 0; j < M; ++j )
            {
                up[j] = s.u( j, p );
                uq[j] = s.u( j, q );
            }
        }
        double cl, sl, cr, sr;
        double const bpp = s.e( p, p ), bpq = s.e( p, q ), bqp = s.e( q, p ), bqq = s.e( q, q );
        if ( sym )
            svd_2x2_sym( bpp, bpq, bqq, cl, sl, cr, sr );
        else
            svd_2x2( bpp, bpq, bqp, bqq, cl, sl, cr, sr );
        sym = sym && ieee_eq( cr, cl ) && ieee_eq( sr, sl );
        if ( sym )
        {
            // rows p and q by the left rotation, columns p and q off the
            // block copied from them, the block by the right rotation
#pragma unroll
            for ( int j = 0; j < M; ++j )
            {
                if ( j == p || j == q )
                    continue;
                double const a = s.e( p, j ), b = s.e( q, j );
                double const x = rot_minus( cl, sl, a, b ), y = rot_plus( cl, sl, a, b );
                s.e( p, j ) = x;
                s.e( q, j ) = y;
                s.e( j, p ) = x;
                s.e( j, q ) = y;
            }
            double const lpp = rot_minus( cl, sl, bpp, bqp ), lpq = rot_minus( cl, sl, bpq, bqq );
            double const lqp = rot_plus( cl, sl, bpp, bqp ), lqq = rot_plus( cl, sl, bpq, bqq );
            double const opq = rot_plus( cr, sr, lpp, lpq );
            s.e( p, p ) = rot_minus( cr, sr, lpp, lpq );
            s.e( p, q ) = opq;
            s.e( q, p ) = opq;
            s.e( q, q ) = rot_plus( cr, sr, lqp, lqq );
        }
        else
        {
            // givens_left(E, cl, sl, p, q)
#pragma unroll
            for ( int j = 0; j < M; ++j )
            {
                double const a = s.e( p, j ), b = s.e( q, j );
                s.e( p, j ) = rot_minus( cl, sl, a, b );
                s.e( q, j ) = rot_plus( cl, sl, a, b );
            }
            // givens_right(E, cr, sr, p, q)
#pragma unroll
            for ( int j = 0; j < M; ++j )
            {
                double const a = s.e( j, p ), b = s.e( j, q );
                s.e( j, p ) = rot_minus( cr, sr, a, b );
                s.e( j, q ) = rot_plus( cr, sr, a, b );
            }
        }
        // givens_right(U, cl, sl, p, q): logged, or applied to a formed U
        if ( formed )
        {
#pragma unroll
            for ( int j = 0; j < M; ++j )
            {
                double const a = up[j], b = uq[j];
                s.u( j, p ) = rot_minus( cl, sl, a, b );
                s.u( j, q ) = rot_plus( cl, sl, a, b );
            }
        }
        else
        {
            s.rot( nlog ) = make_double2( cl, sl );
            s.pivot( nlog ) = (uint8_t)( p * 16 + q );
            ++nlog;
        }
        // givens_left(V, cr, sr, p, q), column 0 only
        {
            double const a = s.v( p ), b = s.v( q );
            s.v( p ) = rot_minus( cr, sr, a, b );
            s.v( q ) = rot_plus( cr, sr, a, b );
        }
    }
    iters += it;
    // pinv(0, j) = sum_k V(k,0) U(j,k) / E(k,k) over |E(k,k)| >= DBL_EPSILON
    int dropped = 0;
    double w[M];
#pragma unroll
    for ( int k = 0; k < M; ++k )
    {
        double const ek = s.e( k, k );
        if ( fabs( ek ) >= tol )
            w[k] = s.v( k ) / ek;
        else
        {
            w[k] = 0.0;
            dropped = 1;
        }
    }
    if ( formed )
    {
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
            double v = 0.0;
#pragma unroll
            for ( int k = 0; k < M; ++k )
                v = fma( s.u( j, k ), w[k], v );
            row0[j] = v;
        }
        return dropped;
    }
    // U w = G_0 (G_1 (... (G_{n-1} w))) in V(:, 0)'s place: G = the right
    // rotation (c, s) of columns p and q, so (G z)_p = c z_p + s z_q and
    // (G z)_q = c z_q - s z_p; the log read four entries ahead
#pragma unroll
    for ( int k = 0; k < M; ++k )
        s.v( k ) = w[k];
    auto turn = [&]( double2 cs, int pq ) {
        int const p = pq >> 4, q = pq & 15;
        double const zp = s.v( p ), zq = s.v( q );
        s.v( p ) = rot_plus( cs.x, cs.y, zq, zp );
        s.v( q ) = rot_minus( cs.x, cs.y, zq, zp );
    };
    int r = nlog;
    for ( ; r >= 4; r -= 4 )
    {
        double2 cs[4];
        int pq[4];
#pragma unroll
        for ( int u = 0; u < 4; ++u )
        {
            cs[u] = s.rot( r - 1 - u );
            pq[u] = s.pivot( r - 1 - u );
        }
#pragma unroll
        for ( int u = 0; u < 4; ++u )
            turn( cs[u], pq[u] );
    }
    for ( ; r > 0; --r )
        turn( s.rot( r - 1 ), s.pivot( r - 1 ) );
#pragma unroll
    for ( int j = 0; j < M; ++j )
        row0[j] = s.v( j );
    return dropped;
}

// Persistent blocks of FP64_THREADS threads: a thread takes targets g,
// g + T, g + 2T, ... (T threads in the grid, g in the targets' Morton order).
// The rotation log (and U, for a target that outruns it) lives in u_work,
// jacobi_work_doubles( M ) doubles per resident thread (about 1.9 KB a
// target touched at M = 10, held in L2), so that E and V(:, 0), 880 B a
// thread in shared memory, let an SM hold 8 warps instead of 4: the FP64
// pipe then has a second warp per sub-partition to interleave with the
// argmax scans and the 2x2 SVD's dependency chain.
template <int M>
__global__ void __launch_bounds__( FP64_THREADS, 1 )
    k_setup_fp64( Neighbours nb, PointsView tgt, int32_t const *offset,
                  uint32_t const *order, int64_t n_tgt, int rbf, bool rows_sorted,
                  double *coeff, unsigned long long *under_count,
                  unsigned long long *rot_count, unsigned *status, unsigned jcap, int jlog, double *u_work )
{
    extern __shared__ double smem[];
    int const nt = blockDim.x; // FP64_THREADS, or 32 when the targets are few
    int64_t const T = (int64_t)gridDim.x * nt;
    int64_t const tid = blockIdx.x * (int64_t)nt + threadIdx.x;
    Smem<M> s{smem, u_work, smem + M * M * nt, (int)threadIdx.x, nt, tid, T};
    unsigned iters = 0;
    int dropped_all = 0;
    for ( int64_t g = tid; g - threadIdx.x < n_tgt; g += T ) // block-uniform trip count
    {
    int dropped = 0;
    if ( g < n_tgt )
    {
        int64_t const i = order ? (int64_t)order[g] : g;
        int64_t const b = offset[i];
        int len = offset[i + 1] - (int)b;
        for ( int j = 0; j < len; ++j )
            if ( (uint32_t)nb.ref( b + j ) >= (uint64_t)nb.src.n )
            {
                atomicOr( status, DEV_BAD_INDEX );
                len = 0;
            }
        double const tx = tgt( i, 0 ), ty = tgt( i, 1 ), tz = tgt( i, 2 );

        // computeRadius: the largest neighbour distance (last entry when the
        // row is sorted by distance).
        double d2max = 0.0;
        for ( int j = rows_sorted ? max( 0, len - 1 ) : 0; j < len; ++j )
        {
            double sx, sy, sz;
            nb.xyz( b + j, sx, sy, sz );
            d2max = fmax( d2max, dist2_rn( sx, sy, sz, tx, ty, tz ) );
        }
        double distance = 10. * DBL_EPSILON;
        double const dmax = __dsqrt_rn( d2max );
        if ( dmax > distance )
            distance = dmax;
        double const radius = 1.1 * distance;

        // computeMoments (upper triangle, registers)
        double A[M * ( M + 1 ) / 2];
#pragma unroll
        for ( int a = 0; a < M * ( M + 1 ) / 2; ++a )
            A[a] = 0.0;
        for ( int j = 0; j < len; ++j )
        {
            double sx, sy, sz;
            nb.xyz( b + j, sx, sy, sz );
            double const x = __dsub_rn( sx, tx ), y = __dsub_rn( sy, ty ), z = __dsub_rn( sz, tz );
            double P[M];
            basis_eval<M>( x, y, z, P );
            double const dist =
                __dsqrt_rn( __dadd_rn( __dadd_rn( __dmul_rn( x, x ), __dmul_rn( y, y ) ), __dmul_rn( z, z ) ) );
            double const phi = rbf_eval<double>( rbf, dist / radius );
            int o = 0;
#pragma unroll
            for ( int a = 0; a < M; ++a )
            {
                double const pa = P[a] * phi;
#pragma unroll
                for ( int c = a; c < M; ++c, ++o )
                    A[o] = fma( pa, P[c], A[o] );
            }
        }
        {
            int o = 0;
#pragma unroll
            for ( int a = 0; a < M; ++a )
#pragma unroll
                for ( int c = a; c < M; ++c )
                {
                    s.e( a, c ) = A[o];
                    s.e( c, a ) = A[o];
                    ++o;
                }
#pragma unroll
            for ( int a = 0; a < M; ++a )
                s.v( a ) = a == 0 ? 1.0 : 0.0;
        }
        double row0[M];
        dropped = jacobi_row0<M>( s, row0, iters, jcap, jlog, status );

        // computePolynomialCoefficients: c_k = phi_k * (row0 . P_k)
        for ( int j = 0; j < len; ++j )
        {
            double sx, sy, sz;
            nb.xyz( b + j, sx, sy, sz );
            double const x = __dsub_rn( sx, tx ), y = __dsub_rn( sy, ty ), z = __dsub_rn( sz, tz );
            double P[M];
            basis_eval<M>( x, y, z, P );
            double const dist =
                __dsqrt_rn( __dadd_rn( __dadd_rn( __dmul_rn( x, x ), __dmul_rn( y, y ) ), __dmul_rn( z, z ) ) );
            double const phi = rbf_eval<double>( rbf, dist / radius );
            double acc = 0.0;
#pragma unroll
            for ( int a = 0; a < M; ++a )
                acc = fma( row0[a], P[a], acc );
            coeff[b + j] = acc * phi;
        }
    }
    dropped_all += dropped;
    }
    // warp totals -> one atomic each
    unsigned long long it64 = iters, dr64 = dropped_all;
    for ( int o = 16; o; o >>= 1 )
    {
        it64 += __shfl_xor_sync( FULL, it64, o );
        dr64 += __shfl_xor_sync( FULL, dr64, o );
    }
    if ( ( threadIdx.x & 31 ) == 0 )
    {
        if ( it64 )
            atomicAdd( rot_count, it64 );
        if ( dr64 )
            atomicAdd( under_count, dr64 );
    }
}

// General-n SVDFunctor (one thread per matrix, E/U/V in a global work area):
// the batched pseudo-inverse kernel of DTK_DetailsSVDImpl.hpp:197-302.
__global__ void k_svd_general( int n, int64_t count, double const *a, double *pinv,
                               double *work, unsigned long long *under, unsigned *status,
                               unsigned long long cap )
{
    int64_t const mid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( mid >= count )
        return;
    int64_t const nn = (int64_t)n * n;
    double *E = work + 3 * nn * mid, *U = E + nn, *V = U + nn;
    double const *A = a + nn * mid;
    for ( int64_t i = 0; i < nn; ++i )
        E[i] = A[i];
    for ( int i = 0; i < n; ++i )
        for ( int j = 0; j < n; ++j )
        {
            U[i * n + j] = i == j ? 1.0 : 0.0;
            V[i * n + j] = i == j ? 1.0 : 0.0;
        }
    double const tol = DBL_EPSILON;
    unsigned long long it = 0;
    while ( true )
    {
        double acc = 0.0;
        long long best = -1;
        int p = 0, q = 1;
        for ( int i = 0; i < n; ++i )
            for ( int j = 0; j < n; ++j )
            {
                if ( i == j )
                    continue;
                double const x = E[i * n + j];
                acc = fma( x, x, acc );
                long long const ab = abs_bits( x );
                if ( ab > best )
                {
                    best = ab;
                    p = i;
                    q = j;
                }
            }
        if ( !( sqrt( acc ) > tol ) || n < 2 )
            break;
        if ( ++it > cap )
        {
            atomicOr( status, DEV_TIMEOUT );
            break;
        }
        if ( p > q )
        {
            int const t = p;
            p = q;
            q = t;
        }
        double cl, sl, cr, sr;
        svd_2x2( E[p * n + p], E[p * n + q], E[q * n + p], E[q * n + q], cl, sl, cr, sr );
        for ( int j = 0; j < n; ++j )
        {
            double const x = E[p * n + j], y = E[q * n + j];
            E[p * n + j] = rot_minus( cl, sl, x, y );
            E[q * n + j] = rot_plus( cl, sl, x, y );
        }
        for ( int j = 0; j < n; ++j )
        {
            double const x = E[j * n + p], y = E[j * n + q];
            E[j * n + p] = rot_minus( cr, sr, x, y );
            E[j * n + q] = rot_plus( cr, sr, x, y );
        }
        for ( int j = 0; j < n; ++j )
        {
            double const x = U[j * n + p], y = U[j * n + q];
            U[j * n + p] = rot_minus( cl, sl, x, y );
            U[j * n + q] = rot_plus( cl, sl, x, y );
        }
        for ( int j = 0; j < n; ++j )
        {
            double const x = V[p * n + j], y = V[q * n + j];
            V[p * n + j] = rot_minus( cr, sr, x, y );
            V[q * n + j] = rot_plus( cr, sr, x, y );
        }
    }
    int dropped = 0;
    double *out = pinv + nn * mid;
    for ( int i = 0; i < n; ++i )
        for ( int j = 0; j < n; ++j )
        {
            double v = 0.0;
            for ( int k = 0; k < n; ++k )
            {
                double const ek = E[k * n + k];
                if ( fabs( ek ) >= tol )
                    v += V[k * n + i] * U[j * n + k] / ek;
                else
                    dropped = 1;
            }
            out[i * n + j] = v;
        }
    if ( dropped )
        atomicAdd( under, 1ull );
}

// ---------------------------------------------------------------------------
// Persistent batched setup: every FP64-Jacobi target of a batch, of any
// (basis, rbf) and row length, in one launch.  A warp takes tasks from a
// counter; a task is up to 32 targets of one bucket (same basis and rbf) and
// a lane count G: G lanes per target gather the neighbours for the radius and
// the moments (sums combined by shuffles in the group), the moments go to the
// owning lane's column of the warp's shared-memory E, every lane runs the
// reference Jacobi on its own target, and G lanes per target write the
// coefficients.  With G = 1 a lane walks its target's row alone, in entry
// order: the same arithmetic as k_setup_fp64, so the coefficients equal the
// single operator's bit for bit.
// ---------------------------------------------------------------------------
constexpr int BS_SLOT = ( BS_MAX_M * BS_MAX_M + BS_MAX_M ) * 32; // doubles a warp: E and V(:, 0), by lane

template <int M>
__device__ void setup_task( BatchSetupArgs const &a, SetupTask const &t, int rbf, int G, double *wsm,
                            int64_t ut, int64_t us, unsigned jcap, unsigned &iters, int &dropped, int lane )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    int const per = 32 / G, sub = lane & ( G - 1 ), cnt = t.count;
    double my_radius = 0.0;
    // the moments, G lanes a target, into column ti of E
    for ( int r = 0; r * per < cnt; ++r ) // warp-uniform
    {
        int const ti = r * per + lane / G;
        bool const active = ti < cnt;
        int64_t const i = active ? (int64_t)a.list[t.first + ti] : 0;
        int64_t const b = active ? a.offset[i] : 0;
        int len = active ? a.offset[i + 1] - (int)b : 0;
        double const tx = active ? a.tgt( i, 0 ) : 0.0, ty = active ? a.tgt( i, 1 ) : 0.0,
                     tz = active ? a.tgt( i, 2 ) : 0.0;
        bool bad = false;
        for ( int j = sub; j < len; j += G )
            bad |= (uint32_t)a.nb.ref( b + j ) >= (uint64_t)a.nb.src.n;
        for ( int o = G >> 1; o; o >>= 1 )
            bad |= __shfl_xor_sync( FULL, (int)bad, o ) != 0;
        if ( bad )
        {
            if ( sub == 0 )
                atomicOr( a.status, DEV_BAD_INDEX );
            len = 0;
        }
        // computeRadius: the farthest neighbour (the last of a row sorted by
        // distance)
        double d2max = 0.0;
        for ( int j = a.rows_sorted ? ( sub == 0 ? max( 0, len - 1 ) : len ) : sub; j < len; j += G )
        {
            double sx, sy, sz;
            a.nb.xyz( b + j, sx, sy, sz );
            d2max = fmax( d2max, dist2_rn( sx, sy, sz, tx, ty, tz ) );
        }
        for ( int o = G >> 1; o; o >>= 1 )
            d2max = fmax( d2max, __shfl_xor_sync( FULL, d2max, o ) );
        double distance = 10. * DBL_EPSILON;
        double const dmax = __dsqrt_rn( d2max );
        if ( dmax > distance )
            distance = dmax;
        double const radius = 1.1 * distance;
        double A[NU];
#pragma unroll
        for ( int u = 0; u < NU; ++u )
            A[u] = 0.0;
        for ( int j = sub; j < len; j += G )
        {
            double sx, sy, sz;
            a.nb.xyz( b + j, sx, sy, sz );
            double const x = __dsub_rn( sx, tx ), y = __dsub_rn( sy, ty ), z = __dsub_rn( sz, tz );
            double P[M];
            basis_eval<M>( x, y, z, P );
            double const dist =
                __dsqrt_rn( __dadd_rn( __dadd_rn( __dmul_rn( x, x ), __dmul_rn( y, y ) ), __dmul_rn( z, z ) ) );
            double const phi = rbf_eval<double>( rbf, dist / radius );
            int o = 0;
#pragma unroll
            for ( int p = 0; p < M; ++p )
            {
                double const pa = P[p] * phi;
#pragma unroll
                for ( int c = p; c < M; ++c, ++o )
                    A[o] = fma( pa, P[c], A[o] );
            }
        }
        if ( G > 1 )
        {
#pragma unroll
            for ( int u = 0; u < NU; ++u )
                for ( int o = G >> 1; o; o >>= 1 )
                    A[u] += __shfl_xor_sync( FULL, A[u], o );
        }
        if ( active )
        {
            int o = 0;
#pragma unroll
            for ( int p = 0; p < M; ++p )
#pragma unroll
                for ( int c = p; c < M; ++c, ++o )
                    if ( ( o & ( G - 1 ) ) == sub )
                    {
                        wsm[( p * M + c ) * 32 + ti] = A[o];
                        wsm[( c * M + p ) * 32 + ti] = A[o];
                    }
        }
        // the radius to the target's own lane
        double const rv = __shfl_sync( FULL, radius, ( lane % per ) * G );
        if ( lane / per == r )
            my_radius = rv;
    }
    __syncwarp();
    // the reference Jacobi, a target a lane; row 0 of the pseudo-inverse
    // replaces V(:, 0) in the lane's column
    Smem<M> sm{wsm, a.u_work, wsm + M * M * 32, lane, 32, ut, us};
    if ( lane < cnt )
    {
#pragma unroll
        for ( int p = 0; p < M; ++p )
            sm.v( p ) = p == 0 ? 1.0 : 0.0;
        double row0[M];
        dropped += jacobi_row0<M>( sm, row0, iters, jcap, a.jlog, a.status );
#pragma unroll
        for ( int p = 0; p < M; ++p )
            sm.v( p ) = row0[p];
    }
    __syncwarp();
    // computePolynomialCoefficients, G lanes a target
    for ( int r = 0; r * per < cnt; ++r )
    {
        int const ti = r * per + lane / G;
        double const radius = __shfl_sync( FULL, my_radius, ti & 31 );
        if ( ti >= cnt )
            continue;
        int64_t const i = a.list[t.first + ti];
        int64_t const b = a.offset[i];
        int const len = a.offset[i + 1] - (int)b;
        double const tx = a.tgt( i, 0 ), ty = a.tgt( i, 1 ), tz = a.tgt( i, 2 );
        double row0[M];
#pragma unroll
        for ( int p = 0; p < M; ++p )
            row0[p] = wsm[M * M * 32 + p * 32 + ti];
        for ( int j = sub; j < len; j += G )
        {
            if ( (uint32_t)a.nb.ref( b + j ) >= (uint64_t)a.nb.src.n )
                continue; // reported above
            double sx, sy, sz;
            a.nb.xyz( b + j, sx, sy, sz );
            double const x = __dsub_rn( sx, tx ), y = __dsub_rn( sy, ty ), z = __dsub_rn( sz, tz );
            double P[M];
            basis_eval<M>( x, y, z, P );
            double const dist =
                __dsqrt_rn( __dadd_rn( __dadd_rn( __dmul_rn( x, x ), __dmul_rn( y, y ) ), __dmul_rn( z, z ) ) );
            double const phi = rbf_eval<double>( rbf, dist / radius );
            double acc = 0.0;
#pragma unroll
            for ( int p = 0; p < M; ++p )
                acc = fma( row0[p], P[p], acc );
            if ( a.coeff32 )
                a.coeff32[b + j] = (float)( acc * phi );
            else
                a.coeff64[b + j] = acc * phi;
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__( BS_WARPS * 32, 1 ) k_batch_setup( BatchSetupArgs a )
{
    extern __shared__ double smem[];
    int const lane = threadIdx.x & 31;
    double *const wsm = smem + (size_t)( threadIdx.x >> 5 ) * BS_SLOT;
    int64_t const ut = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const us = (int64_t)gridDim.x * blockDim.x;
    int64_t const t_end = a.t_end >= 0 ? a.t_end : *a.n_tasks;
    unsigned iters = 0;
    int dropped = 0;
    for ( ;; )
    {
        unsigned c = 0;
        if ( lane == 0 )
            c = atomicAdd( a.counter, 1u );
        int64_t const ti = a.t_begin + __shfl_sync( FULL, c, 0 );
        if ( ti >= t_end )
            break;
        SetupTask const t = a.tasks[ti];
        int const key = t.key;
        int const basis = key / SETUP_PATHS / SETUP_RBFS, rbf = key / SETUP_PATHS % SETUP_RBFS;
        int const G = a.force_lanes ? a.force_lanes : t.lanes;
        // a task out of range is reported and skipped, never followed
        if ( key >= SETUP_KEYS || t.count < 1 || t.count > 32 || G < 1 || G > 32 || ( G & ( G - 1 ) ) ||
             t.first < 0 || (int64_t)t.first + t.count > a.n_list )
        {
            if ( lane == 0 )
                atomicOr( a.status, DEV_BAD_TASK );
            continue;
        }
        if ( basis == DTK_CONSTANT3 )
            setup_task<1>( a, t, rbf, G, wsm, ut, us, a.jcap[0], iters, dropped, lane );
        else if ( basis == DTK_LINEAR3 )
            setup_task<4>( a, t, rbf, G, wsm, ut, us, a.jcap[1], iters, dropped, lane );
        else
            setup_task<10>( a, t, rbf, G, wsm, ut, us, a.jcap[2], iters, dropped, lane );
    }
    unsigned long long it64 = iters, dr64 = dropped;
    for ( int o = 16; o; o >>= 1 )
    {
        it64 += __shfl_xor_sync( FULL, it64, o );
        dr64 += __shfl_xor_sync( FULL, dr64, o );
    }
    if ( lane == 0 )
    {
        if ( it64 )
            atomicAdd( a.rotations, it64 );
        if ( dr64 )
            atomicAdd( a.underdetermined, dr64 );
    }
}

template <int M>
void launch_fp64( SetupArgs const &a, cudaStream_t s )
{
    JacobiGrid const jg = jacobi_grid<M>( a.n_tgt );
    ensure_dynamic_smem( k_setup_fp64<M>, jg.smem );
    DeviceBuffer<double> u_work( (size_t)jacobi_work_doubles( M ) * jg.threads * jg.blocks, s );
    Neighbours const nb{a.src, a.idx, a.pos, a.s2};
    k_setup_fp64<M><<<jg.blocks, jg.threads, jg.smem, s>>>( nb, a.tgt, a.offset, a.order,
                                                         a.n_tgt, a.rbf, a.rows_sorted, a.coeff64,
                                                         a.underdetermined, a.rotations, a.status,
                                                         (unsigned)jacobi_cap( M ), jacobi_log_cap(),
                                                         u_work.get() );
    check_launch( "k_setup_fp64" );
}

} // namespace

void setup_fp64( SetupArgs const &a, cudaStream_t s )
{
    NvtxRange const nvtx_range( "DTK_compute_polynomial_coeffs" );
    if ( a.n_tgt == 0 )
        return;
    switch ( a.basis )
    {
    case DTK_CONSTANT3:
        launch_fp64<1>( a, s );
        break;
    case DTK_LINEAR3:
        launch_fp64<4>( a, s );
        break;
    default:
        launch_fp64<10>( a, s );
        break;
    }
}

size_t batch_setup_smem()
{
    return (size_t)BS_WARPS * BS_SLOT * sizeof( double );
}

int64_t batch_setup_threads()
{
    return (int64_t)num_sms() * BS_WARPS * 32;
}

void batch_setup( BatchSetupArgs const &args, cudaStream_t s )
{
    NvtxRange const nvtx_range( "DTK_compute_polynomial_coeffs" );
    BatchSetupArgs a = args;
    a.jcap[0] = (unsigned)jacobi_cap( 1 );
    a.jcap[1] = (unsigned)jacobi_cap( 4 );
    a.jcap[2] = (unsigned)jacobi_cap( 10 );
    a.jlog = jacobi_log_cap();
    ensure_dynamic_smem( k_batch_setup, batch_setup_smem() );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( a.counter, 0, sizeof( unsigned ), s ) );
    k_batch_setup<<<(unsigned)num_sms(), BS_WARPS * 32, batch_setup_smem(), s>>>( a );
    check_launch( "k_batch_setup" );
}

void svd_pinv_batched_work( int n, int64_t count, double const *a, double *pinv, double *work,
                            unsigned long long *underdetermined, unsigned *status, cudaStream_t s )
{
    if ( count == 0 )
        return;
    unsigned const blocks = (unsigned)( ( count + 63 ) / 64 );
    k_svd_general<<<blocks, 64, 0, s>>>( n, count, a, pinv, work, underdetermined, status, jacobi_cap( n ) );
    check_launch( "k_svd_general" );
}

void svd_pinv_batched( int n, int64_t count, double const *a, double *pinv,
                       unsigned long long *underdetermined, unsigned *status, cudaStream_t s )
{
    if ( count == 0 )
        return;
    DeviceBuffer<double> work( 3 * (size_t)n * n * count, s );
    unsigned const blocks = (unsigned)( ( count + 63 ) / 64 );
    k_svd_general<<<blocks, 64, 0, s>>>( n, count, a, pinv, work.get(), underdetermined, status,
                                         jacobi_cap( n ) );
    check_launch( "k_svd_general" );
}

} // namespace dtk
