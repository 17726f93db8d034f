// Adjoint of the MLS transfer (extension; the reference has none).
//
// For L with dL/d(target values) = cot:
//   dL/d(source values) = C^T cot, C the operator's CSR coefficients.  The
//     transpose (source -> its entries) is built once per handle by a stable
//     radix sort of (source index, entry), so each source sums its entries
//     in ascending entry order: deterministic, no atomics.
//   dL/d(source coordinates): per target, with x_j = s_j - t, rho_j = |x_j|,
//     R = 1.1 max(10 eps, max rho), phi_j = rbf(rho_j / R),
//     A = sum phi P P^T, a = A^+ e0, z = A^+ b, b = sum phi_j v_j P_j, y = a.b,
//     and in the radius-scaled frame (x^ = x / R, P^ = P(x^), J^ = dP^/dx^):
//       dy/dx_j = (phi_j / R) J^_j^T (e_j a^ - alpha_j z^) + (g_j / R) u_j
//                 - [j farthest] 1.1 (sum_l g_l rho^_l) / R u_j
//     with alpha_j = a^.P^_j, e_j = v_j - P^_j.z^, g_j = alpha_j e_j rbf'(rho^_j),
//     u_j = x_j / rho_j; the radius max sends its gradient to the farthest
//     neighbour (the last of largest rho in row order).  The per-entry
//     contributions cot_i dy/dx_j are written once and gathered through the
//     same transpose.  The pseudo-inverse is recomputed per target (never
//     stored) from FP64 scaled moments.  Well-conditioned targets take an
//     FP64 Cholesky (A^+ = A^-1 there); the rest take an FP32 round-robin
//     Jacobi, one FP64 sweep on B = V32^T A V32 and truncation at 2^-40 of
//     the largest eigenvalue.  Both end with one FP64 refinement step for a^
//     and z^ each.
#include "dtk_common.cuh"
#include "dtk_handle.cuh"
#include "dtk_jacobi.cuh"

#include <algorithm>
#include <new>

namespace dtk
{
namespace
{

constexpr int AB = 32; // threads per block of the coordinate kernel

__global__ void k_entry_pairs( int32_t const *idx, int64_t nnz, uint32_t *keys, uint32_t *vals )
{
    int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( e < nnz )
    {
        keys[e] = (uint32_t)idx[e];
        vals[e] = (uint32_t)e;
    }
}

__global__ void k_source_counts( uint32_t const *sorted_keys, int64_t nnz, int64_t *counts )
{
    int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( e < nnz )
        atomicAdd( reinterpret_cast<unsigned long long *>( counts + sorted_keys[e] ), 1ull );
}

__global__ void k_narrow( int64_t const *in, int32_t *out, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        out[i] = (int32_t)in[i];
}

__global__ void k_entry_rows( int32_t const *offset, int64_t n_tgt, int32_t *row_of )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < n_tgt )
        for ( int e = offset[i]; e < offset[i + 1]; ++e )
            row_of[e] = (int32_t)i;
}

// One thread per source: grad_values[s] = sum_e coeff[e] cot[row(e)] and
// grad_coords[s] = sum_e contrib[e] over the source's entries, ascending.
template <bool F32>
__global__ void k_transpose_gather( int64_t n_src, int32_t const *t_offset, int32_t const *t_entry,
                                    int uniform_row, int32_t const *row_of, void const *coeff,
                                    double const *cot, double const *contrib, double *grad_values,
                                    double *grad_coords )
{
    int64_t const s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( s >= n_src )
        return;
    double gv = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    for ( int q = t_offset[s]; q < t_offset[s + 1]; ++q )
    {
        int64_t const e = t_entry[q];
        int64_t const row = uniform_row > 0 ? e / uniform_row : row_of[e];
        double const c = F32 ? (double)static_cast<float const *>( coeff )[e]
                             : static_cast<double const *>( coeff )[e];
        gv = fma( c, cot[row], gv );
        if ( contrib )
        {
            gx += contrib[3 * e + 0];
            gy += contrib[3 * e + 1];
            gz += contrib[3 * e + 2];
        }
    }
    grad_values[s] = gv;
    if ( grad_coords )
    {
        grad_coords[3 * s + 0] = gx;
        grad_coords[3 * s + 1] = gy;
        grad_coords[3 * s + 2] = gz;
    }
}

// Jacobian of the scaled basis: row c of dP/dx^ at x^ (3 entries).
template <int M>
__device__ __forceinline__ void basis_jac_row( int c, double x, double y, double z, double *g )
{
    g[0] = g[1] = g[2] = 0.0;
    if constexpr ( M >= 4 )
    {
        if ( c >= 1 && c <= 3 )
            g[c - 1] = 1.0;
    }
    if constexpr ( M == 10 )
    {
        switch ( c )
        {
        case 4: g[0] = 2.0 * x; break;
        case 5: g[0] = y; g[1] = x; break;
        case 6: g[0] = z; g[2] = x; break;
        case 7: g[1] = 2.0 * y; break;
        case 8: g[1] = z; g[2] = y; break;
        case 9: g[2] = 2.0 * z; break;
        default: break;
        }
    }
}

// Per-target pieces shared by the two coordinate-adjoint kernels.
struct AdjTarget
{
    int64_t i, b0;
    int len, far;
    bool radius_live;
    double tx, ty, tz, ci, inv_r;
};

// Returns false when the target needs no more work (no entries, a zero
// cotangent: its contributions are zero, or a bad index: reported).
__device__ __forceinline__ bool adjoint_prologue( int64_t i, double const *src, double const *tgt,
                                                 int32_t const *offset, int32_t const *idx, int64_t n_src,
                                                 double const *cot, double *contrib, unsigned *status,
                                                 AdjTarget &T )
{
    T.i = i;
    T.b0 = offset[i];
    T.len = offset[i + 1] - (int)T.b0;
    T.ci = cot[i];
    if ( T.len == 0 )
        return false;
    for ( int j = 0; j < T.len; ++j )
        if ( (uint32_t)idx[T.b0 + j] >= (uint64_t)n_src )
        {
            atomicOr( status, DEV_BAD_INDEX );
            return false;
        }
    if ( T.ci == 0.0 )
    {
        for ( int j = 0; j < T.len; ++j )
            contrib[3 * ( T.b0 + j )] = contrib[3 * ( T.b0 + j ) + 1] = contrib[3 * ( T.b0 + j ) + 2] = 0.0;
        return false;
    }
    T.tx = tgt[3 * i];
    T.ty = tgt[3 * i + 1];
    T.tz = tgt[3 * i + 2];
    // radius and the farthest neighbour (last of largest distance)
    double dmax = 0.0;
    T.far = 0;
    for ( int j = 0; j < T.len; ++j )
    {
        int64_t const sj = idx[T.b0 + j];
        double const x = src[3 * sj] - T.tx, y = src[3 * sj + 1] - T.ty, z = src[3 * sj + 2] - T.tz;
        double const d = sqrt( ( x * x + y * y ) + z * z );
        if ( d >= dmax )
        {
            dmax = d;
            T.far = j;
        }
    }
    double const floor_d = 10. * DBL_EPSILON;
    T.radius_live = dmax > floor_d;
    T.inv_r = 1.0 / ( 1.1 * ( T.radius_live ? dmax : floor_d ) );
    return true;
}

// Scaled moments A^ (upper triangle) and b^ = sum phi v P^ (FP64).
template <int M>
__device__ __forceinline__ void adjoint_moments( AdjTarget const &T, double const *src, int32_t const *idx,
                                                 int rbf, double const *values, double *A, double *bh )
{
    constexpr int NU = M * ( M + 1 ) / 2;
#pragma unroll
    for ( int u = 0; u < NU; ++u )
        A[u] = 0.0;
#pragma unroll
    for ( int c = 0; c < M; ++c )
        bh[c] = 0.0;
    for ( int j = 0; j < T.len; ++j )
    {
        int64_t const sj = idx[T.b0 + j];
        double const x = ( src[3 * sj] - T.tx ) * T.inv_r, y = ( src[3 * sj + 1] - T.ty ) * T.inv_r,
                     z = ( src[3 * sj + 2] - T.tz ) * T.inv_r;
        double P[M];
        basis_eval<M, double>( x, y, z, P );
        double const phi = rbf_eval<double>( rbf, sqrt( ( x * x + y * y ) + z * z ) );
        double const pv = phi * values[sj];
#pragma unroll
        for ( int a = 0; a < M; ++a )
        {
            double const pa = phi * P[a];
            bh[a] = fma( pv, P[a], bh[a] );
#pragma unroll
            for ( int c = a; c < M; ++c )
                A[ut<M>( a, c )] = fma( pa, P[c], A[ut<M>( a, c )] );
        }
    }
}

// Given a^ = A^+ e0 and z^ = A^+ b^: pass 1, S = sum g_l rho^_l; pass 2, the
// per-entry contributions cot_i dy/dx_j.
template <int M>
__device__ __forceinline__ void adjoint_passes( AdjTarget const &T, double const *src, int32_t const *idx,
                                                int rbf, double const *values, double const *ah,
                                                double const *zh, double *contrib )
{
    double S = 0.0;
    for ( int j = 0; j < T.len; ++j )
    {
        int64_t const sj = idx[T.b0 + j];
        double const x = ( src[3 * sj] - T.tx ) * T.inv_r, y = ( src[3 * sj + 1] - T.ty ) * T.inv_r,
                     z = ( src[3 * sj + 2] - T.tz ) * T.inv_r;
        double P[M];
        basis_eval<M, double>( x, y, z, P );
        double const rh = sqrt( ( x * x + y * y ) + z * z );
        double al = 0.0, pz = 0.0;
#pragma unroll
        for ( int c = 0; c < M; ++c )
        {
            al = fma( ah[c], P[c], al );
            pz = fma( P[c], zh[c], pz );
        }
        double const e = values[sj] - pz;
        S = fma( al * e * rbf_deriv( rbf, rh ), rh, S );
    }
    for ( int j = 0; j < T.len; ++j )
    {
        int64_t const sj = idx[T.b0 + j];
        double x = src[3 * sj] - T.tx, y = src[3 * sj + 1] - T.ty, z = src[3 * sj + 2] - T.tz;
        double const rho = sqrt( ( x * x + y * y ) + z * z );
        double const ux = rho > 0.0 ? x / rho : 0.0, uy = rho > 0.0 ? y / rho : 0.0,
                     uz = rho > 0.0 ? z / rho : 0.0;
        x *= T.inv_r;
        y *= T.inv_r;
        z *= T.inv_r;
        double P[M];
        basis_eval<M, double>( x, y, z, P );
        double const rh = sqrt( ( x * x + y * y ) + z * z );
        double const phi = rbf_eval<double>( rbf, rh );
        double al = 0.0, pz = 0.0;
#pragma unroll
        for ( int c = 0; c < M; ++c )
        {
            al = fma( ah[c], P[c], al );
            pz = fma( P[c], zh[c], pz );
        }
        double const e = values[sj] - pz;
        double const gj = al * e * rbf_deriv( rbf, rh );
        double G[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for ( int c = 1; c < M; ++c )
        {
            double jr[3];
            basis_jac_row<M>( c, x, y, z, jr );
            double const w = e * ah[c] - al * zh[c];
            G[0] = fma( w, jr[0], G[0] );
            G[1] = fma( w, jr[1], G[1] );
            G[2] = fma( w, jr[2], G[2] );
        }
        double coef = gj;
        if ( j == T.far && T.radius_live )
            coef -= 1.1 * S;
        double const sp = phi * T.inv_r, sc = coef * T.inv_r;
        contrib[3 * ( T.b0 + j ) + 0] = T.ci * ( sp * G[0] + sc * ux );
        contrib[3 * ( T.b0 + j ) + 1] = T.ci * ( sp * G[1] + sc * uy );
        contrib[3 * ( T.b0 + j ) + 2] = T.ci * ( sp * G[2] + sc * uz );
    }
}

// Fast path, one thread per target: FP64 Cholesky A^ = R^T R and S = R^-1,
// in place in a per-thread shared-memory work area (in registers they spill
// at M = 10); a^ and z^ as S (S^T v) with one refinement step against the
// moments (also kept in shared memory).  Taken when the factorization succeeds
// and trace(A^) ||S||_F^2 <= 2^39, a bound on cond(A^) below the eigen path's
// 2^-40 truncation, so A^+ = A^-1; other targets are listed for the eigen
// path.
constexpr int AF = 32; // threads per block of the fast kernel

template <int M>
__global__ void __launch_bounds__( AF )
    k_adjoint_fast( double const *src, double const *tgt, int32_t const *offset, int32_t const *idx,
                    uint32_t const *order, int64_t n_tgt, int64_t n_src, int rbf, double const *values,
                    double const *cot, double *contrib, int32_t *list, unsigned *count, unsigned *status )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    // per thread, interleaved: NU moments, M of b^, NU of the Cholesky work area
    extern __shared__ double s_mom[];
    auto Wk = [&]( int u ) -> double & { return s_mom[( NU + M + u ) * AF + threadIdx.x]; };
    int64_t const g = blockIdx.x * (int64_t)AF + threadIdx.x;
    if ( g >= n_tgt )
        return;
    int64_t const i = order ? (int64_t)order[g] : g;
    AdjTarget T;
    if ( !adjoint_prologue( i, src, tgt, offset, idx, n_src, cot, contrib, status, T ) )
        return;
    double A[NU];
    {
        double bh[M];
        adjoint_moments<M>( T, src, idx, rbf, values, A, bh );
#pragma unroll
        for ( int c = 0; c < M; ++c )
            s_mom[( NU + c ) * AF + threadIdx.x] = bh[c];
    }
    double trace = 0.0;
#pragma unroll
    for ( int u = 0; u < NU; ++u )
    {
        s_mom[u * AF + threadIdx.x] = A[u];
        Wk( u ) = A[u];
    }
#pragma unroll
    for ( int k = 0; k < M; ++k )
        trace += A[ut<M>( k, k )];
    // Cholesky in place (R upper, row-major packed), then S = R^-1 in place
    bool ok = trace > 0.0;
    {
        double rinv[M];
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
            double d = Wk( ut<M>( j, j ) );
#pragma unroll
            for ( int k = 0; k < j; ++k )
                d = fma( -Wk( ut<M>( k, j ) ), Wk( ut<M>( k, j ) ), d );
            ok = ok && d > 0.0;
            double const r = d > 0.0 ? sqrt( d ) : 1.0;
            rinv[j] = 1.0 / r;
            Wk( ut<M>( j, j ) ) = r;
#pragma unroll
            for ( int c = j + 1; c < M; ++c )
            {
                double v = Wk( ut<M>( j, c ) );
#pragma unroll
                for ( int k = 0; k < j; ++k )
                    v = fma( -Wk( ut<M>( k, j ) ), Wk( ut<M>( k, c ) ), v );
                Wk( ut<M>( j, c ) ) = v * rinv[j];
            }
        }
#pragma unroll
        for ( int j = 0; j < M; ++j )
        {
#pragma unroll
            for ( int r = 0; r < j; ++r )
            {
                double v = 0.0;
#pragma unroll
                for ( int k = r; k < j; ++k )
                    v = fma( Wk( ut<M>( r, k ) ), Wk( ut<M>( k, j ) ), v );
                Wk( ut<M>( r, j ) ) = -v * rinv[j];
            }
            Wk( ut<M>( j, j ) ) = rinv[j];
        }
    }
    double fro = 0.0;
#pragma unroll
    for ( int u = 0; u < NU; ++u )
        fro = fma( Wk( u ), Wk( u ), fro );
    if ( !ok || !( trace * fro <= 549755813888.0 ) ) // 2^39; false for NaN
    {
        list[atomicAdd( count, 1u )] = (int32_t)i;
        return;
    }
    // x = S (S^T v)
    auto apply_inv = [&]( double const *v, double *x ) {
        double w[M];
#pragma unroll
        for ( int k = 0; k < M; ++k )
        {
            double acc = 0.0;
#pragma unroll
            for ( int r = 0; r <= k; ++r )
                acc = fma( Wk( ut<M>( r, k ) ), v[r], acc );
            w[k] = acc;
        }
#pragma unroll
        for ( int r = 0; r < M; ++r )
        {
            double acc = 0.0;
#pragma unroll
            for ( int k = r; k < M; ++k )
                acc = fma( Wk( ut<M>( r, k ) ), w[k], acc );
            x[r] = acc;
        }
    };
    // right-hand side rhs_r = (r == 0) for e0, else b^ from shared memory
    auto solve = [&]( bool unit, double *x ) {
        double v[M];
#pragma unroll
        for ( int r = 0; r < M; ++r )
            v[r] = unit ? ( r == 0 ? 1.0 : 0.0 ) : s_mom[( NU + r ) * AF + threadIdx.x];
        apply_inv( v, x );
#pragma unroll
        for ( int r = 0; r < M; ++r )
        {
            double acc = unit ? ( r == 0 ? 1.0 : 0.0 ) : s_mom[( NU + r ) * AF + threadIdx.x];
#pragma unroll
            for ( int c = 0; c < M; ++c )
                acc = fma( -s_mom[ut<M>( r, c ) * AF + threadIdx.x], x[c], acc );
            v[r] = acc;
        }
        double d[M];
        apply_inv( v, d );
#pragma unroll
        for ( int r = 0; r < M; ++r )
            x[r] += d[r];
    };
    double ah[M], zh[M];
    solve( true, ah );
    solve( false, zh );
    adjoint_passes<M>( T, src, idx, rbf, values, ah, zh, contrib );
}

// Eigen path over the targets the fast path listed (list[0 .. *count),
// persistent blocks): FP32 Jacobi, B = V32^T A V32, one FP64 sweep,
// truncation at 2^-40 of the largest eigenvalue, one FP64 refinement step.
template <int M>
__global__ void __launch_bounds__( AB )
    k_adjoint_entries( double const *src, double const *tgt, int32_t const *offset, int32_t const *idx,
                       int32_t const *list, unsigned const *count, int64_t n_src, int rbf,
                       double const *values, double const *cot, double *contrib, unsigned *status )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    extern __shared__ unsigned char smem_raw[];
    // per thread, interleaved: A64 (NU doubles), B (NU doubles; A32 first),
    // W (M*M doubles), V32 (M*M floats)
    double *sa = reinterpret_cast<double *>( smem_raw );
    double *sb = sa + NU * AB;
    double *sw = sb + NU * AB;
    float *sv = reinterpret_cast<float *>( sw + M * M * AB );
    int const t = threadIdx.x;
    auto A64 = [&]( int u ) -> double & { return sa[u * AB + t]; };
    auto B = [&]( int u ) -> double & { return sb[u * AB + t]; };
    auto A32 = [&]( int u ) -> float & { return reinterpret_cast<float *>( sb )[u * AB + t]; };
    auto W = [&]( int r, int c ) -> double & { return sw[( r * M + c ) * AB + t]; };
    auto V32 = [&]( int r, int c ) -> float & { return sv[( r * M + c ) * AB + t]; };

    int64_t const n_list = *count;
    for ( int64_t g = blockIdx.x * (int64_t)AB + threadIdx.x; g < n_list; g += (int64_t)gridDim.x * AB )
    {
        AdjTarget T;
        if ( !adjoint_prologue( list[g], src, tgt, offset, idx, n_src, cot, contrib, status, T ) )
            continue;
        double bh[M];
        {
            double A[NU];
            adjoint_moments<M>( T, src, idx, rbf, values, A, bh );
#pragma unroll
            for ( int u = 0; u < NU; ++u )
            {
                A64( u ) = A[u];
                A32( u ) = (float)A[u];
            }
        }
#pragma unroll
        for ( int r = 0; r < M; ++r )
#pragma unroll
            for ( int c = 0; c < M; ++c )
                V32( r, c ) = r == c ? 1.f : 0.f;
        for ( int sweep = 0; sweep < 12; ++sweep )
            if ( jacobi_sweep<M, float>( A32, V32, 1e-7f ) == 0 )
                break;
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
#pragma unroll
        for ( int r = 0; r < M; ++r )
#pragma unroll
            for ( int c = 0; c < M; ++c )
                W( r, c ) = (double)V32( r, c );
        jacobi_sweep<M, double>( B, W, 1e-15 );
        double lmax = 0.0;
        for ( int k = 0; k < M; ++k )
            lmax = fmax( lmax, fabs( B( ut<M>( k, k ) ) ) );
        double const cut = lmax * 9.094947017729282e-13; // 2^-40
        for ( int k = 0; k < M; ++k )
        {
            double const lk = B( ut<M>( k, k ) );
            B( ut<M>( k, k ) ) = ( fabs( lk ) > cut && lk != 0.0 ) ? 1.0 / lk : 0.0;
        }
        // y += A^+ v, then one refinement step against the FP64 moments
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
        auto solve = [&]( double const *rhs, double *x ) {
#pragma unroll
            for ( int r = 0; r < M; ++r )
                x[r] = 0.0;
            pinv_add( rhs, x );
            double res[M];
#pragma unroll
            for ( int r = 0; r < M; ++r )
            {
                double acc = rhs[r];
#pragma unroll
                for ( int c = 0; c < M; ++c )
                    acc = fma( -A64( ut<M>( r, c ) ), x[c], acc );
                res[r] = acc;
            }
            pinv_add( res, x );
        };
        double e0[M], ah[M], zh[M];
#pragma unroll
        for ( int r = 0; r < M; ++r )
            e0[r] = r == 0 ? 1.0 : 0.0;
        solve( e0, ah );
        solve( bh, zh );
        adjoint_passes<M>( T, src, idx, rbf, values, ah, zh, contrib );
    }
}

template <int M>
void launch_adjoint_entries( dtk_mls_s const *h, double const *values, double const *cot,
                             double *contrib, unsigned *status, cudaStream_t s )
{
    constexpr int NU = M * ( M + 1 ) / 2;
    DeviceBuffer<int32_t> list( std::max<int64_t>( 1, h->n_tgt ), s );
    DeviceBuffer<unsigned> count( 1, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( count.get(), 0, sizeof( unsigned ), s ) );
    k_adjoint_fast<M><<<(unsigned)( ( h->n_tgt + AF - 1 ) / AF ), AF, ( 2 * NU + M ) * sizeof( double ) * AF, s>>>(
        h->src_copy.get(), h->tgt_copy.get(), h->offset.get(), h->idx.get(), h->order.get(), h->n_tgt, h->n_src,
        h->opts.rbf, values, cot, contrib, list.get(), count.get(), status );
    check_launch( "k_adjoint_fast" );
    size_t const smem = ( 2 * NU * sizeof( double ) + M * M * sizeof( double ) +
                          M * M * sizeof( float ) ) * AB;
    ensure_dynamic_smem( k_adjoint_entries<M>, smem );
    int64_t const want = ( h->n_tgt + AB - 1 ) / AB;
    unsigned const blocks = (unsigned)std::max<int64_t>( 1, std::min<int64_t>( want, 4 * num_sms() ) );
    k_adjoint_entries<M><<<blocks, AB, smem, s>>>( h->src_copy.get(), h->tgt_copy.get(), h->offset.get(),
                                                    h->idx.get(), list.get(), count.get(), h->n_src,
                                                    h->opts.rbf, values, cot, contrib, status );
    check_launch( "k_adjoint_entries" );
}

void build_transpose_for( dtk_mls_s *h, cudaStream_t s )
{
    if ( h->t_offset.get() )
        return;
    int64_t const nnz = h->nnz, n_src = h->n_src;
    DeviceBuffer<uint32_t> keys( std::max<int64_t>( 1, nnz ), s );
    h->t_entry.allocate( std::max<int64_t>( 1, nnz ), s );
    unsigned const blocks = (unsigned)std::max<int64_t>( 1, ( nnz + 255 ) / 256 );
    if ( nnz )
    {
        k_entry_pairs<<<blocks, 256, 0, s>>>( h->idx.get(), nnz, keys.get(),
                                              reinterpret_cast<uint32_t *>( h->t_entry.get() ) );
        check_launch( "k_entry_pairs" );
        int bits = 1;
        while ( ( int64_t( 1 ) << bits ) < n_src )
            ++bits;
        radix_sort_pairs( keys.get(), reinterpret_cast<uint32_t *>( h->t_entry.get() ), nnz,
                          ( bits + 7 ) / 8 * 8, s );
    }
    DeviceBuffer<int64_t> counts( n_src, s ), offs( n_src + 1, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( counts.get(), 0, n_src * sizeof( int64_t ), s ) );
    if ( nnz )
    {
        k_source_counts<<<blocks, 256, 0, s>>>( keys.get(), nnz, counts.get() );
        check_launch( "k_source_counts" );
    }
    exclusive_scan_i64( counts.get(), offs.get(), n_src, s );
    h->t_offset.allocate( n_src + 1, s );
    k_narrow<<<(unsigned)( ( n_src + 256 ) / 256 ), 256, 0, s>>>( offs.get(), h->t_offset.get(), n_src );
    check_launch( "k_narrow" );
}

} // namespace
} // namespace dtk

using namespace dtk;

extern "C" dtk_status dtk_mls_apply_adjoint( dtk_mls_handle h, const double *cot, int64_t n_cot,
                                             const double *source_values, double *grad_values,
                                             double *grad_coords, dtk_stream_t stream_ )
{
    try
    {
        NvtxRange const nvtx_range( "DTK_apply_adjoint" );
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        DTK_REQUIRE_OR_THROW( n_cot == h->n_tgt, "cot.extent(0) == n_target_points" );
        DTK_REQUIRE_OR_THROW( h->n_tgt == 0 || cot != nullptr, "cot is null" );
        DTK_REQUIRE_OR_THROW( grad_values != nullptr, "grad_values is null" );
        if ( grad_coords )
        {
            DTK_REQUIRE_OR_THROW( source_values != nullptr,
                                  "the coordinate adjoint needs the source values" );
            DTK_REQUIRE_OR_THROW( h->src_copy.get() != nullptr,
                                  "the coordinate adjoint needs a handle created with keep_points" );
        }
        require_device_memory( h->n_tgt ? cot : nullptr, "cot" );
        require_device_memory( grad_values, "grad_values" );
        require_device_memory( source_values, "source_values" );
        require_device_memory( grad_coords, "grad_coords" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        build_transpose_for( h, s );
        DeviceBuffer<unsigned> status( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        DeviceBuffer<int32_t> row_of;
        if ( h->uniform_row <= 0 && h->nnz )
        {
            row_of.allocate( h->nnz, s );
            k_entry_rows<<<(unsigned)( ( h->n_tgt + 255 ) / 256 ), 256, 0, s>>>( h->offset.get(), h->n_tgt,
                                                                                 row_of.get() );
            check_launch( "k_entry_rows" );
        }
        DeviceBuffer<double> contrib;
        if ( grad_coords && h->nnz )
        {
            contrib.allocate( 3 * h->nnz, s );
            switch ( h->opts.basis )
            {
            case DTK_CONSTANT3:
                launch_adjoint_entries<1>( h, source_values, cot, contrib.get(), status.get(), s );
                break;
            case DTK_LINEAR3:
                launch_adjoint_entries<4>( h, source_values, cot, contrib.get(), status.get(), s );
                break;
            default:
                launch_adjoint_entries<10>( h, source_values, cot, contrib.get(), status.get(), s );
                break;
            }
        }
        if ( h->n_src )
        {
            unsigned const blocks = (unsigned)( ( h->n_src + 255 ) / 256 );
            bool const f32 = h->coeff32.get() != nullptr;
            void const *coeff = f32 ? (void const *)h->coeff32.get() : (void const *)h->coeff64.get();
            if ( f32 )
                k_transpose_gather<true><<<blocks, 256, 0, s>>>(
                    h->n_src, h->t_offset.get(), h->t_entry.get(), h->uniform_row, row_of.get(), coeff,
                    cot, contrib.get(), grad_values, grad_coords );
            else
                k_transpose_gather<false><<<blocks, 256, 0, s>>>(
                    h->n_src, h->t_offset.get(), h->t_entry.get(), h->uniform_row, row_of.get(), coeff,
                    cot, contrib.get(), grad_values, grad_coords );
            check_launch( "k_transpose_gather" );
        }
        unsigned st = 0;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "adjoint found a bad neighbour index"};
        return DTK_OK;
    }
    catch ( Error const &e )
    {
        set_error( e.msg );
        return e.status;
    }
    catch ( std::bad_alloc const & )
    {
        set_error( "host allocation failed" );
        return DTK_ERR_OOM;
    }
    catch ( std::exception const &e )
    {
        set_error( e.what() );
        return DTK_ERR_INTERNAL;
    }
}
