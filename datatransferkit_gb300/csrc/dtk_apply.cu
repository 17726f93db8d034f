// MLS apply: CSR gather-SpMV (sm_103a).
//
// Replaces MovingLeastSquaresOperator::apply
// (packages/Meshfree/src/DTK_MovingLeastSquaresOperator_def.hpp:121-141):
// the single-rank fetch (a gather of source values into per-neighbour
// order, DTK_DetailsNearestNeighborOperatorImpl.hpp:152-192), computeTargetValues
// (DTK_DetailsMovingLeastSquaresOperatorImpl.hpp:49-70) and the deep_copy fuse
// into one kernel that reads idx/coeff once and writes each target once.
//
// Rows of equal length R with R % 4 == 0 and R/4 a power of two (kNN rows,
// e.g. R = 32) use R/8 lanes per row (8 entries each; R/4 lanes of 4 for
// FP64 coefficients) with 128-bit loads:
// int4 of indices and two double2 (FP64 form) or one float4 (mixed form) of
// coefficients per 4 entries, then a shuffle reduction.  Other rows use S lanes per row (S a power of two chosen
// from the mean row length) with coalesced scalar loads.  Source values are
// gathered through the read-only path; at 8M sources they are 64 MB and stay
// resident in the 129 MB L2 while the CSR streams from HBM.
#include "dtk_common.cuh"

#include <algorithm>

namespace dtk
{
namespace
{

constexpr unsigned FULL = 0xffffffffu;

template <int L>
__device__ __forceinline__ double group_sum( double v )
{
#pragma unroll
    for ( int o = L / 2; o > 0; o >>= 1 )
        v += __shfl_xor_sync( FULL, v, o );
    return v;
}

// L lanes per row, each lane EPL consecutive entries (EPL a multiple of 4).
template <int L, int EPL, bool F32>
__global__ void __launch_bounds__( 256 )
    k_apply_vec( int64_t n_tgt, int32_t const *__restrict__ idx,
                 void const *__restrict__ coeff, double const *__restrict__ values,
                 double *__restrict__ target )
{
    constexpr int R = EPL * L;
    int64_t const gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const row = gt / L;
    int const sub = (int)( gt % L );
    double acc = 0.0;
    if ( row < n_tgt )
    {
#pragma unroll
        for ( int q = 0; q < EPL; q += 4 )
        {
            int64_t const e = row * R + EPL * sub + q;
            int4 const ix = __ldcs( reinterpret_cast<int4 const *>( idx + e ) );
            if constexpr ( F32 )
            {
                float4 const c =
                    __ldcs( reinterpret_cast<float4 const *>( static_cast<float const *>( coeff ) + e ) );
                acc += (double)c.x * __ldg( values + ix.x ) + (double)c.y * __ldg( values + ix.y ) +
                       (double)c.z * __ldg( values + ix.z ) + (double)c.w * __ldg( values + ix.w );
            }
            else
            {
                double const *cp = static_cast<double const *>( coeff ) + e;
                double2 const c0 = __ldcs( reinterpret_cast<double2 const *>( cp ) );
                double2 const c1 = __ldcs( reinterpret_cast<double2 const *>( cp + 2 ) );
                acc += c0.x * __ldg( values + ix.x ) + c0.y * __ldg( values + ix.y ) +
                       c1.x * __ldg( values + ix.z ) + c1.y * __ldg( values + ix.w );
            }
        }
    }
    acc = group_sum<L>( acc );
    if ( row < n_tgt && sub == 0 )
        target[row] = acc;
}

// S lanes per row, strided scalar loads.
template <int S, bool F32>
__global__ void __launch_bounds__( 256 )
    k_apply_csr( int64_t n_tgt, int32_t const *__restrict__ offset,
                 int32_t const *__restrict__ idx, void const *__restrict__ coeff,
                 double const *__restrict__ values, double *__restrict__ target )
{
    int64_t const gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const row = gt / S;
    int const sub = (int)( gt % S );
    double acc = 0.0;
    if ( row < n_tgt )
    {
        int const b = offset[row], e = offset[row + 1];
        for ( int j = b + sub; j < e; j += S )
        {
            double const c = F32 ? (double)static_cast<float const *>( coeff )[j]
                                 : static_cast<double const *>( coeff )[j];
            acc += c * __ldg( values + idx[j] );
        }
    }
    acc = group_sum<S>( acc );
    if ( row < n_tgt && sub == 0 )
        target[row] = acc;
}

// Row length R = 4 * 2^j (at most 128): R / EPL lanes per row, each EPL
// entries (4 entries a lane for rows shorter than EPL).  FP32 coefficients
// take EPL = 8 (one reduction level fewer: -9% at 8M x 32), FP64 ones 4
// (twice the coefficient bytes a lane: +5% at 8).
template <bool F32>
constexpr int apply_epl()
{
    return F32 ? 8 : 4;
}

template <int EPL, bool F32>
void launch_vec_epl( int L, unsigned blocks, int64_t n_tgt, int32_t const *idx, void const *coeff,
                     double const *values, double *target, cudaStream_t s )
{
    switch ( L )
    {
    case 1: k_apply_vec<1, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    case 2: k_apply_vec<2, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    case 4: k_apply_vec<4, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    case 8: k_apply_vec<8, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    case 16: k_apply_vec<16, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    default: k_apply_vec<32, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, idx, coeff, values, target ); break;
    }
}

template <bool F32>
void launch_vec( int R, int64_t n_tgt, int32_t const *idx, void const *coeff,
                 double const *values, double *target, cudaStream_t s )
{
    constexpr int EPL = apply_epl<F32>();
    int const epl = R >= EPL ? EPL : 4;
    int const L = R / epl;
    unsigned const blocks = (unsigned)( ( n_tgt * L + 255 ) / 256 );
    if ( epl == EPL )
        launch_vec_epl<EPL, F32>( L, blocks, n_tgt, idx, coeff, values, target, s );
    else
        launch_vec_epl<4, F32>( L, blocks, n_tgt, idx, coeff, values, target, s );
    check_launch( "k_apply_vec" );
}

template <bool F32>
void launch_csr( int S, int64_t n_tgt, int32_t const *offset, int32_t const *idx,
                 void const *coeff, double const *values, double *target, cudaStream_t s )
{
    int64_t const threads = n_tgt * S;
    unsigned const blocks = (unsigned)( ( threads + 255 ) / 256 );
    switch ( S )
    {
    case 1: k_apply_csr<1, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    case 2: k_apply_csr<2, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    case 4: k_apply_csr<4, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    case 8: k_apply_csr<8, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    case 16: k_apply_csr<16, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    default: k_apply_csr<32, F32><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff, values, target ); break;
    }
    check_launch( "k_apply_csr" );
}

bool is_pow2( int v ) { return v > 0 && ( v & ( v - 1 ) ) == 0; }

} // namespace

// ---------------------------------------------------------------------------
// Apply over sorted positions (kNN operators): the source values are first
// permuted into the tree's Morton order (one pass over the sources), and the
// rows gather them by sorted position, so a row's neighbours sit in a few
// sectors of an L2-resident array instead of 32 scattered ones.  The mixed
// form keeps the permuted values as double-floats (hi = fl32(v), lo =
// fl32(v - hi)) and sums c_j (hi_j + lo_j) in double-float arithmetic on the
// FP32 pipe (TwoProd / TwoSum, the compensated scheme of the mixed setup):
// the FP32 coefficients are the only rounding left, as with an FP64 sum.
// The FP64 form permutes the doubles and sums with FP64 FMAs.  Rows go in
// the targets' Morton order when the operator has it, so that consecutive
// rows share most of their neighbours' values in L1 (0.70 -> 0.59 ms for 8M
// rows of 32; 16 entries a lane instead of 8 was 1.26 ms, 4 no different).
// ---------------------------------------------------------------------------
namespace
{

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

// sorted[p] = values[perm[p]] (perm null: the identity) as a double (FP64
// form) or a double-float
__global__ void k_permute_values( int64_t n, uint32_t const *__restrict__ perm, double const *__restrict__ values,
                                  double *__restrict__ sorted64, float2 *__restrict__ sorted32 )
{
    int64_t const p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( p >= n )
        return;
    double const v = __ldg( values + ( perm ? (int64_t)__ldg( perm + p ) : p ) );
    if ( sorted32 )
    {
        float const hi = __double2float_rn( v );
        sorted32[p] = make_float2( hi, __double2float_rn( v - (double)hi ) );
    }
    else
        sorted64[p] = v;
}

// c * (v.x + v.y) added to the double-float (s, c_acc)
__device__ __forceinline__ void df_axpy( float c, float2 v, float &s, float &cs )
{
    float p, e, t, f;
    two_prod( c, v.x, p, e );
    e = __fmaf_rn( c, v.y, e );
    two_sum( s, p, t, f );
    s = t;
    cs = __fadd_rn( cs, __fadd_rn( f, e ) );
}

// L lanes per row, each lane EPL consecutive entries (EPL a multiple of 4).
template <int L, int EPL, bool F32>
__global__ void __launch_bounds__( 256 )
    k_apply_pos( int64_t n_tgt, int32_t const *__restrict__ pos, void const *__restrict__ coeff,
                 void const *__restrict__ sorted, double *__restrict__ target, uint32_t const *__restrict__ order )
{
    constexpr int R = EPL * L;
    int64_t const gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const row0 = gt / L;
    int64_t const row = ( order && row0 < n_tgt ) ? (int64_t)__ldg( order + row0 ) : row0;
    int const sub = (int)( gt % L );
    if constexpr ( F32 )
    {
        float2 const *vals = static_cast<float2 const *>( sorted );
        float s = 0.f, cs = 0.f;
        if ( row < n_tgt )
        {
#pragma unroll
            for ( int q = 0; q < EPL; q += 4 )
            {
                int64_t const e = row * R + EPL * sub + q;
                int4 const ix = __ldcs( reinterpret_cast<int4 const *>( pos + e ) );
                float4 const c =
                    __ldcs( reinterpret_cast<float4 const *>( static_cast<float const *>( coeff ) + e ) );
                df_axpy( c.x, __ldg( vals + ix.x ), s, cs );
                df_axpy( c.y, __ldg( vals + ix.y ), s, cs );
                df_axpy( c.z, __ldg( vals + ix.z ), s, cs );
                df_axpy( c.w, __ldg( vals + ix.w ), s, cs );
            }
        }
#pragma unroll
        for ( int o = L / 2; o > 0; o >>= 1 )
        {
            float const os = __shfl_xor_sync( FULL, s, o ), oc = __shfl_xor_sync( FULL, cs, o );
            float t, f;
            two_sum( s, os, t, f );
            s = t;
            cs = __fadd_rn( cs, __fadd_rn( oc, f ) );
        }
        if ( row < n_tgt && sub == 0 )
            target[row] = (double)s + (double)cs;
    }
    else
    {
        double const *vals = static_cast<double const *>( sorted );
        double acc = 0.0;
        if ( row < n_tgt )
        {
#pragma unroll
            for ( int q = 0; q < EPL; q += 4 )
            {
                int64_t const e = row * R + EPL * sub + q;
                int4 const ix = __ldcs( reinterpret_cast<int4 const *>( pos + e ) );
                double const *cp = static_cast<double const *>( coeff ) + e;
                double2 const c0 = __ldcs( reinterpret_cast<double2 const *>( cp ) );
                double2 const c1 = __ldcs( reinterpret_cast<double2 const *>( cp + 2 ) );
                acc += c0.x * __ldg( vals + ix.x ) + c0.y * __ldg( vals + ix.y ) +
                       c1.x * __ldg( vals + ix.z ) + c1.y * __ldg( vals + ix.w );
            }
        }
        acc = group_sum<L>( acc );
        if ( row < n_tgt && sub == 0 )
            target[row] = acc;
    }
}

template <int EPL, bool F32>
void launch_pos_epl( int L, unsigned blocks, int64_t n_tgt, int32_t const *pos, void const *coeff,
                     void const *sorted, double *target, cudaStream_t s, uint32_t const *order )
{
    switch ( L )
    {
    case 1: k_apply_pos<1, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    case 2: k_apply_pos<2, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    case 4: k_apply_pos<4, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    case 8: k_apply_pos<8, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    case 16: k_apply_pos<16, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    default: k_apply_pos<32, EPL, F32><<<blocks, 256, 0, s>>>( n_tgt, pos, coeff, sorted, target, order ); break;
    }
}

} // namespace

bool apply_sorted_supported( int uniform_row )
{
    return uniform_row > 0 && uniform_row % 4 == 0 && is_pow2( uniform_row / 4 ) && uniform_row / 4 <= 32;
}

SortedValues permute_values( int64_t n_src, uint32_t const *perm, double const *values, bool f32,
                             cudaStream_t s )
{
    SortedValues v;
    if ( f32 )
        v.v32.allocate( std::max<int64_t>( 1, n_src ), s );
    else
        v.v64.allocate( std::max<int64_t>( 1, n_src ), s );
    if ( n_src > 0 )
    {
        k_permute_values<<<(unsigned)( ( n_src + 255 ) / 256 ), 256, 0, s>>>( n_src, perm, values, v.v64.get(),
                                                                            v.v32.get() );
        check_launch( "k_permute_values" );
    }
    return v;
}

void apply_pos( int64_t n_rows, int uniform_row, int32_t const *pos, double const *coeff64, float const *coeff32,
                SortedValues const &v, double *target, cudaStream_t s, uint32_t const *order )
{
    if ( n_rows == 0 )
        return;
    int const R = uniform_row;
    if ( coeff32 )
    {
        int const epl = R >= 8 ? 8 : 4;
        int const L = R / epl;
        unsigned const blocks = (unsigned)( ( n_rows * L + 255 ) / 256 );
        if ( epl == 8 )
            launch_pos_epl<8, true>( L, blocks, n_rows, pos, coeff32, v.v32.get(), target, s, order );
        else
            launch_pos_epl<4, true>( L, blocks, n_rows, pos, coeff32, v.v32.get(), target, s, order );
    }
    else
    {
        int const L = R / 4;
        unsigned const blocks = (unsigned)( ( n_rows * L + 255 ) / 256 );
        launch_pos_epl<4, false>( L, blocks, n_rows, pos, coeff64, v.v64.get(), target, s, order );
    }
    check_launch( "k_apply_pos" );
}

void apply_sorted( int64_t n_tgt, int uniform_row, int32_t const *pos, double const *coeff64,
                   float const *coeff32, int64_t n_src, uint32_t const *perm, double const *values,
                   double *target, cudaStream_t s, uint32_t const *order )
{
    if ( n_tgt == 0 )
        return;
    SortedValues const v = permute_values( n_src, perm, values, coeff32 != nullptr, s );
    apply_pos( n_tgt, uniform_row, pos, coeff64, coeff32, v, target, s, order );
}

// uniform_row > 0: every row has that length (offset[i] = i * uniform_row);
// otherwise mean_row picks the lanes per row.
namespace
{

// Rank-2 fields: 8 lanes per row, 4 components per pass; the row's indices
// and coefficients are read once per pass for 4 components.
template <bool F32>
__global__ void __launch_bounds__( 256 )
    k_apply_multi( int64_t n_tgt, int32_t const *__restrict__ offset, int32_t const *__restrict__ idx,
                   void const *__restrict__ coeff, FieldView in, FieldView out )
{
    constexpr int S = 8, CB = 4;
    int64_t const gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t const row = gt / S;
    int const sub = (int)( gt % S );
    bool const live = row < n_tgt;
    int const b = live ? offset[row] : 0, e = live ? offset[row + 1] : 0;
    for ( int c0 = 0; c0 < in.n_comp; c0 += CB ) // uniform across the warp
    {
        double acc[CB] = {0.0, 0.0, 0.0, 0.0};
        for ( int j = b + sub; j < e; j += S )
        {
            double const cj = F32 ? (double)__ldg( static_cast<float const *>( coeff ) + j )
                                  : __ldg( static_cast<double const *>( coeff ) + j );
            int64_t const sj = __ldg( idx + j );
#pragma unroll
            for ( int q = 0; q < CB; ++q )
                if ( c0 + q < in.n_comp )
                    acc[q] = fma( cj, __ldg( in.base + sj * in.ps + ( c0 + q ) * in.cs ), acc[q] );
        }
#pragma unroll
        for ( int q = 0; q < CB; ++q )
            acc[q] = group_sum<S>( acc[q] );
        if ( live && sub == 0 )
#pragma unroll
            for ( int q = 0; q < CB; ++q )
                if ( c0 + q < in.n_comp )
                    out.wbase[row * out.ps + ( c0 + q ) * out.cs] = acc[q];
    }
}

} // namespace

void apply_csr_multi( int64_t n_tgt, int32_t const *offset, int32_t const *idx, double const *coeff64,
                      float const *coeff32, FieldView in, FieldView out, cudaStream_t s )
{
    if ( n_tgt == 0 )
        return;
    unsigned const blocks = (unsigned)( ( n_tgt * 8 + 255 ) / 256 );
    if ( coeff32 )
        k_apply_multi<true><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff32, in, out );
    else
        k_apply_multi<false><<<blocks, 256, 0, s>>>( n_tgt, offset, idx, coeff64, in, out );
    check_launch( "k_apply_multi" );
}

void apply_csr( int64_t n_tgt, int32_t const *offset, int32_t const *idx, double const *coeff64,
                float const *coeff32, int uniform_row, int mean_row, double const *values,
                double *target, cudaStream_t s )
{
    if ( n_tgt == 0 )
        return;
    bool const f32 = coeff32 != nullptr;
    void const *coeff = f32 ? (void const *)coeff32 : (void const *)coeff64;
    if ( uniform_row > 0 && uniform_row % 4 == 0 && is_pow2( uniform_row / 4 ) &&
         uniform_row / 4 <= 32 )
    {
        if ( f32 )
            launch_vec<true>( uniform_row, n_tgt, idx, coeff, values, target, s );
        else
            launch_vec<false>( uniform_row, n_tgt, idx, coeff, values, target, s );
        return;
    }
    int const len = uniform_row > 0 ? uniform_row : mean_row;
    int S = 1;
    while ( S < 32 && S * 2 <= len )
        S *= 2;
    if ( f32 )
        launch_csr<true>( S, n_tgt, offset, idx, coeff, values, target, s );
    else
        launch_csr<false>( S, n_tgt, offset, idx, coeff, values, target, s );
}

} // namespace dtk
