// Comparisons and sign operations on the IEEE bits of doubles, for the FP64
// Jacobi: on the GPU they run on the integer pipe, where the FP64 pipe (one
// warp instruction per 64 cycles per SM sub-partition on GB300) would spend
// slots on them.  Each gives exactly the IEEE result of the operation it
// replaces, signed zeros, infinities and NaN included (a NaN result keeps
// the operand's payload, where the FP64 instruction may not); host builds of
// the same functions are tested against the host's IEEE arithmetic.
#ifndef DTK_IEEE_CUH
#define DTK_IEEE_CUH

#include <cstring>

namespace dtk
{

constexpr unsigned long long SIGN_BIT = 0x8000000000000000ull, ABS_BITS = 0x7fffffffffffffffull,
                             INF_BITS = 0x7ff0000000000000ull;

__host__ __device__ __forceinline__ unsigned long long bits_of( double x )
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong( x );
#else
    unsigned long long b;
    std::memcpy( &b, &x, sizeof b );
    return b;
#endif
}
__host__ __device__ __forceinline__ double of_bits( unsigned long long b )
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double( (long long)b );
#else
    double x;
    std::memcpy( &x, &b, sizeof x );
    return x;
#endif
}
__host__ __device__ __forceinline__ bool nan_bits( unsigned long long b )
{
    return ( b & ABS_BITS ) > INF_BITS;
}
__host__ __device__ __forceinline__ bool zero_bits( unsigned long long b )
{
    return ( b & ABS_BITS ) == 0;
}
// x == y
__host__ __device__ __forceinline__ bool ieee_eq( double x, double y )
{
    unsigned long long const a = bits_of( x ), b = bits_of( y );
    return ( a == b && !nan_bits( a ) ) || ( zero_bits( a ) && zero_bits( b ) );
}
// x >= 0 (true for -0, false for NaN)
__host__ __device__ __forceinline__ bool ieee_nonneg( double x )
{
    unsigned long long const a = bits_of( x );
    return zero_bits( a ) || ( !( a & SIGN_BIT ) && !nan_bits( a ) );
}
// (x > 0) - (x < 0)
__host__ __device__ __forceinline__ int ieee_sign( double x )
{
    unsigned long long const a = bits_of( x );
    return zero_bits( a ) || nan_bits( a ) ? 0 : ( a & SIGN_BIT ? -1 : 1 );
}
// -x, and x * copysign(1, s): a sign-bit flip, exactly the product
__host__ __device__ __forceinline__ double ieee_neg( double x )
{
    return of_bits( bits_of( x ) ^ SIGN_BIT );
}
__host__ __device__ __forceinline__ double times_sign_of( double x, double s )
{
    return of_bits( bits_of( x ) ^ ( bits_of( s ) & SIGN_BIT ) );
}
// 1e-280 < r2 < 1e280 for r2 >= 0 or NaN (whose bits order like the values)
__host__ __device__ __forceinline__ bool r2_in_range( unsigned long long b2 )
{
    return b2 > 0x05cd0b15a491eb84ull && b2 < 0x7a11a0fc668aac70ull; // 1e-280, 1e280
}
// 2 r for r >= 0 that is normal, +inf or NaN (its exponent raised by one;
// +inf and NaN as they are): exactly the product
__host__ __device__ __forceinline__ double twice_normal( double r )
{
    unsigned long long const b = bits_of( r );
    return of_bits( b < INF_BITS ? b + ( 1ull << 52 ) : b );
}

} // namespace dtk

#endif
