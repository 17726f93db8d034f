// Device-wide exclusive scan and stable LSD radix sort (no CUB).
//
// Radix sort: 8-bit digits; per pass a per-tile histogram kernel, a scan of
// the digit-major (digit, tile) count table, and a stable scatter that ranks
// equal digits with __match_any_sync inside each warp and a shared-memory
// prefix across the 8 warps of a 256-thread block, reorders the tile by digit
// in shared memory and writes it out in digit runs.
#include "dtk_common.cuh"

#include <algorithm>
#include <utility>

namespace dtk
{
namespace
{

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class T>
__device__ T block_exclusive_scan( T v, T *s_warp, T &total )
{
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for ( int o = 1; o < 32; o <<= 1 )
    {
        T n = __shfl_up_sync( 0xffffffffu, incl, o );
        if ( lane >= o )
            incl += n;
    }
    if ( lane == 31 )
        s_warp[warp] = incl;
    __syncthreads();
    if ( warp == 0 )
    {
        T w = lane < ( SCAN_THREADS / 32 ) ? s_warp[lane] : T( 0 );
        T wi = w;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            T n = __shfl_up_sync( 0xffffffffu, wi, o );
            if ( lane >= o )
                wi += n;
        }
        if ( lane < ( SCAN_THREADS / 32 ) )
            s_warp[lane] = wi - w;
        if ( lane == ( SCAN_THREADS / 32 ) - 1 )
            s_warp[SCAN_THREADS / 32] = wi;
    }
    __syncthreads();
    T const res = s_warp[warp] + incl - v;
    total = s_warp[SCAN_THREADS / 32];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__( SCAN_THREADS )
    k_tile_reduce( int64_t const *in, int64_t n, int64_t *tile_sums )
{
    __shared__ int64_t s_warp[SCAN_THREADS / 32 + 1];
    int64_t const base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int64_t acc = 0;
#pragma unroll
    for ( int i = 0; i < SCAN_ITEMS; ++i )
        if ( base + i < n )
            acc += in[base + i];
    int64_t total;
    block_exclusive_scan<int64_t>( acc, s_warp, total );
    if ( threadIdx.x == 0 )
        tile_sums[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile sums in place, with carry.
__global__ void __launch_bounds__( SCAN_THREADS )
    k_scan_tile_sums( int64_t *sums, int64_t n_tiles, int64_t *grand_total )
{
    __shared__ int64_t s_warp[SCAN_THREADS / 32 + 1];
    int64_t carry = 0;
    for ( int64_t b = 0; b < n_tiles; b += SCAN_THREADS )
    {
        int64_t const i = b + threadIdx.x;
        int64_t const v = i < n_tiles ? sums[i] : 0;
        int64_t total;
        int64_t const ex = block_exclusive_scan<int64_t>( v, s_warp, total );
        if ( i < n_tiles )
            sums[i] = carry + ex;
        carry += total;
    }
    if ( threadIdx.x == 0 )
        *grand_total = carry;
}

__global__ void __launch_bounds__( SCAN_THREADS )
    k_tile_scan( int64_t const *in, int64_t *out, int64_t n, int64_t const *tile_offsets )
{
    __shared__ int64_t s_warp[SCAN_THREADS / 32 + 1];
    int64_t const base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int64_t vals[SCAN_ITEMS];
    int64_t acc = 0;
#pragma unroll
    for ( int i = 0; i < SCAN_ITEMS; ++i )
    {
        vals[i] = base + i < n ? in[base + i] : 0;
        acc += vals[i];
    }
    int64_t total;
    int64_t run = block_exclusive_scan<int64_t>( acc, s_warp, total ) + tile_offsets[blockIdx.x];
#pragma unroll
    for ( int i = 0; i < SCAN_ITEMS; ++i )
    {
        if ( base + i < n )
            out[base + i] = run;
        run += vals[i];
    }
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__( RS_THREADS )
    k_radix_hist( uint32_t const *keys, int64_t n, int shift, int64_t n_tiles,
                  int64_t *hist )
{
    __shared__ unsigned s_hist[256];
    s_hist[threadIdx.x] = 0;
    __syncthreads();
    int64_t const base = (int64_t)blockIdx.x * RS_TILE;
    for ( int r = 0; r < RS_ROUNDS; ++r )
    {
        int64_t const e = base + r * RS_THREADS + threadIdx.x;
        if ( e < n )
            atomicAdd( &s_hist[( keys[e] >> shift ) & 255u], 1u );
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x] = s_hist[threadIdx.x];
}

// Stable scatter of one tile: the ranks of equal digits come from
// __match_any_sync inside each warp, a shared-memory prefix across the 8
// warps and a running count across the tile's rounds; the tile is first
// reordered by digit in shared memory, then written out in that order, so
// that consecutive threads write consecutive positions of a digit's run
// (coalesced) instead of one element per digit bucket per round.
__global__ void __launch_bounds__( RS_THREADS )
    k_radix_scatter( uint32_t const *keys, uint32_t const *vals, uint32_t *keys_out,
                     uint32_t *vals_out, int64_t n, int shift, int64_t n_tiles,
                     int64_t const *offsets )
{
    __shared__ int64_t s_base[256];      // global position of the tile's first element of each digit
    __shared__ unsigned s_start[256];    // tile position of the first element of each digit
    __shared__ unsigned s_run[256];      // elements of each digit placed so far
    __shared__ unsigned s_wcount[RS_WARPS][256];
    __shared__ uint32_t s_key[RS_TILE], s_val[RS_TILE];
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int64_t const base = (int64_t)blockIdx.x * RS_TILE;
    int64_t const rem = n - base;
    int const count = rem < RS_TILE ? (int)rem : RS_TILE;
    s_base[tid] = offsets[(int64_t)tid * n_tiles + blockIdx.x];
    s_run[tid] = 0;
    // tile-local digit starts: the tile's counts from consecutive global offsets
    {
        int64_t const next = blockIdx.x + 1 < n_tiles ? offsets[(int64_t)tid * n_tiles + blockIdx.x + 1]
                                                      : offsets[(int64_t)( tid + 1 ) * n_tiles];
        unsigned const cnt = (unsigned)( next - s_base[tid] );
        // exclusive scan of the 256 counts (one per thread)
        unsigned incl = cnt;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            unsigned const v = __shfl_up_sync( 0xffffffffu, incl, o );
            if ( lane >= o )
                incl += v;
        }
        if ( lane == 31 )
            s_wcount[0][warp] = incl;
        __syncthreads();
        unsigned wpre = 0;
        for ( int w = 0; w < warp; ++w )
            wpre += s_wcount[0][w];
        s_start[tid] = wpre + incl - cnt;
    }
    unsigned const lt_mask = ( 1u << lane ) - 1u;
    for ( int r = 0; r < RS_ROUNDS; ++r )
    {
        __syncthreads();
#pragma unroll
        for ( int w = 0; w < RS_WARPS; ++w )
            s_wcount[w][tid] = 0;
        __syncthreads();
        int const t = r * RS_THREADS + tid;
        bool const valid = t < count;
        uint32_t const key = valid ? keys[base + t] : 0u;
        unsigned const digit = valid ? ( ( key >> shift ) & 255u ) : 256u;
        unsigned const peers = __match_any_sync( 0xffffffffu, digit );
        unsigned const rank = __popc( peers & lt_mask );
        if ( valid && rank == 0 )
            s_wcount[warp][digit] = __popc( peers );
        __syncthreads();
        if ( valid )
        {
            unsigned pos = s_start[digit] + s_run[digit] + rank;
            for ( int w = 0; w < warp; ++w )
                pos += s_wcount[w][digit];
            s_key[pos] = key;
            s_val[pos] = vals[base + t];
        }
        __syncthreads();
        unsigned add = 0;
#pragma unroll
        for ( int w = 0; w < RS_WARPS; ++w )
            add += s_wcount[w][tid];
        s_run[tid] += add;
    }
    __syncthreads();
    for ( int i = tid; i < count; i += RS_THREADS )
    {
        uint32_t const key = s_key[i];
        unsigned const digit = ( key >> shift ) & 255u;
        int64_t const pos = s_base[digit] + ( i - s_start[digit] );
        keys_out[pos] = key;
        vals_out[pos] = s_val[i];
    }
}

} // namespace

void exclusive_scan_i64( int64_t const *in, int64_t *out, int64_t n, cudaStream_t s )
{
    int64_t const n_tiles = std::max<int64_t>( 1, ( n + SCAN_TILE - 1 ) / SCAN_TILE );
    DeviceBuffer<int64_t> sums( n_tiles + 1, s );
    if ( n > 0 )
    {
        k_tile_reduce<<<(unsigned)n_tiles, SCAN_THREADS, 0, s>>>( in, n, sums.get() );
        check_launch( "k_tile_reduce" );
    }
    else
    {
        DTK_CUDA_OR_THROW( cudaMemsetAsync( sums.get(), 0, sizeof( int64_t ), s ) );
    }
    k_scan_tile_sums<<<1, SCAN_THREADS, 0, s>>>( sums.get(), n > 0 ? n_tiles : 1, out + n );
    check_launch( "k_scan_tile_sums" );
    if ( n > 0 )
    {
        k_tile_scan<<<(unsigned)n_tiles, SCAN_THREADS, 0, s>>>( in, out, n, sums.get() );
        check_launch( "k_tile_scan" );
    }
}

void radix_sort_pairs( uint32_t *keys, uint32_t *values, int64_t n, int bits,
                       cudaStream_t s )
{
    if ( n <= 1 || bits <= 0 )
        return;
    int64_t const n_tiles = ( n + RS_TILE - 1 ) / RS_TILE;
    DeviceBuffer<uint32_t> k2( n, s ), v2( n, s );
    DeviceBuffer<int64_t> hist( 256 * n_tiles, s ), offs( 256 * n_tiles + 1, s );
    uint32_t *ka = keys, *va = values, *kb = k2.get(), *vb = v2.get();
    for ( int shift = 0; shift < bits; shift += 8 )
    {
        k_radix_hist<<<(unsigned)n_tiles, RS_THREADS, 0, s>>>( ka, n, shift, n_tiles, hist.get() );
        check_launch( "k_radix_hist" );
        exclusive_scan_i64( hist.get(), offs.get(), 256 * n_tiles, s );
        k_radix_scatter<<<(unsigned)n_tiles, RS_THREADS, 0, s>>>( ka, va, kb, vb, n, shift,
                                                                  n_tiles, offs.get() );
        check_launch( "k_radix_scatter" );
        std::swap( ka, kb );
        std::swap( va, vb );
    }
    if ( ka != keys )
    {
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( keys, ka, n * sizeof( uint32_t ),
                                            cudaMemcpyDeviceToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( values, va, n * sizeof( uint32_t ),
                                            cudaMemcpyDeviceToDevice, s ) );
    }
}

} // namespace dtk
