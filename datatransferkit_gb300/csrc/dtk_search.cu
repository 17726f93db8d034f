// Linear BVH and warp-cooperative kNN / radius search (sm_103a).
//
// Replaces the ArborX tree and query the MLS constructor runs
// (packages/Meshfree/src/DTK_MovingLeastSquaresOperator_def.hpp:47-62).
//
// Build: scene box -> 30-bit Morton codes (FP32 quantization) -> stable
// radix sort (codes, ids) -> Morton-sorted FP64 coordinates (packed with the
// original index, plus FP32 copies centred on the scene with each point's
// leaf start) -> leaves: the Morton cells of at most 32
// points (the key trie split one bit at a time) -> Karras (2012) binary radix
// tree over the leaf keys (first code of each leaf, ties broken by leaf
// index) -> bottom-up refit of FP32 boxes rounded outward -> collapse into an
// 8-wide BVH (three binary levels per wide node), so that 8 lanes test the 8
// children of a node at once; each wide node also keeps its Morton cell (an
// inset FP32 box) and its parent.
//
// kNN query: a warp runs chunks of 48 Morton-consecutive targets one after
// the other, taking the next chunk from a counter; the k best (d2, index)
// keys sit one per lane, sorted across lanes.
// The first target of a chunk starts from the 32 Morton-sorted sources around
// its code, every later one from the previous target's final list re-keyed
// for it (neighbouring targets share most neighbours).  The list's members
// are screened out of a leaf (a warp OR-reduction of the lanes whose
// position lies in the leaf), so no source enters the list twice.  A seeded
// target also prunes with a speculative bound, 1.25 times the previous
// target's k-th squared distance, and starts at the deepest wide node whose
// cell holds the ball of that radius, or scans its chunk's leaf list (the
// leaves near the chunk's targets, collected after the chunk's first
// search); when the search ends with a k-th key above the bound, a
// second pass (from the root, with the whole list screened out and the
// list's own bound) finds what it skipped.  A box is pruned only when its
// FP32 round-down lower bound exceeds the round-up bound with a 2^-20
// relative margin, and a leaf point only when its FP32 lower bound (with a
// rigorous rounding bound) does, so no point whose FP64 distance could tie or
// beat the bound is skipped.  The survivors get exact FP64 keys 32 at a time
// and are merged into the list as a batch (bitonic sort, merge against the
// reversed candidates, bitonic clean; the networks run on 32-bit keys and
// fall back to exact ones on a collision).  Distances of points are exact
// FP64 with separately rounded operations: (dx*dx + dy*dy) + dz*dz.  Keys
// compare as integers (d2 >= 0, so its IEEE bits are monotone),
// lexicographic with the source index.
#include "dtk_common.cuh"

#include <climits>

#include <algorithm>
#include <functional>
#include <vector>

namespace dtk
{
namespace
{

constexpr int LEAF = 32;
constexpr int STACK = 256; // wide-node stack entries per warp (kNN and radius search)
constexpr int NODE_GROUPS = 4; // wide nodes a kNN warp tests per step (8 lanes each)
static_assert( NODE_GROUPS * 8 == 32, "one lane per child slot" );
constexpr int Q_WARPS = 16; // warps per block in the kNN query kernel
constexpr int R_WARPS = 4; // warps per block in the radius query kernel
constexpr int Q_SEQ = 48;  // kNN queries per chunk, run in order by one warp (each seeds the next)
// kNN blocks per SM: 4 blocks of 16 warps (all 64 warp slots) cap the kernel
// at 32 registers, with the query in shared memory; the values spilled cost
// less than the warps gained (8M-point query, 4-warp blocks: 39.0 ms at 8
// blocks, 34.5 ms at 16; then 8-, 16- and 32-warp blocks: 22.0, 21.4 and
// 21.7 ms)
constexpr int KNN_BLOCKS_PER_SM = 4;
constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned long long KEY_INF = 0xffffffffffffffffull;

__device__ __forceinline__ uint32_t expand10( uint32_t v )
{
    v &= 0x3ffu;
    v = ( v | ( v << 16 ) ) & 0x030000FFu;
    v = ( v | ( v << 8 ) ) & 0x0300F00Fu;
    v = ( v | ( v << 4 ) ) & 0x030C30C3u;
    v = ( v | ( v << 2 ) ) & 0x09249249u;
    return v;
}

// Morton codes only order the points (the tree's shape and the order of the
// queries), they never decide a result, so they are computed in FP32 (the
// FP64 pipe is 1/64 of the FP32 rate): one rounding of each coordinate, then
// the FP32 copies of lo and 1024 / extent written at scene[13..15].
__device__ __forceinline__ uint32_t quantize( float c, float lo, float scale )
{
    float const u = ( c - lo ) * scale;
    if ( !( u > 0.f ) )
        return 0u;
    if ( u >= 1023.f )
        return 1023u;
    return (uint32_t)u;
}

__device__ __forceinline__ uint32_t morton3( double x, double y, double z,
                                             double const *scene )
{
    float const *sf = reinterpret_cast<float const *>( scene + 13 ); // lo[3], scale[3]
    return ( expand10( quantize( __double2float_rn( x ), sf[0], sf[3] ) ) << 2 ) |
           ( expand10( quantize( __double2float_rn( y ), sf[1], sf[4] ) ) << 1 ) |
           expand10( quantize( __double2float_rn( z ), sf[2], sf[5] ) );
}

// ---------------------------------------------------------------------------
// Scene bounds (two-stage reduction).  Min/max of doubles through an
// order-preserving integer map, so the reduction stays off the FP64 pipe.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ord_of( double v )
{
    unsigned long long b = (unsigned long long)__double_as_longlong( v );
    return ( b >> 63 ) ? ~b : ( b | 0x8000000000000000ull );
}
__device__ __forceinline__ double double_of( unsigned long long o )
{
    unsigned long long b = ( o >> 63 ) ? ( o & 0x7fffffffffffffffull ) : ~o;
    return __longlong_as_double( (long long)b );
}

constexpr int BND_THREADS = 256;

__global__ void __launch_bounds__( BND_THREADS )
    k_bounds_partial( PointsView p, unsigned long long *partial, unsigned *status )
{
    unsigned long long mn[3] = {KEY_INF, KEY_INF, KEY_INF}, mx[3] = {0, 0, 0};
    bool bad = false;
    for ( int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n;
          i += (int64_t)gridDim.x * blockDim.x )
        for ( int d = 0; d < 3; ++d )
        {
            double const v = p( i, d );
            bad |= nonfinite_bits( v );
            unsigned long long const o = ord_of( v );
            mn[d] = min( mn[d], o );
            mx[d] = max( mx[d], o );
        }
    if ( bad )
        atomicOr( status, DEV_NONFINITE_SOURCE );
    __shared__ unsigned long long s[6][BND_THREADS / 32];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for ( int d = 0; d < 3; ++d )
    {
        for ( int o = 16; o; o >>= 1 )
        {
            mn[d] = min( mn[d], __shfl_xor_sync( FULL, mn[d], o ) );
            mx[d] = max( mx[d], __shfl_xor_sync( FULL, mx[d], o ) );
        }
        if ( lane == 0 )
        {
            s[d][warp] = mn[d];
            s[3 + d][warp] = mx[d];
        }
    }
    __syncthreads();
    if ( threadIdx.x < 6 )
    {
        unsigned long long v = s[threadIdx.x][0];
        for ( int w = 1; w < BND_THREADS / 32; ++w )
            v = threadIdx.x < 3 ? min( v, s[threadIdx.x][w] ) : max( v, s[threadIdx.x][w] );
        partial[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

// scene[0..2] = lo, scene[3..5] = 1024/extent (0 when flat), scene[6..8] = hi,
// scene[9..11] = centre c, scene[12] = S >= max_i,d |p_id - c_d| (with slack),
// scene[13..16] = lo and 1024/extent as six floats (the Morton codes), then
// S rounded up to a float
__global__ void k_bounds_final( unsigned long long const *partial, int nblocks,
                                double *scene )
{
    __shared__ double half[3];
    // one warp: lane l folds the partials of blocks l, l + 32, ..., then a
    // shuffle reduction per axis
    int const lane = threadIdx.x & 31;
    unsigned long long pmn[3] = {KEY_INF, KEY_INF, KEY_INF}, pmx[3] = {0, 0, 0};
    for ( int b = lane; b < nblocks; b += 32 )
        for ( int d = 0; d < 3; ++d )
        {
            pmn[d] = min( pmn[d], partial[b * 6 + d] );
            pmx[d] = max( pmx[d], partial[b * 6 + 3 + d] );
        }
    for ( int d = 0; d < 3; ++d )
        for ( int o = 16; o; o >>= 1 )
        {
            pmn[d] = min( pmn[d], __shfl_xor_sync( FULL, pmn[d], o ) );
            pmx[d] = max( pmx[d], __shfl_xor_sync( FULL, pmx[d], o ) );
        }
    if ( threadIdx.x < 3 )
    {
        int const d = threadIdx.x;
        unsigned long long const mn = d == 0 ? pmn[0] : d == 1 ? pmn[1] : pmn[2];
        unsigned long long const mx = d == 0 ? pmx[0] : d == 1 ? pmx[1] : pmx[2];
        double const lo = double_of( mn ), hi = double_of( mx );
        double const e = hi - lo;
        scene[d] = lo;
        scene[3 + d] = e > 0.0 ? 1024.0 / e : 0.0;
        reinterpret_cast<float *>( scene + 13 )[d] = __double2float_rn( lo );
        reinterpret_cast<float *>( scene + 13 )[3 + d] = __double2float_rn( scene[3 + d] );
        scene[6 + d] = hi;
        double const c = 0.5 * lo + 0.5 * hi;
        scene[9 + d] = c;
        half[d] = fmax( hi - c, c - lo );
    }
    __syncthreads();
    if ( threadIdx.x == 0 )
    {
        scene[12] = fmax( half[0], fmax( half[1], half[2] ) ) * ( 1.0 + 1e-6 ) + 1e-300;
        reinterpret_cast<float *>( scene + 13 )[6] = __double2float_ru( scene[12] );
    }
}

// (bad_flag: when not null, a point with a NaN or infinite coordinate sets
// DEV_NONFINITE_TARGET there; codes of such points are clamped, never out of
// range)
__global__ void k_morton( PointsView p, double const *scene, uint32_t *codes,
                          uint32_t *ids, int drop = 0, unsigned *bad_flag = nullptr )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < p.n )
    {
        double const x = p( i, 0 ), y = p( i, 1 ), z = p( i, 2 );
        codes[i] = morton3( x, y, z, scene ) >> drop;
        ids[i] = (uint32_t)i;
        if ( bad_flag && ( nonfinite_bits( x ) || nonfinite_bits( y ) || nonfinite_bits( z ) ) )
            atomicOr( bad_flag, DEV_NONFINITE_TARGET );
    }
}

__global__ void k_group_of( uint32_t const *group, uint32_t const *perm, int64_t n, uint32_t *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < n )
        out[i] = group[perm[i]];
}

__global__ void k_morton_of( PointsView p, uint32_t const *perm, double const *scene, uint32_t *codes )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < p.n )
    {
        int64_t const o = perm[i];
        codes[i] = morton3( p( o, 0 ), p( o, 1 ), p( o, 2 ), scene );
    }
}

__global__ void k_gather_sorted( PointsView p, uint32_t const *perm, double const *scene, double2 *s2,
                                 float4 *f4 )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < p.n )
    {
        int64_t const o = perm[i];
        double const x = p( o, 0 ), y = p( o, 1 ), z = p( o, 2 );
        s2[2 * i] = make_double2( x, y );
        s2[2 * i + 1] = make_double2( z, __longlong_as_double( o ) );
        f4[i] = make_float4( (float)( x - scene[9] ), (float)( y - scene[10] ), (float)( z - scene[11] ), 0.f );
    }
}

// ---------------------------------------------------------------------------
// Leaves: the Morton cells of at most LEAF points.  Splitting the bit trie of
// the sorted keys one bit at a time until a cell holds <= LEAF points keeps
// every leaf inside one cell (compact boxes; a fixed bucket of 32 consecutive
// points straddles cell boundaries and spans far more space): at 1M uniform
// points, 44k leaves of 22.6 points on average, and a query ball meets 12 of
// them instead of 22 buckets.
// ---------------------------------------------------------------------------
// Common-prefix length of the sorted keys of points j and j + 1 (key = group
// << 32 | Morton code; equal keys are ranked by position, below every key bit,
// as in the tree over the leaves).
__device__ __forceinline__ unsigned long long point_key( uint32_t const *codes, uint32_t const *grp,
                                                         int64_t p )
{
    unsigned long long k = codes[p];
    if ( grp )
        k |= (unsigned long long)grp[p] << 32;
    return k;
}

__global__ void k_point_delta( uint32_t const *codes, uint32_t const *grp, int64_t n, int *dlt )
{
    int64_t const j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( j >= n - 1 )
        return;
    unsigned long long const a = point_key( codes, grp, j ), b = point_key( codes, grp, j + 1 );
    dlt[j] = a != b ? __clzll( a ^ b ) : 64 + __clzll( (unsigned long long)( j ^ ( j + 1 ) ) );
}

// Position i (0 < i < n) starts a leaf when the smallest cell holding points
// i - 1 and i has more than LEAF points: the points of that cell are the run
// of adjacent pairs around (i - 1, i) whose common prefix is at least
// dlt[i - 1], so the test counts at most LEAF pairs.  Position 0 starts the
// first leaf.
__global__ void k_leaf_flags( int const *dlt, int64_t n, int64_t *flag )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    if ( i == 0 )
    {
        flag[0] = 1;
        return;
    }
    int const L = dlt[i - 1];
    int run = 1;
    for ( int64_t j = i - 2; j >= 0 && run < LEAF && dlt[j] >= L; --j )
        ++run;
    for ( int64_t j = i; j < n - 1 && run < LEAF && dlt[j] >= L; ++j )
        ++run;
    flag[i] = run >= LEAF ? 1 : 0;
}

// leaf_of[i] and leaf_start[] from the exclusive scan of the flags.
__global__ void k_leaf_index( int64_t const *flag, int64_t const *scan, int64_t n, int32_t *leaf_of,
                              int32_t *leaf_start )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    int64_t const leaf = scan[i] + flag[i] - 1;
    leaf_of[i] = (int32_t)leaf;
    if ( flag[i] )
        leaf_start[scan[i]] = (int32_t)i;
    if ( i == n - 1 )
        leaf_start[leaf + 1] = (int32_t)n;
}

// ---------------------------------------------------------------------------
// Karras hierarchy over leaf keys.
// ---------------------------------------------------------------------------
// Leaf key: (group of the leaf's first point, its Morton code); groups are
// the problems of a batch (absent for a single operator).
__device__ __forceinline__ unsigned long long leaf_key( uint32_t const *codes, uint32_t const *grp,
                                                        int32_t const *leaf_start, int64_t leaf )
{
    return point_key( codes, grp, leaf_start[leaf] );
}

__device__ __forceinline__ int delta( uint32_t const *codes, uint32_t const *grp, int32_t const *leaf_start,
                                      int64_t nl, int64_t i, int64_t j )
{
    if ( j < 0 || j >= nl )
        return -1;
    unsigned long long const ki = leaf_key( codes, grp, leaf_start, i ),
                             kj = leaf_key( codes, grp, leaf_start, j );
    if ( ki != kj )
        return __clzll( ki ^ kj );
    // equal leaf keys: ranks by leaf index, always above any 64-bit key prefix
    return 64 + __clzll( (unsigned long long)( i ^ j ) );
}

// Internal node i covers leaves [lo[i], hi[i]]; its left child covers
// [lo, gamma] and its right child [gamma + 1, hi], gamma being the index of
// the left child (leaf or internal, Karras 2012).
__global__ void k_karras( uint32_t const *codes, uint32_t const *grp, int32_t const *leaf_start, int64_t nl,
                          int *left,
                          int *right, int *parent_node, int *parent_leaf, int *range_lo,
                          int *range_hi )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= nl - 1 )
        return;
    int const d = ( delta( codes, grp, leaf_start, nl, i, i + 1 ) - delta( codes, grp, leaf_start, nl, i, i - 1 ) ) >= 0 ? 1 : -1;
    int const dmin = delta( codes, grp, leaf_start, nl, i, i - d );
    int64_t lmax = 2;
    while ( delta( codes, grp, leaf_start, nl, i, i + lmax * d ) > dmin )
        lmax <<= 1;
    int64_t l = 0;
    for ( int64_t t = lmax >> 1; t >= 1; t >>= 1 )
        if ( delta( codes, grp, leaf_start, nl, i, i + ( l + t ) * d ) > dmin )
            l += t;
    int64_t const j = i + l * d;
    int const dnode = delta( codes, grp, leaf_start, nl, i, j );
    int64_t s = 0;
    int64_t t = l;
    do
    {
        t = ( t + 1 ) >> 1;
        if ( delta( codes, grp, leaf_start, nl, i, i + ( s + t ) * d ) > dnode )
            s += t;
    } while ( t > 1 );
    int64_t const gamma = i + s * d + min( d, 0 );
    int64_t const lo = min( i, j ), hi = max( i, j );
    int lc, rc;
    if ( lo == gamma )
    {
        lc = ~(int)gamma;
        parent_leaf[gamma] = (int)i;
    }
    else
    {
        lc = (int)gamma;
        parent_node[gamma] = (int)i;
    }
    if ( hi == gamma + 1 )
    {
        rc = ~(int)( gamma + 1 );
        parent_leaf[gamma + 1] = (int)i;
    }
    else
    {
        rc = (int)( gamma + 1 );
        parent_node[gamma + 1] = (int)i;
    }
    left[i] = lc;
    right[i] = rc;
    range_lo[i] = (int)lo;
    range_hi[i] = (int)hi;
}

struct Box
{
    float lo[3], hi[3];
};

__device__ __forceinline__ void store_child_box( float4 *nodes, int parent, bool is_left,
                                                 Box const &b )
{
    float *n = reinterpret_cast<float *>( nodes + 4 * (int64_t)parent );
    int const o = is_left ? 0 : 6;
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        __stcg( n + o + d, b.lo[d] );
        __stcg( n + o + 3 + d, b.hi[d] );
    }
}

__device__ __forceinline__ Box load_child_box( float4 const *nodes, int parent, bool is_left )
{
    float const *n = reinterpret_cast<float const *>( nodes + 4 * (int64_t)parent );
    int const o = is_left ? 0 : 6;
    Box b;
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        b.lo[d] = __ldcg( n + o + d );
        b.hi[d] = __ldcg( n + o + 3 + d );
    }
    return b;
}

// One thread per leaf: leaf box, then walk up; the second child to arrive at
// a node computes its box and continues.
__global__ void k_refit( double2 const *s2,
                         double const *scene, int32_t const *leaf_start, int64_t nl, int const *left,
                         int const *right,
                         int const *parent_node, int const *parent_leaf, float4 *nodes,
                         unsigned *flags, float4 *root_box, unsigned *status )
{
    int64_t const leaf = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( leaf >= nl )
        return;
    int64_t const begin = leaf_start[leaf], end = leaf_start[leaf + 1];
    double lo[3] = {s2[2 * begin].x, s2[2 * begin].y, s2[2 * begin + 1].x};
    double hi[3] = {lo[0], lo[1], lo[2]};
    for ( int64_t p = begin + 1; p < end; ++p )
    {
        double const c[3] = {s2[2 * p].x, s2[2 * p].y, s2[2 * p + 1].x};
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            lo[d] = fmin( lo[d], c[d] );
            hi[d] = fmax( hi[d], c[d] );
        }
    }
    // centred FP32 box, rounded outward and widened by one FP32 ulp so that
    // it contains the exact centred coordinates despite the FP64 subtraction
    Box b;
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        b.lo[d] = nextafterf( __double2float_rd( lo[d] - scene[9 + d] ), -INFINITY );
        b.hi[d] = nextafterf( __double2float_ru( hi[d] - scene[9 + d] ), INFINITY );
    }
    if ( nl == 1 )
    {
        root_box[0] = make_float4( b.lo[0], b.lo[1], b.lo[2], b.hi[0] );
        root_box[1] = make_float4( b.hi[1], b.hi[2], 0.f, 0.f );
        return;
    }
    int node = parent_leaf[leaf];
    int child = ~(int)leaf;
    // A radix tree over nl leaves is at most nl - 1 levels deep; the cap only
    // turns a malformed tree into a reported error instead of a hang.
    for ( int64_t guard = 0; guard < nl; ++guard )
    {
        store_child_box( nodes, node, left[node] == child, b );
        __threadfence();
        unsigned const prev = atomicAdd( &flags[node], 1u );
        if ( prev == 0 )
            return; // sibling not done yet; it will continue upwards
        __threadfence();
        Box const a = load_child_box( nodes, node, true );
        Box const c = load_child_box( nodes, node, false );
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            b.lo[d] = fminf( a.lo[d], c.lo[d] );
            b.hi[d] = fmaxf( a.hi[d], c.hi[d] );
        }
        if ( node == 0 )
        {
            root_box[0] = make_float4( b.lo[0], b.lo[1], b.lo[2], b.hi[0] );
            root_box[1] = make_float4( b.hi[1], b.hi[2], 0.f, 0.f );
            return;
        }
        child = node;
        node = parent_node[node];
        if ( node < 0 || node >= nl - 1 )
            break;
    }
    atomicOr( status, DEV_BAD_INDEX ); // malformed tree
}

__global__ void k_pack_children( int64_t n_internal, int const *left, int const *right,
                                 int const *range_lo, int const *range_hi, float4 *nodes )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i < n_internal )
        nodes[4 * i + 3] = make_float4( __int_as_float( left[i] ), __int_as_float( right[i] ),
                                        __int_as_float( range_lo[i] ), __int_as_float( range_hi[i] ) );
}

// ---------------------------------------------------------------------------
// 8-wide BVH: the binary radix tree collapsed three levels at a time.  Every
// binary node at a depth divisible by 3 becomes a wide node whose children
// are its descendants three levels down (or the leaves met on the way), in
// binary left-to-right order, so child leaf ranges ascend.  Child slot c of
// wide node w is 3 float4 at wide[24 w + 3 c]: (lo.x, lo.y, lo.z, hi.x),
// (hi.y, hi.z, ref, end), (range_lo, range_hi, -, -), with ref >= 0 a wide
// node, ref < 0 a leaf of the sorted positions [~ref, end), and WIDE_EMPTY
// an unused slot (box lo = +inf, hi = -inf, so its lower bound is +inf);
// range_lo/hi are the leaf indices the child covers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_node( float4 const *nodes, int node, float *l_lo,
                                           float *l_hi, float *r_lo, float *r_hi, int &lc,
                                           int &rc, int &lo, int &hi )
{
    float4 const a = __ldg( nodes + 4 * (int64_t)node );
    float4 const b = __ldg( nodes + 4 * (int64_t)node + 1 );
    float4 const c = __ldg( nodes + 4 * (int64_t)node + 2 );
    float4 const e = __ldg( nodes + 4 * (int64_t)node + 3 );
    l_lo[0] = a.x;
    l_lo[1] = a.y;
    l_lo[2] = a.z;
    l_hi[0] = a.w;
    l_hi[1] = b.x;
    l_hi[2] = b.y;
    r_lo[0] = b.z;
    r_lo[1] = b.w;
    r_lo[2] = c.x;
    r_hi[0] = c.y;
    r_hi[1] = c.z;
    r_hi[2] = c.w;
    lc = __float_as_int( e.x );
    rc = __float_as_int( e.y );
    lo = __float_as_int( e.z );
    hi = __float_as_int( e.w );
}

constexpr int WIDE = 8;
constexpr int WIDE_EMPTY = INT_MIN;

// Child slot c of wide node `node`: its box, ref and (RANGE) leaf range.
// A node is 8 x 32 bytes (one sector a child); the leaf ranges, needed only
// by trees over several problems, are a separate array.
template <bool RANGE>
__device__ __forceinline__ void load_wide( float4 const *wide, int2 const *wide_range, int node, int c,
                                           float *lo, float *hi, int &ref, int &end, int &rlo, int &rhi )
{
    float4 const *p = wide + 16 * (int64_t)node + 2 * c;
    float4 const a = __ldg( p ), b = __ldg( p + 1 );
    lo[0] = a.x;
    lo[1] = a.y;
    lo[2] = a.z;
    hi[0] = a.w;
    hi[1] = b.x;
    hi[2] = b.y;
    ref = __float_as_int( b.z );
    end = __float_as_int( b.w );
    if ( RANGE )
    {
        int2 const e = __ldg( wide_range + 8 * (int64_t)node + c );
        rlo = e.x;
        rhi = e.y;
    }
}

// Wide nodes: the binary nodes at depths 0, 3, 6, ...; max_depth gets the
// largest binary depth (the wide levels bound the traversal stacks).
__global__ void k_depth_flags( int64_t ni, int const *parent_node, int64_t *flag, unsigned *max_depth,
                               unsigned *status )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= ni )
        return;
    int64_t d = 0;
    int j = (int)i;
    while ( j != 0 )
    {
        j = parent_node[j];
        ++d;
        if ( d > ni || j < 0 || j >= ni )
        {
            atomicOr( status, DEV_BAD_INDEX ); // malformed tree
            break;
        }
    }
    flag[i] = d % 3 == 0 ? 1 : 0;
    unsigned const m = __activemask();
    unsigned const dm = __reduce_max_sync( m, (unsigned)d );
    if ( ( threadIdx.x & 31 ) == __ffs( m ) - 1 )
        atomicMax( max_depth, dm );
}

__device__ __forceinline__ uint32_t compact10( uint32_t v )
{
    v &= 0x09249249u;
    v = ( v ^ ( v >> 2 ) ) & 0x030C30C3u;
    v = ( v ^ ( v >> 4 ) ) & 0x0300F00Fu;
    v = ( v ^ ( v >> 8 ) ) & 0x030000FFu;
    v = ( v ^ ( v >> 16 ) ) & 0x000003FFu;
    return v;
}

// The Morton cell of each wide node (binary node i at a depth divisible by 3)
// as a box in the scene-centred FP32 frame, and its parent wide node.  Every
// point of the node lies in the cell of the common prefix of its first and
// last leaves' first codes (the leaves are cells).  The box is inset by a
// margin of 2^-18 (|c| + S + extent), which covers the FP32 rounding of the
// Morton quantization; a side at the end of the quantized range is open (no
// source lies beyond the scene box).  A cell that also holds points outside
// the node (a run of equal codes split between leaves by position: the
// point just before or just after the node's range shares the prefix) holds
// no ball: its box is left empty, so a search never starts there.
// wide_cell[2 w] = (lo, parent), wide_cell[2 w + 1] = (hi, -).
__global__ void k_wide_cells( int64_t ni, int64_t n, int64_t const *flag, int64_t const *widx,
                              int const *parent_node, int const *range_lo, int const *range_hi,
                              int32_t const *leaf_start, uint32_t const *codes, double const *scene,
                              float4 *wide_cell )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= ni || !flag[i] )
        return;
    uint32_t const c1 = codes[leaf_start[range_lo[i]]], c2 = codes[leaf_start[range_hi[i]]];
    int const len = c1 == c2 ? 30 : __clz( c1 ^ c2 ) - 2;
    int64_t const p0 = leaf_start[range_lo[i]], p1 = leaf_start[range_hi[i] + 1];
    bool shared = false;
    if ( len > 0 )
    {
        auto same = [&]( uint32_t c ) { return ( c >> ( 30 - len ) ) == ( c1 >> ( 30 - len ) ); };
        shared = ( p0 > 0 && same( codes[p0 - 1] ) ) || ( p1 < n && same( codes[p1] ) );
    }
    double const ext = fmax( scene[6] - scene[0], fmax( scene[7] - scene[1], scene[8] - scene[2] ) );
    double const cmax = fmax( fabs( scene[9] ), fmax( fabs( scene[10] ), fabs( scene[11] ) ) );
    double const mg = ldexp( cmax + scene[12] + ext, -18 );
    float lo[3], hi[3];
#pragma unroll
    for ( int a = 0; a < 3; ++a )
    {
        int const nb = len > a ? ( len - a + 2 ) / 3 : 0; // fixed bits of axis a
        uint32_t const q = compact10( c1 >> ( 2 - a ) );
        uint32_t const qmin = nb ? ( q >> ( 10 - nb ) ) << ( 10 - nb ) : 0u;
        uint32_t const qmax = qmin + ( 1u << ( 10 - nb ) ) - 1u;
        double const scale = scene[3 + a], c = scene[9 + a];
        double const dlo = ( qmin == 0u || scale == 0.0 ) ? -INFINITY : scene[a] + qmin / scale - c + mg;
        double const dhi = ( qmax >= 1023u || scale == 0.0 ) ? INFINITY : scene[a] + ( qmax + 1 ) / scale - c - mg;
        lo[a] = __double2float_ru( dlo );
        hi[a] = __double2float_rd( dhi );
    }
    if ( shared )
#pragma unroll
        for ( int a = 0; a < 3; ++a )
        {
            lo[a] = __int_as_float( 0x7f800000 );  // +inf
            hi[a] = -__int_as_float( 0x7f800000 ); // -inf
        }
    int p = (int)i;
    for ( int t = 0; t < 3 && p != 0; ++t )
        p = parent_node[p];
    int const parent = i == 0 ? -1 : (int)widx[p];
    wide_cell[2 * widx[i]] = make_float4( lo[0], lo[1], lo[2], __int_as_float( parent ) );
    wide_cell[2 * widx[i] + 1] = make_float4( hi[0], hi[1], hi[2], 0.f );
}

__global__ void k_collapse( int64_t ni, float4 const *nodes, int64_t const *flag, int64_t const *widx,
                            int32_t const *leaf_start, float4 *wide, int2 *wide_range )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= ni || !flag[i] )
        return;
    int ref[WIDE];
    Box box[WIDE];
    int rlo[WIDE], rhi[WIDE];
    int cnt = 0;
    // the children of binary node j from its record
    auto append_children = [&]( int j, int *r, Box *bx, int *lo, int *hi, int &c ) {
        float l_lo[3], l_hi[3], r_lo[3], r_hi[3];
        int lc, rc, nlo, nhi;
        load_node( nodes, j, l_lo, l_hi, r_lo, r_hi, lc, rc, nlo, nhi );
        int const gamma = lc >= 0 ? lc : ~lc;
        r[c] = lc;
        lo[c] = nlo;
        hi[c] = gamma;
        for ( int d = 0; d < 3; ++d )
        {
            bx[c].lo[d] = l_lo[d];
            bx[c].hi[d] = l_hi[d];
        }
        ++c;
        r[c] = rc;
        lo[c] = gamma + 1;
        hi[c] = nhi;
        for ( int d = 0; d < 3; ++d )
        {
            bx[c].lo[d] = r_lo[d];
            bx[c].hi[d] = r_hi[d];
        }
        ++c;
    };
    append_children( (int)i, ref, box, rlo, rhi, cnt );
    for ( int round = 0; round < 2; ++round )
    {
        int nref[WIDE], nlo[WIDE], nhi[WIDE], n2 = 0;
        Box nbox[WIDE];
        for ( int c = 0; c < cnt; ++c )
        {
            if ( ref[c] >= 0 )
                append_children( ref[c], nref, nbox, nlo, nhi, n2 );
            else
            {
                nref[n2] = ref[c];
                nbox[n2] = box[c];
                nlo[n2] = rlo[c];
                nhi[n2] = rhi[c];
                ++n2;
            }
        }
        for ( int c = 0; c < n2; ++c )
        {
            ref[c] = nref[c];
            box[c] = nbox[c];
            rlo[c] = nlo[c];
            rhi[c] = nhi[c];
        }
        cnt = n2;
    }
    float4 *out = wide + 16 * widx[i];
    int2 *out_range = wide_range + 8 * widx[i];
    for ( int c = 0; c < WIDE; ++c )
    {
        if ( c < cnt )
        {
            // a leaf child carries its first and end positions
            int const r = ref[c] >= 0 ? (int)widx[ref[c]] : ~leaf_start[~ref[c]];
            int const end = ref[c] >= 0 ? 0 : leaf_start[~ref[c] + 1];
            out[2 * c] = make_float4( box[c].lo[0], box[c].lo[1], box[c].lo[2], box[c].hi[0] );
            out[2 * c + 1] = make_float4( box[c].hi[1], box[c].hi[2], __int_as_float( r ), __int_as_float( end ) );
            out_range[c] = make_int2( rlo[c], rhi[c] );
        }
        else
        {
            out[2 * c] = make_float4( INFINITY, INFINITY, INFINITY, -INFINITY );
            out[2 * c + 1] = make_float4( -INFINITY, -INFINITY, __int_as_float( WIDE_EMPTY ), 0.f );
            out_range[c] = make_int2( 1, 0 );
        }
    }
}

// ---------------------------------------------------------------------------
// Queries
// ---------------------------------------------------------------------------
struct GroupView
{
    int64_t const *src_off;  // per group: its sources' sorted positions [src_off[g], src_off[g+1])
    uint32_t const *tgt_grp; // group of each target
    int32_t const *k;        // per-group k (kNN)
    double const *r;         // per-group radius
};

struct TreeView
{
    double2 const *s2; // Morton-sorted FP64 points: (x, y), (z, original index bits)
    float4 const *f4; // centred FP32 coordinates (x, y, z; w unused: one 16-byte load a point)
    uint32_t const *codes, *perm;
    int32_t const *leaf_start, *leaf_of;
    float4 const *wide; // 8-wide nodes (16 float4 each)
    int2 const *wide_range; // per wide node: its children's leaf ranges (8 int2)
    float4 const *wide_cell; // per wide node: its Morton cell (lo + parent, hi)
    double const *scene;
    int64_t n, nl, nw;
    int levels; // the deepest wide node's level (the root's is 0)
    int64_t step_cap; // traversal steps a query may take (<= nw, the most it needs)
};

// FP32 lower bound of the squared distance between any point of [lo, hi]
// and any point of the query interval [qlo, qhi] (round-down arithmetic).
__device__ __forceinline__ float box_lb( float const *lo, float const *hi,
                                         float const *qlo, float const *qhi )
{
    float acc = 0.f;
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        float g = fmaxf( 0.f, fmaxf( __fsub_rd( lo[d], qhi[d] ), __fsub_rd( qlo[d], hi[d] ) ) );
        acc = __fmaf_rd( g, g, acc );
    }
    return acc;
}

// Upper FP32 threshold for pruning against an FP64 bound (2^-20 margin).
// A non-negative double (its bits) rounded up to a float on the integer pipe
// (the conversion instruction runs on the FP64 pipe, the scarcest on GB300):
// the exponent rebiased, the mantissa cut to 23 bits and incremented when
// anything was cut (a carry moves to the next binade, or to +inf); +inf for
// +inf, NaN and values above FLT_MAX.  Results below the normal range take
// the conversion instruction (distances that small are rare).
__device__ __forceinline__ float ru_float_of( unsigned long long b )
{
    if ( b >= 0x7ff0000000000000ull )
        return __int_as_float( 0x7f800000 );
    int const fe = (int)( b >> 52 ) - 1023 + 127;
    if ( fe >= 255 )
        return __int_as_float( 0x7f800000 );
    if ( fe <= 0 )
        return __double2float_ru( __longlong_as_double( (long long)b ) );
    uint32_t const bits = ( (uint32_t)fe << 23 ) | (uint32_t)( ( b >> 29 ) & 0x7fffffu );
    return __uint_as_float( bits + ( ( b & 0x1fffffffull ) != 0 ? 1u : 0u ) );
}

__device__ __forceinline__ float prune_threshold( unsigned long long bound_bits )
{
    if ( bound_bits >= 0x7ff0000000000000ull )
        return __int_as_float( 0x7f800000 ); // +inf (list not full): prune nothing
    return __fmul_ru( ru_float_of( bound_bits ), 1.0f + 9.5367431640625e-07f );
}

__device__ __forceinline__ bool key_less( unsigned long long ad, int ai,
                                          unsigned long long bd, int bi )
{
    return ad < bd || ( ad == bd && ai < bi );
}

// Bitonic network over the warp's 32 (d, i, p) entries, ascending by
// (d, i): every stage (FULL_SORT), or only the final merge of size 32 (for a
// bitonic input).
template <bool FULL_SORT>
__device__ __forceinline__ void exact_network( unsigned long long &d, int &i, int &p, int lane )
{
#pragma unroll
    for ( int size = FULL_SORT ? 2 : 32; size <= 32; size <<= 1 )
#pragma unroll
        for ( int stride = size >> 1; stride > 0; stride >>= 1 )
        {
            unsigned long long const od = __shfl_xor_sync( FULL, d, stride );
            int const oi = __shfl_xor_sync( FULL, i, stride );
            int const op = __shfl_xor_sync( FULL, p, stride );
            bool const up = ( lane & size ) == 0 || size == 32;
            bool const lower = ( lane & stride ) == 0;
            bool const mine_less = key_less( d, i, od, oi );
            if ( ( lower == up ) ? !mine_less : mine_less )
            {
                d = od;
                i = oi;
                p = op;
            }
        }
}

// The same order at a third of the cost: the network runs on 32-bit keys
// (bits 62..31 of d, order-preserving for d >= 0) with the source lane as the
// only payload, and each lane then fetches its entry from its source lane.
// On equal keys a compare-exchange copies one entry over the other, but the
// keys themselves are sorted all the same, so two real entries with equal
// keys (distances within 2^-21, or tied) end up side by side: the warp then
// runs the exact network on its untouched entries.  Sentinels (d = KEY_INF,
// key 0xffffffff, all alike) may be copied freely.
template <bool FULL_SORT>
__device__ __forceinline__ void sort_entries( unsigned long long &d, int &i, int &p, int lane )
{
    uint32_t key = (uint32_t)( d >> 31 );
    int src = lane;
#pragma unroll
    for ( int size = FULL_SORT ? 2 : 32; size <= 32; size <<= 1 )
#pragma unroll
        for ( int stride = size >> 1; stride > 0; stride >>= 1 )
        {
            uint32_t const ok = __shfl_xor_sync( FULL, key, stride );
            int const os = __shfl_xor_sync( FULL, src, stride );
            bool const up = ( lane & size ) == 0 || size == 32;
            bool const lower = ( lane & stride ) == 0;
            bool const mine_less = key < ok;
            if ( ( lower == up ) ? !mine_less : mine_less )
            {
                key = ok;
                src = os;
            }
        }
    uint32_t const next = __shfl_down_sync( FULL, key, 1 );
    bool const tie = lane < 31 && key == next && key != 0xffffffffu;
    if ( __ballot_sync( FULL, tie ) )
        exact_network<FULL_SORT>( d, i, p, lane );
    else
    {
        unsigned long long const nd = __shfl_sync( FULL, d, src );
        int const ni = __shfl_sync( FULL, i, src );
        int const np = __shfl_sync( FULL, p, src );
        d = nd;
        i = ni;
        p = np;
    }
}


// 32-ary lower_bound of `code` in the sorted codes (warp-uniform result).
__device__ __forceinline__ int64_t warp_lower_bound( uint32_t const *codes, int64_t n,
                                                     uint32_t code, int lane )
{
    int64_t lo = 0, hi = n;
    while ( hi - lo > 32 )
    {
        int64_t const step = ( hi - lo + 31 ) / 32;
        int64_t const p = lo + lane * step;
        bool const pred = p < hi && __ldg( codes + p ) < code;
        unsigned const b = __ballot_sync( FULL, pred );
        int const cnt = __popc( b );
        int64_t const nlo = cnt ? lo + ( cnt - 1 ) * step + 1 : lo;
        int64_t const nhi = ( cnt < 32 && lo + cnt * step < hi ) ? lo + cnt * step : hi;
        lo = nlo;
        hi = nhi;
    }
    bool const pred = lo + lane < hi && __ldg( codes + lo + lane ) < code;
    return lo + __popc( __ballot_sync( FULL, pred ) );
}


// The problem (group) of a query: its sources' sorted-position range
// [ps, pe) and leaf range [lps, lpe]; an ungrouped tree has one group.
struct Range
{
    int64_t ps, pe;
    int lps, lpe;
    int g;
};

template <bool GROUPED>
__device__ __forceinline__ Range query_range( TreeView const &tr, GroupView const &gv, int64_t qi )
{
    Range r;
    r.g = GROUPED ? (int)gv.tgt_grp[qi] : 0;
    r.ps = GROUPED ? gv.src_off[r.g] : 0;
    r.pe = GROUPED ? gv.src_off[r.g + 1] : tr.n;
    r.lps = GROUPED && r.pe > r.ps ? tr.leaf_of[r.ps] : 0;
    r.lpe = GROUPED ? ( r.pe > r.ps ? tr.leaf_of[r.pe - 1] : -1 ) : (int)tr.nl - 1;
    return r;
}

// The query in the centred frame: an FP32 interval [qlo, qhi] certain to
// contain t - c, its FP32 rounding tf, and the per-axis error bound E of an
// FP32 coordinate difference: |fl(pf - tf) - (p - t)| <= E for every source
// (E = 2^-22 (S + T), twice the 2u(|p - c| + |t - c|) bound).
struct Query
{
    double tx, ty, tz;
    float qlo[3], qhi[3], tf[3];
    float err;
};

__device__ __forceinline__ Query make_query( double const *scene, PointsView const &tgt, int64_t qi )
{
    Query q;
    q.tx = tgt( qi, 0 );
    q.ty = tgt( qi, 1 );
    q.tz = tgt( qi, 2 );
    double const tc[3] = {q.tx - scene[9], q.ty - scene[10], q.tz - scene[11]};
    float tmax = 0.f;
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        // one rounding to nearest (within half an ulp of t - c), widened by
        // an ulp each way: the conversions run on the FP64 pipe
        q.tf[d] = __double2float_rn( tc[d] );
        q.qlo[d] = nextafterf( q.tf[d], -INFINITY );
        q.qhi[d] = nextafterf( q.tf[d], INFINITY );
        tmax = fmaxf( tmax, fmaxf( fabsf( q.qlo[d] ), fabsf( q.qhi[d] ) ) );
    }
    q.err = ( reinterpret_cast<float const *>( scene + 13 )[6] + tmax ) * 2.384185791015625e-07f; // 2^-22
    return q;
}

// The w-th query in processing order, prepared once per target (the FP64
// subtractions and conversions off the search's FP64 pipe, the interval's
// round-ups off its issue slots): the search copies the 64-byte record into
// shared memory with one coalesced load.
static_assert( sizeof( Query ) == 64, "a query record is 16 words" );
__global__ void k_query_frame( PointsView tgt, uint32_t const *order, double const *scene, Query *qrec )
{
    int64_t const w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( w >= tgt.n )
        return;
    qrec[w] = make_query( scene, tgt, order ? (int64_t)order[w] : w );
}

// Sorted source p: the FP64 squared distance to the query (the exact key)
// and the source's original index (its bits in .y); two 16-byte loads.
__device__ __forceinline__ double2 sorted_dist2( TreeView const &tr, int64_t p, Query const &q )
{
    double2 const a = __ldg( tr.s2 + 2 * p ), b = __ldg( tr.s2 + 2 * p + 1 );
    return make_double2( dist2_rn( a.x, a.y, b.x, q.tx, q.ty, q.tz ), b.y );
}

// FP32 bounds lo <= d2(p, t) <= hi for sorted source p (centred FP32 copy).
__device__ __forceinline__ void d2_bounds( TreeView const &tr, Query const &q, int64_t p,
                                           float &lo, float &hi )
{
    float4 const f = __ldg( tr.f4 + p );
    float const dx = f.x - q.tf[0];
    float const dy = f.y - q.tf[1];
    float const dz = f.z - q.tf[2];
    float const d2 = fmaf( dz, dz, fmaf( dy, dy, dx * dx ) );
    float const spread = q.err * ( 4.f * ( fabsf( dx ) + fabsf( dy ) + fabsf( dz ) ) + 3.f * q.err ) +
                         d2 * 9.5367431640625e-07f;
    lo = d2 - spread;
    hi = d2 + spread;
}

// Screen threshold for the computed FP32 squared distance d2_f of a point
// (d2_bounds without the spread): every point whose rigorous lower bound
// d2_f - spread(p) is at most b, spread(p) = E (4 (|dx| + |dy| + |dz|) + 3E)
// + d2_f 2^-20, has d2_f <= T.  With |dx| + |dy| + |dz| <= sqrt(3.0001 d2_f)
// (Cauchy-Schwarz and the FP32 rounding of d2_f), x = sqrt(d2_f) satisfies
// (1 - 2^-20) x^2 - 7E x - c <= 0 for c = b + 3E^2, so
// d2_f <= (c + 14E sqrt(c) + 49E^2) / (1 - 2^-20)^2; every step rounds up
// and the factor 1 + 2^-16 covers the division.
__device__ __forceinline__ float screen_threshold( float b, float err )
{
    if ( !( b < __int_as_float( 0x7f800000 ) ) )
        return __int_as_float( 0x7f800000 );
    float const c = __fmaf_ru( __fmul_ru( 3.f, err ), err, b );
    float const e7 = __fmul_ru( 7.f, err );
    float const t = __fmaf_ru( e7, e7, __fmaf_ru( __fmul_ru( 2.f, e7 ), __fsqrt_ru( c ), c ) );
    return __fmul_ru( t, 1.0000152587890625f ); // 1 + 2^-16
}

constexpr int QUEUE = 64;
constexpr float SPEC_GROWTH = 1.25f; // speculative k-th squared distance over the previous query's
// A chunk's leaf list: after the chunk's first query, the leaves within
// LIST_GROWTH x its k-th squared distance of the box of the chunk's other
// queries (at most LIST_CAP, else none), which those queries scan instead of
// traversing the tree.
constexpr int LIST_CAP = 128;
constexpr float LIST_GROWTH = 1.5f;

// Queries go to warps in chunks of Morton-consecutive queries (each query
// seeds the next): n_big chunks of seq queries, then chunks of seq / 2 up to
// the end, so that the warps finish close together.  A warp takes the next
// chunk from a counter as soon as it is done with one.
struct KnnChunks
{
    int seq;
    int64_t n_big;
    unsigned *next;
};

__device__ __forceinline__ void chunk_range( KnnChunks const &ch, unsigned c, int64_t &w0, int64_t &len )
{
    if ( c < ch.n_big )
    {
        w0 = (int64_t)c * ch.seq;
        len = ch.seq;
    }
    else
    {
        int const tail = ch.seq > 1 ? ch.seq / 2 : 1;
        w0 = ch.n_big * ch.seq + ( (int64_t)c - ch.n_big ) * tail;
        len = tail;
    }
}

// The leaf list of a kNN chunk: every leaf whose box lies within r2 =
// LIST_GROWTH x kth (the chunk's first query's k-th key, rounded up) of the
// box of queries [x0, x1) (the union of their FP32 intervals), collected by
// one traversal into list; a query of the chunk whose k-th key is proven
// below r2 then lost nothing to the leaves left out.  Too many leaves: no
// list (*n_list = -1).  Out of line: it runs once a chunk, and its
// registers stay out of the query loop's.
__device__ __noinline__ void chunk_leaf_list( float4 const *wide, int64_t step_cap, int levels,
                                              Query const *qrec, int64_t x0, int64_t x1, float kth,
                                              int *stack, int *list, int *n_list, float *list_r2 )
{
    int const lane = threadIdx.x & 31;
    unsigned const lt_mask = ( 1u << lane ) - 1u;
    float const r2 = __fmul_ru( kth, LIST_GROWTH );
    float blo[3], bhi[3];
#pragma unroll
    for ( int d = 0; d < 3; ++d )
    {
        blo[d] = __int_as_float( 0x7f800000 );
        bhi[d] = -__int_as_float( 0x7f800000 );
    }
    for ( int64_t x = x0 + lane; x < x1; x += 32 )
    {
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            blo[d] = fminf( blo[d], __ldg( qrec[x].qlo + d ) );
            bhi[d] = fmaxf( bhi[d], __ldg( qrec[x].qhi + d ) );
        }
    }
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
#pragma unroll
        for ( int d = 0; d < 3; ++d )
        {
            blo[d] = fminf( blo[d], __shfl_xor_sync( FULL, blo[d], o ) );
            bhi[d] = fmaxf( bhi[d], __shfl_xor_sync( FULL, bhi[d], o ) );
        }
    int n = 0, sp = 0;
    bool over = !( r2 < __int_as_float( 0x7f800000 ) );
    int const grp = lane >> 3, slot = lane & 7;
    int node = grp == 0 ? 0 : -1;
    for ( int64_t guard = 0; !over; ++guard )
    {
        if ( guard >= step_cap )
        {
            over = true;
            break;
        }
        float lb = __int_as_float( 0x7f800000 );
        int ref = WIDE_EMPTY, lend = 0;
        if ( node >= 0 )
        {
            float lo[3], hi[3];
            int rlo = 0, rhi = 0;
            load_wide<false>( wide, nullptr, node, slot, lo, hi, ref, lend, rlo, rhi );
            lb = box_lb( lo, hi, blo, bhi );
        }
        bool const cand = ref != WIDE_EMPTY && lb <= r2;
        unsigned const ml = __ballot_sync( FULL, cand && ref < 0 );
        unsigned const mi = __ballot_sync( FULL, cand && ref >= 0 );
        int const n_int = __popc( mi ), n_leaf = __popc( ml );
        if ( sp + n_int > STACK || n + n_leaf > LIST_CAP )
        {
            over = true;
            break;
        }
        if ( cand && ref >= 0 )
            stack[sp + __popc( mi & lt_mask )] = ref;
        if ( cand && ref < 0 )
            list[n + __popc( ml & lt_mask )] = node * WIDE + slot;
        sp += n_int;
        n += n_leaf;
        __syncwarp();
        // as the query traversal: four nodes a step while a descent fits
        int const P = sp + ( NODE_GROUPS + levels ) * ( WIDE - 1 ) <= STACK ? NODE_GROUPS : 1;
        int const taken = sp < P ? sp : P;
        if ( taken == 0 )
            break;
        node = grp < taken ? stack[sp - 1 - grp] : -1;
        sp -= taken;
        __syncwarp();
    }
    if ( lane == 0 )
    {
        *n_list = over ? -1 : n;
        *list_r2 = r2;
    }
    __syncwarp();
}

template <bool GROUPED>
__global__ void __launch_bounds__( Q_WARPS * 32, KNN_BLOCKS_PER_SM )
    k_knn( TreeView tr, PointsView tgt, uint32_t const *order, Query const *qrec, int k_all, KnnChunks ch,
           GroupView gv,
           int32_t const *offset, int32_t *idx_out, int32_t *pos_out, unsigned *status )
{
    // the stack of wide nodes to enter: small, to leave most of the SM's L1
    // to the tree and the points
    __shared__ int s_stack[Q_WARPS][STACK];
    __shared__ int s_queue[Q_WARPS][QUEUE];
    __shared__ Query s_query[Q_WARPS];
    __shared__ int s_entry[Q_WARPS]; // the wide node the previous query started from
    __shared__ int s_list[Q_WARPS][LIST_CAP]; // the chunk's leaf list (wide node * WIDE + child slot)
    __shared__ int s_nlist[Q_WARPS];          // its length, -1 while there is none
    __shared__ float s_list_r2[Q_WARPS];      // every leaf within this of the chunk's box is listed
    int const lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    unsigned const lt_mask = ( 1u << lane ) - 1u;
    if ( lane == 0 )
        s_entry[wib] = 0;
    for ( ;; )
    {
    unsigned c = 0;
    if ( lane == 0 )
        c = atomicAdd( ch.next, 1u );
    c = __shfl_sync( FULL, c, 0 );
    int64_t w0, len;
    chunk_range( ch, c, w0, len );
    if ( w0 >= tgt.n )
        return;
    if ( lane == 0 )
        s_nlist[wib] = -1;
    __syncwarp();
    // the list of the previous query (its sorted positions kp and indices ki)
    // seeds the next one: Morton-consecutive queries share most neighbours
    int prev_g = -1, prev_row = 0;
    // the previous query's k-th distance (squared) times SPEC_GROWTH: a guess
    // of this query's, proven or retried after the search
    float next_spec = __int_as_float( 0x7f800000 );
    unsigned long long kd = KEY_INF;
    int ki = 0x7fffffff, kp = -1;
    // positions and targets are below 2^31 (int32 offsets): 32-bit loop state
    int const wb = (int)w0, we = (int)( w0 + len < tgt.n ? w0 + len : tgt.n );
    bool head = true; // the chunk's first query
    for ( int w = wb; w < we; ++w )
    {
    Range const rg = query_range<GROUPED>( tr, gv, order ? (int)order[w] : w );
    int64_t const ng = rg.pe - rg.ps;
    int const k = GROUPED ? gv.k[rg.g] : k_all;
    int const row = (int)( k < ng ? k : ng );
    if ( row <= 0 )
    {
        prev_row = 0;
        head = false;
        continue;
    }
    // the query waits in shared memory: registers limit how many warps an
    // SM holds, and values there can be re-read instead of spilled
    if ( lane < 16 )
        reinterpret_cast<uint32_t *>( &s_query[wib] )[lane] =
            __ldg( reinterpret_cast<uint32_t const *>( qrec + w ) + lane );
    __syncwarp();
    Query const &q = s_query[wib];
    bool const seeded = prev_row == row && ( !GROUPED || prev_g == rg.g );

    if ( seeded )
    {
        // the previous list with exact keys for this query (lanes past the
        // row hold entries that insertions shifted out: cleared)
        if ( lane < row )
            kd = (unsigned long long)__double_as_longlong(
                sorted_dist2( tr, kp, q ).x );
        else
        {
            kd = KEY_INF;
            ki = 0x7fffffff;
            kp = -1;
        }
    }
    else
    {
        // the 32 Morton-sorted sources of the query's problem around the
        // target's code, with exact keys
        uint32_t const code = morton3( q.tx, q.ty, q.tz, tr.scene );
        int64_t const pos = rg.ps + warp_lower_bound( tr.codes + rg.ps, ng, code, lane );
        int64_t const W = ng < 32 ? ng : (int64_t)32;
        int64_t s0 = pos - 16;
        if ( s0 > rg.pe - W )
            s0 = rg.pe - W;
        if ( s0 < rg.ps )
            s0 = rg.ps;
        kd = KEY_INF;
        ki = 0x7fffffff;
        kp = -1;
        if ( lane < W )
        {
            int64_t const p = s0 + lane;
            double2 const e = sorted_dist2( tr, p, q );
            kd = (unsigned long long)__double_as_longlong( e.x );
            ki = (int)__double_as_longlong( e.y );
            kp = (int)p;
        }
    }
    // the 32 keys ascending across lanes
    sort_entries<true>( kd, ki, kp, lane );
    if ( lane >= k )
    {
        kd = KEY_INF;
        ki = 0x7fffffff;
        kp = -1;
    }
    // speculative bound (seeded queries with full rows): boxes and points
    // beyond it are skipped as if the list were already that tight.  A query
    // that scans its chunk's leaf list skips every leaf beyond the list's
    // bound as well.
    float spec = seeded && row == k ? next_spec : __int_as_float( 0x7f800000 );
    bool list_pass = !GROUPED && !head && row == k && s_nlist[wib] >= 0;
    if ( list_pass )
        spec = fminf( spec, s_list_r2[wib] );
    float bound_f = fminf( prune_threshold( __shfl_sync( FULL, kd, k - 1 ) ), spec );
    float screen_f = screen_threshold( bound_f, q.err ); // the leaf screen's bound
    int qn = 0; // queued survivors (warp-uniform)
    float kth_ru = __int_as_float( 0x7f800000 ); // the final k-th key rounded up to FP32

    // Exact FP64 keys for up to 32 queued sources, merged into the list as a
    // batch: the candidates below the bound are sorted (bitonic) and merged
    // with the list (elementwise minimum against the reversed candidates, then
    // a bitonic clean), keeping the k smallest (d2, index).  No candidate is
    // in the list already: the list's members are screened out of a leaf.
    auto flush = [&]( int count, bool last ) {
        int const p = lane < count ? s_queue[wib][lane] : -1;
        __syncwarp();
        unsigned long long cd = KEY_INF;
        int ci = 0x7fffffff, cp = -1;
        if ( p >= 0 )
        {
            double2 const e = sorted_dist2( tr, p, q );
            cd = (unsigned long long)__double_as_longlong( e.x );
            ci = (int)__double_as_longlong( e.y );
            cp = p;
        }
        // the list's k-th key, the bound a candidate must beat
        unsigned long long const bd = __shfl_sync( FULL, kd, k - 1 );
        int const bi = __shfl_sync( FULL, ki, k - 1 );
        bool live = key_less( cd, ci, bd, bi );
        if ( __ballot_sync( FULL, live ) )
        {
            if ( !live )
            {
                cd = KEY_INF;
                ci = 0x7fffffff;
                cp = -1;
            }
            // candidates ascending
            sort_entries<true>( cd, ci, cp, lane );
            // the list (ascending) against the reversed candidates: the 32
            // smallest as a bitonic sequence, then sorted
            {
                unsigned long long const rd = __shfl_sync( FULL, cd, 31 - lane );
                int const ri = __shfl_sync( FULL, ci, 31 - lane );
                int const rp = __shfl_sync( FULL, cp, 31 - lane );
                if ( key_less( rd, ri, kd, ki ) )
                {
                    kd = rd;
                    ki = ri;
                    kp = rp;
                }
            }
            sort_entries<false>( kd, ki, kp, lane );
            if ( lane >= k )
            {
                kd = KEY_INF;
                ki = 0x7fffffff;
                kp = -1;
            }
        }
        // (the pass's last merge: the proof reads the list itself, and a
        // second pass sets its own bounds)
        if ( last )
        {
            qn = 0;
            return;
        }
        bound_f = fminf( prune_threshold( __shfl_sync( FULL, kd, k - 1 ) ), spec );
        screen_f = screen_threshold( bound_f, q.err );
        // move the remaining queue entries to the front
        int const rest = qn - count;
        int const v = lane < rest ? s_queue[wib][count + lane] : 0;
        __syncwarp();
        if ( lane < rest )
            s_queue[wib][lane] = v;
        __syncwarp();
        qn = rest;
    };

    // FP32 screen of a leaf: a source whose FP32 lower bound exceeds the
    // bound cannot beat or tie it (screen_threshold keeps all the others);
    // the survivors queue for exact keys.
    auto process_leaf = [&]( int start, int end ) {
        int const p = start + lane;
        bool surv = false;
        // the list's members in this leaf are screened out: a leaf is
        // screened once a pass, so they are members it started with
        unsigned const seen =
            __reduce_or_sync( FULL, (unsigned)( kp - start ) < (unsigned)( end - start ) ? 1u << ( kp - start ) : 0u );
        if ( ( GROUPED ? p >= rg.ps && p < rg.pe : true ) && p < end && !( ( seen >> lane ) & 1u ) )
        {
            float4 const f = __ldg( tr.f4 + p );
            float const dx = f.x - q.tf[0];
            float const dy = f.y - q.tf[1];
            float const dz = f.z - q.tf[2];
            surv = fmaf( dz, dz, fmaf( dy, dy, dx * dx ) ) <= screen_f;
        }
        unsigned const m = __ballot_sync( FULL, surv );
        if ( surv )
            s_queue[wib][qn + __popc( m & lt_mask )] = p;
        __syncwarp();
        qn += __popc( m );
        if ( qn >= 32 )
            flush( 32, false );
    };

    // A pass searches the tree; a second one follows only when the
    // speculative bound is not proven: the k-th key exceeds it (or the list
    // is not full), so points it skipped may belong to the list.  The second
    // pass screens out the whole list and prunes with the list's own bound.
    for ( ;; )
    {
        if ( tr.nl == 1 )
        {
            process_leaf( 0, (int)tr.n );
        }
        else if ( list_pass )
        {
            // the chunk's leaf list, 32 leaves a round: lane j tests leaf j's
            // box, the leaves that pass are screened in list order
            int const n_list = s_nlist[wib];
            for ( int b = 0; b < n_list; b += 32 )
            {
                int const e = b + lane < n_list ? s_list[wib][b + lane] : -1;
                float lb = __int_as_float( 0x7f800000 );
                int ref = WIDE_EMPTY, lend = 0;
                if ( e >= 0 )
                {
                    float lo[3], hi[3];
                    int rlo = 0, rhi = 0;
                    load_wide<false>( tr.wide, tr.wide_range, e / WIDE, e % WIDE, lo, hi, ref, lend, rlo, rhi );
                    lb = box_lb( lo, hi, q.qlo, q.qhi );
                }
                unsigned const ml = __ballot_sync( FULL, e >= 0 && lb <= bound_f );
                for ( unsigned m = ml; m; m &= m - 1 )
                {
                    int const from = __ffs( m ) - 1;
                    float const lbr = __shfl_sync( FULL, lb, from );
                    int const lref = __shfl_sync( FULL, ref, from );
                    int const le = __shfl_sync( FULL, lend, from );
                    if ( lbr <= bound_f )
                        process_leaf( ~lref, le );
                }
            }
        }
        else
        {
            // Wide-node traversal, up to NODE_GROUPS nodes a step: lane group g
            // (lanes 8g .. 8g+7) tests the 8 children of its node; leaf children
            // are screened in lane order, internal children go on the stack in
            // lane order, and the next step takes the top entries.  A step
            // takes four nodes only while a depth-first descent after them
            // fits, else one
            // entries (at least one), so its children fit on the stack.
            int sp = 0;
            int const grp = lane >> 3, slot = lane & 7;
            // Start node: every point within the speculative bound lies in the
            // subtree of a wide node whose Morton cell holds the ball of that
            // radius (the cell's points are the subtree's), so the search may
            // start there; the proof after the search covers the bound.  A
            // second pass (the bound not proven) starts from the cell that
            // holds the ball of the list's own k-th distance, which bounds
            // every point that can still enter (from the root while the list
            // is not full).  The previous start node is the first guess: up
            // while its cell misses the ball, then down while one internal
            // child's cell holds it.  (Ungrouped trees: the keys of a batch
            // tree carry the problem above the code.)
            int start = 0;
            float const ball = spec < __int_as_float( 0x7f800000 ) ? spec : bound_f;
            if ( !GROUPED && ball < __int_as_float( 0x7f800000 ) )
            {
                float const R = __fadd_ru( __fsqrt_ru( ball ), q.err );
                auto holds = [&]( int w ) {
                    float4 const lo = __ldg( tr.wide_cell + 2 * (int64_t)w ),
                                 hi = __ldg( tr.wide_cell + 2 * (int64_t)w + 1 );
                    return q.tf[0] - R > lo.x && q.tf[1] - R > lo.y && q.tf[2] - R > lo.z &&
                           q.tf[0] + R < hi.x && q.tf[1] + R < hi.y && q.tf[2] + R < hi.z;
                };
                int e = s_entry[wib];
                for ( int64_t g = 0; e > 0 && g < tr.nw && !holds( e ); ++g )
                    e = __float_as_int( __ldg( tr.wide_cell + 2 * (int64_t)e ).w );
                if ( e < 0 )
                    e = 0;
                for ( int64_t g = 0; g < tr.nw; ++g )
                {
                    int cref = -1;
                    if ( lane < WIDE )
                        cref = __float_as_int( __ldg( tr.wide + 16 * (int64_t)e + 2 * lane + 1 ).z );
                    unsigned const m = __ballot_sync( FULL, lane < WIDE && cref >= 0 && holds( cref ) );
                    if ( !m )
                        break;
                    e = __shfl_sync( FULL, cref, __ffs( m ) - 1 );
                }
                __syncwarp();
                if ( lane == 0 )
                    s_entry[wib] = e;
                start = e;
            }
            int node = grp == 0 ? start : -1;
            // every step enters at least one wide node, and every wide node is
            // entered at most once
            for ( int guard = 0;; ++guard )
            {
                if ( guard >= tr.step_cap )
                {
                    if ( lane == 0 )
                        atomicOr( status, DEV_TIMEOUT );
                    break;
                }
                float lb = __int_as_float( 0x7f800000 );
                int ref = WIDE_EMPTY, lend = 0;
                bool ok = false;
                if ( node >= 0 )
                {
                    float lo[3], hi[3];
                    int rlo = 0, rhi = 0;
                    load_wide<GROUPED>( tr.wide, tr.wide_range, node, slot, lo, hi, ref, lend, rlo, rhi );
                    lb = box_lb( lo, hi, q.qlo, q.qhi );
                    ok = ref != WIDE_EMPTY && ( GROUPED ? !( rhi < rg.lps || rlo > rg.lpe ) : true );
                }
                bool const cand = ok && lb <= bound_f;
                unsigned const ml = __ballot_sync( FULL, cand && ref < 0 );
                unsigned const mi = __ballot_sync( FULL, cand && ref >= 0 );
                int const n_int = __popc( mi );
                if ( sp + n_int <= STACK )
                {
                    if ( cand && ref >= 0 )
                    {
                        int const pos = sp + __popc( mi & lt_mask );
                        s_stack[wib][pos] = ref;
                    }
                    sp += n_int;
                }
                else if ( lane == 0 )
                    atomicOr( status, DEV_STACK_OVERFLOW );
                __syncwarp();
                for ( unsigned m = ml; m; m &= m - 1 )
                {
                    int const from = __ffs( m ) - 1;
                    float const lbr = __shfl_sync( FULL, lb, from );
                    int const lref = __shfl_sync( FULL, ref, from );
                    int const le = __shfl_sync( FULL, lend, from );
                    if ( lbr <= bound_f )
                        process_leaf( ~lref, le );
                }
                // the next nodes: the top P entries (a node is pushed only when
                // its box passes the bound; the bound tightens rarely during a
                // search, and a node's children are tested against it again).
                // Four only while the stack has room for their children and
                // for a depth-first descent below them (one node a step adds
                // at most 7 entries a level), else one: the stack holds at
                // most 7 entries per wide level on top of what a four-node
                // step left, so it cannot overflow while 7 levels + 1 fit.
                int const P = sp + ( NODE_GROUPS + tr.levels ) * ( WIDE - 1 ) <= STACK ? NODE_GROUPS : 1;
                int const taken = sp < P ? sp : P;
                if ( taken == 0 )
                    break;
                node = grp < taken ? s_stack[wib][sp - 1 - grp] : -1;
                sp -= taken;
                __syncwarp();
            }
        }
        if ( qn > 0 )
            flush( qn, true );
        // Proof: a skipped box or point had an FP32 lower bound above spec,
        // so its exact squared distance exceeds spec and its FP64 key (a few
        // ulps off the exact value) exceeds spec (1 - 2^-40); a k-th key at
        // or below spec (1 - 2^-20) (tested as its FP32 round-up against the
        // round-down product) loses nothing.
        unsigned long long const bd = __shfl_sync( FULL, kd, k - 1 );
        kth_ru = ru_float_of( bd );
        if ( !( spec < __int_as_float( 0x7f800000 ) ) || kth_ru <= __fmul_rd( spec, 1.0f - 9.5367431640625e-07f ) )
            break;
        spec = __int_as_float( 0x7f800000 );
        list_pass = false;
        bound_f = prune_threshold( bd );
        screen_f = screen_threshold( bound_f, q.err );
    }
    if ( lane < row )
    {
        int const qi = order ? (int)__ldg( order + w ) : w; // reloaded: not kept across the search
        int64_t const o = offset[qi] + lane;
        idx_out[o] = ki;
        if ( pos_out )
            pos_out[o] = kp;
    }
    prev_g = rg.g;
    prev_row = row;
    next_spec = __fmul_ru( __fmul_ru( kth_ru, 1.0f + 9.5367431640625e-07f ), SPEC_GROWTH ); // prune_threshold
    __syncwarp();
    if ( !GROUPED && head && w + 1 < we && row == k && tr.nl > 1 )
        chunk_leaf_list( tr.wide, tr.step_cap, tr.levels, qrec, w + 1, we, kth_ru,
                         s_stack[wib], s_list[wib], s_nlist + wib, s_list_r2 + wib );
    head = false;
    }
    }
}

// Radius traversal shared by the count and fill passes.  FILL=false counts
// hits into counts[qi]; FILL=true writes them at offset[qi] in traversal
// order (Morton order of the sources, lane order inside a leaf).  A source
// is a hit iff sqrt(d2) <= r with the exact FP64 d2; the FP32 bounds decide
// every source whose bound interval lies clear of r^2 (2^-20 margins), and
// only the rest pay for an FP64 distance.
template <bool FILL, bool GROUPED>
__global__ void __launch_bounds__( R_WARPS * 32 )
    k_radius( TreeView tr, PointsView tgt, uint32_t const *order, double r_all, GroupView gv,
              int64_t *counts, int32_t const *offset, int32_t *idx_out, unsigned *status )
{
    __shared__ int s_stack[R_WARPS][STACK];
    int const lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int64_t const w = blockIdx.x * (int64_t)R_WARPS + wib;
    if ( w >= tgt.n )
        return;
    int64_t const qi = order ? (int64_t)order[w] : w;
    Range const rg = query_range<GROUPED>( tr, gv, qi );
    double const r = GROUPED ? gv.r[rg.g] : r_all;
    Query const q = make_query( tr.scene, tgt, qi );
    double const r2 = __dmul_ru( r, r );
    float const bound_f = prune_threshold( (unsigned long long)__double_as_longlong( r2 ) );
    float const in_f = __fmul_rd( __double2float_rd( __dmul_rd( r, r ) ), 1.0f - 9.5367431640625e-07f );
    int64_t cnt = 0;
    int64_t out = FILL ? offset[qi] : 0;
    int64_t const out_end = FILL ? offset[qi + 1] : 0;

    auto process_leaf = [&]( int start, int end ) {
        int const p = start + lane;
        bool hit = false, unsure = false;
        if ( ( GROUPED ? p >= rg.ps && p < rg.pe : true ) && p < end )
        {
            float lo, hi;
            d2_bounds( tr, q, p, lo, hi );
            hit = hi < in_f;                  // certainly inside
            unsure = !hit && !( lo > bound_f ); // neither certainly in nor out
        }
        if ( __any_sync( FULL, unsure ) && unsure )
        {
            double const d2 = sorted_dist2( tr, p, q ).x;
            hit = __dsqrt_rn( d2 ) <= r;
        }
        unsigned const b = __ballot_sync( FULL, hit );
        if ( FILL && hit )
        {
            int64_t const o = out + __popc( b & ( ( 1u << lane ) - 1u ) );
            if ( o < out_end )
                idx_out[o] = (int32_t)__ldg( tr.perm + p );
            else
                atomicOr( status, DEV_BAD_INDEX );
        }
        out += __popc( b );
        cnt += __popc( b );
    };

    if ( tr.nl == 1 )
    {
        process_leaf( 0, (int)tr.n );
    }
    else
    {
        // up to NODE_GROUPS wide nodes a step, lane group g testing the
        // children of its node, as in the kNN traversal; the bound is fixed,
        // so the next step takes the top entries of the stack as they are
        int sp = 0;
        int const grp = lane >> 3, slot = lane & 7;
        int node = grp == 0 ? 0 : -1;
        unsigned const lt_mask = ( 1u << lane ) - 1u;
        // every step enters at least one wide node, and every wide node is
        // entered at most once
        for ( int64_t guard = 0;; ++guard )
        {
            if ( guard >= tr.step_cap )
            {
                if ( lane == 0 )
                    atomicOr( status, DEV_TIMEOUT );
                break;
            }
            bool cand = false;
            int ref = WIDE_EMPTY, lend = 0;
            if ( node >= 0 )
            {
                float lo[3], hi[3];
                int rlo = 0, rhi = 0;
                load_wide<GROUPED>( tr.wide, tr.wide_range, node, slot, lo, hi, ref, lend, rlo, rhi );
                cand = ref != WIDE_EMPTY && box_lb( lo, hi, q.qlo, q.qhi ) <= bound_f &&
                       ( GROUPED ? !( rhi < rg.lps || rlo > rg.lpe ) : true );
            }
            unsigned const ml = __ballot_sync( FULL, cand && ref < 0 );
            unsigned const mi = __ballot_sync( FULL, cand && ref >= 0 );
            int const n_int = __popc( mi );
            if ( sp + n_int <= STACK )
            {
                if ( cand && ref >= 0 )
                    s_stack[wib][sp + __popc( mi & lt_mask )] = ref;
                sp += n_int;
            }
            else if ( lane == 0 )
                atomicOr( status, DEV_STACK_OVERFLOW );
            __syncwarp();
            for ( unsigned m = ml; m; m &= m - 1 )
            {
                int const from = __ffs( m ) - 1;
                int const lref = __shfl_sync( FULL, ref, from );
                process_leaf( ~lref, __shfl_sync( FULL, lend, from ) );
            }
            if ( sp == 0 )
                break;
            // four nodes only while a depth-first descent after them fits
            // (as in the kNN traversal), else one
            int const P = sp + ( NODE_GROUPS + tr.levels ) * ( WIDE - 1 ) <= STACK ? NODE_GROUPS : 1;
            int const take = P < sp ? P : sp;
            node = grp < take ? s_stack[wib][sp - 1 - grp] : -1;
            sp -= take;
            __syncwarp();
        }
    }
    if ( !FILL && lane == 0 )
        counts[qi] = cnt;
    if ( FILL && lane == 0 && out != out_end )
        atomicOr( status, DEV_BAD_INDEX );
}

TreeView view_of( Lbvh const &t )
{
    return TreeView{t.s2.get(), t.f4.get(),
                    t.codes.get(), t.perm.get(), t.leaf_start.get(), t.leaf_of.get(), t.wide.get(),
                    t.wide_range.get(), t.wide_cell.get(), t.scene.get(), t.n, t.n_leaves, t.n_wide,
                    t.wide_levels, traversal_cap( t.n_wide )};
}

unsigned blocks_for( int64_t n, int threads )
{
    return (unsigned)std::max<int64_t>( 1, ( n + threads - 1 ) / threads );
}

} // namespace

void build_lbvh( PointsView src, Lbvh &tree, unsigned *status, cudaStream_t s,
                 uint32_t const *group, int64_t n_groups, std::function<void()> const &after_scene )
{
    int64_t const n = src.n;
    tree.n = n;
    int64_t nl = 0; // known after the sort
    tree.scene.allocate( 17, s );
    int const nb = std::max( 1, std::min<int>( 4 * num_sms(), (int)( ( n + BND_THREADS - 1 ) / BND_THREADS ) ) );
    DeviceBuffer<unsigned long long> partial( 6 * nb, s );
    k_bounds_partial<<<nb, BND_THREADS, 0, s>>>( src, partial.get(), status );
    check_launch( "k_bounds_partial" );
    k_bounds_final<<<1, 32, 0, s>>>( partial.get(), nb, tree.scene.get() );
    check_launch( "k_bounds_final" );
    if ( after_scene )
        after_scene();

    tree.codes.allocate( n, s );
    tree.perm.allocate( n, s );
    k_morton<<<blocks_for( n, 256 ), 256, 0, s>>>( src, tree.scene.get(), tree.codes.get(),
                                                     tree.perm.get() );
    check_launch( "k_morton" );
    radix_sort_pairs( tree.codes.get(), tree.perm.get(), n, 30, s );
    if ( group )
    {
        // problem-major order: a stable sort of the Morton order by group
        tree.grp.allocate( n, s );
        k_group_of<<<blocks_for( n, 256 ), 256, 0, s>>>( group, tree.perm.get(), n, tree.grp.get() );
        check_launch( "k_group_of" );
        int bits = 1;
        while ( ( int64_t( 1 ) << bits ) < n_groups )
            ++bits;
        radix_sort_pairs( tree.grp.get(), tree.perm.get(), n, ( bits + 7 ) / 8 * 8, s );
        k_morton_of<<<blocks_for( n, 256 ), 256, 0, s>>>( src, tree.perm.get(), tree.scene.get(),
                                                            tree.codes.get() );
        check_launch( "k_morton_of" );
    }

    // leaves: the Morton cells of at most LEAF points (their count is needed
    // on the host to size the tree)
    {
        DeviceBuffer<int> dlt( std::max<int64_t>( 1, n - 1 ), s );
        DeviceBuffer<int64_t> lflag( n, s ), lscan( n + 1, s );
        if ( n > 1 )
        {
            k_point_delta<<<blocks_for( n - 1, 256 ), 256, 0, s>>>( tree.codes.get(), tree.grp.get(), n,
                                                                    dlt.get() );
            check_launch( "k_point_delta" );
        }
        k_leaf_flags<<<blocks_for( n, 256 ), 256, 0, s>>>( dlt.get(), n, lflag.get() );
        check_launch( "k_leaf_flags" );
        exclusive_scan_i64( lflag.get(), lscan.get(), n, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &nl, lscan.get() + n, sizeof( int64_t ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        tree.leaf_start.allocate( nl + 1, s );
        tree.leaf_of.allocate( n, s );
        k_leaf_index<<<blocks_for( n, 256 ), 256, 0, s>>>( lflag.get(), lscan.get(), n, tree.leaf_of.get(),
                                                           tree.leaf_start.get() );
        check_launch( "k_leaf_index" );
    }
    tree.n_leaves = nl;

    tree.s2.allocate( 2 * n, s );
    tree.f4.allocate( n, s );
    k_gather_sorted<<<blocks_for( n, 256 ), 256, 0, s>>>( src, tree.perm.get(), tree.scene.get(),
                                                            tree.s2.get(), tree.f4.get() );
    check_launch( "k_gather_sorted" );

    int64_t const ni = std::max<int64_t>( 0, nl - 1 );
    tree.nodes.allocate( 4 * std::max<int64_t>( 1, ni ), s );
    tree.root_box.allocate( 2, s );
    DeviceBuffer<int> left( std::max<int64_t>( 1, ni ), s ), right( std::max<int64_t>( 1, ni ), s ),
        parent_node( std::max<int64_t>( 1, ni ), s ), parent_leaf( nl, s ),
        range_lo( std::max<int64_t>( 1, ni ), s ), range_hi( std::max<int64_t>( 1, ni ), s );
    DeviceBuffer<unsigned> flags( std::max<int64_t>( 1, ni ), s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( flags.get(), 0, flags.n * sizeof( unsigned ), s ) );
    if ( ni > 0 )
    {
        k_karras<<<blocks_for( ni, 256 ), 256, 0, s>>>( tree.codes.get(), tree.grp.get(), tree.leaf_start.get(),
                                                          nl, left.get(),
                                                          right.get(), parent_node.get(), parent_leaf.get(),
                                                          range_lo.get(), range_hi.get() );
        check_launch( "k_karras" );
        k_pack_children<<<blocks_for( ni, 256 ), 256, 0, s>>>( ni, left.get(), right.get(), range_lo.get(),
                                                                 range_hi.get(), tree.nodes.get() );
        check_launch( "k_pack_children" );
    }
    k_refit<<<blocks_for( nl, 128 ), 128, 0, s>>>( tree.s2.get(),
                                                     tree.scene.get(), tree.leaf_start.get(), nl,
                                                     left.get(), right.get(), parent_node.get(),
                                                     parent_leaf.get(), tree.nodes.get(), flags.get(),
                                                     tree.root_box.get(), status );
    check_launch( "k_refit" );
    tree.n_wide = 0;
    if ( ni > 0 )
    {
        DeviceBuffer<int64_t> flag( ni, s ), widx( ni + 1, s );
        DeviceBuffer<unsigned> max_depth( 1, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( max_depth.get(), 0, sizeof( unsigned ), s ) );
        k_depth_flags<<<blocks_for( ni, 256 ), 256, 0, s>>>( ni, parent_node.get(), flag.get(), max_depth.get(),
                                                             status );
        check_launch( "k_depth_flags" );
        exclusive_scan_i64( flag.get(), widx.get(), ni, s );
        int64_t nw = 0;
        unsigned depth = 0;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &nw, widx.get() + ni, sizeof( int64_t ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &depth, max_depth.get(), sizeof( unsigned ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        tree.n_wide = nw;
        tree.wide_levels = (int)( depth / 3 );
        tree.wide.allocate( 16 * std::max<int64_t>( 1, nw ), s );
        tree.wide_range.allocate( 8 * std::max<int64_t>( 1, nw ), s );
        k_collapse<<<blocks_for( ni, 128 ), 128, 0, s>>>( ni, tree.nodes.get(), flag.get(), widx.get(),
                                                           tree.leaf_start.get(), tree.wide.get(),
                                                           tree.wide_range.get() );
        check_launch( "k_collapse" );
        tree.wide_cell.allocate( 2 * std::max<int64_t>( 1, nw ), s );
        k_wide_cells<<<blocks_for( ni, 256 ), 256, 0, s>>>( ni, n, flag.get(), widx.get(), parent_node.get(),
                                                              range_lo.get(), range_hi.get(), tree.leaf_start.get(),
                                                              tree.codes.get(), tree.scene.get(),
                                                              tree.wide_cell.get() );
        check_launch( "k_wide_cells" );
    }
    tree.nodes = DeviceBuffer<float4>(); // the queries use the wide nodes
}

void sort_queries( Lbvh const &tree, PointsView tgt, DeviceBuffer<uint32_t> &order,
                   cudaStream_t s, uint32_t const *group, int64_t n_groups, unsigned *status )
{
    int64_t const n = tgt.n;
    if ( order.n < (size_t)std::max<int64_t>( 1, n ) )
        order.allocate( std::max<int64_t>( 1, n ), s );
    if ( n == 0 )
        return;
    DeviceBuffer<uint32_t> codes( n, s );
    // the queries' order needs only the top 24 bits of their codes (a 256^3
    // grid): three radix passes instead of four
    k_morton<<<blocks_for( n, 256 ), 256, 0, s>>>( tgt, tree.scene.get(), codes.get(), order.get(), 6,
                                                     status );
    check_launch( "k_morton(targets)" );
    radix_sort_pairs( codes.get(), order.get(), n, 24, s );
    if ( group )
    {
        k_group_of<<<blocks_for( n, 256 ), 256, 0, s>>>( group, order.get(), n, codes.get() );
        check_launch( "k_group_of(targets)" );
        int bits = 1;
        while ( ( int64_t( 1 ) << bits ) < n_groups )
            ++bits;
        radix_sort_pairs( codes.get(), order.get(), n, ( bits + 7 ) / 8 * 8, s );
    }
}

void build_tree_and_order( PointsView src, PointsView tgt, Lbvh &tree, DeviceBuffer<uint32_t> &order,
                           unsigned *status, cudaStream_t s, uint32_t const *src_group,
                           uint32_t const *tgt_group, int64_t n_groups, cudaEvent_t tgt_ready )
{
    NvtxRange const nvtx_range( "DTK_build_tree" );
    struct Side
    {
        cudaStream_t s2 = nullptr;
        cudaEvent_t scene = nullptr, done = nullptr;
        ~Side()
        {
            if ( scene )
                cudaEventDestroy( scene );
            if ( done )
                cudaEventDestroy( done );
            if ( s2 )
                cudaStreamDestroy( s2 );
        }
    } side;
    DTK_CUDA_OR_THROW( cudaStreamCreateWithFlags( &side.s2, cudaStreamNonBlocking ) );
    DTK_CUDA_OR_THROW( cudaEventCreateWithFlags( &side.scene, cudaEventDisableTiming ) );
    DTK_CUDA_OR_THROW( cudaEventCreateWithFlags( &side.done, cudaEventDisableTiming ) );
    order.allocate( std::max<int64_t>( 1, tgt.n ), s ); // owned by s, filled on the side stream
    build_lbvh( src, tree, status, s, src_group, n_groups, [&] {
        DTK_CUDA_OR_THROW( cudaEventRecord( side.scene, s ) );
        DTK_CUDA_OR_THROW( cudaStreamWaitEvent( side.s2, side.scene, 0 ) );
        if ( tgt_ready )
            DTK_CUDA_OR_THROW( cudaStreamWaitEvent( side.s2, tgt_ready, 0 ) );
        sort_queries( tree, tgt, order, side.s2, tgt_group, n_groups, status );
        DTK_CUDA_OR_THROW( cudaEventRecord( side.done, side.s2 ) );
    } );
    DTK_CUDA_OR_THROW( cudaStreamWaitEvent( s, side.done, 0 ) );
    // Points with a NaN or infinite coordinate were flagged by the passes
    // that read them (scene bounds, target Morton codes), whose results stay
    // in range either way; no search runs on them.
    unsigned st = 0;
    DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status, sizeof( st ), cudaMemcpyDeviceToHost, s ) );
    DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
    if ( st & DEV_NONFINITE_SOURCE )
        throw Error{DTK_ERR_INVALID_ARG, "DTK_REQUIRE: source point coordinates must be finite"};
    if ( st & DEV_NONFINITE_TARGET )
        throw Error{DTK_ERR_INVALID_ARG, "DTK_REQUIRE: target point coordinates must be finite"};
}

void knn_query( Lbvh const &tree, PointsView tgt, uint32_t const *order, int k,
                GroupArgs const &groups, int32_t const *offset, int32_t *idx, unsigned *status,
                cudaStream_t s, int32_t *pos )
{
    NvtxRange const nvtx_range( "DTK_knn_query" );
    if ( tgt.n == 0 || tree.n == 0 || ( k == 0 && !groups.k ) )
        return;
    GroupView const gv{groups.src_off, groups.tgt_grp, groups.k, groups.r};
    // chunk length: up to Q_SEQ queries, fewer when that leaves under four
    // chunks per resident warp; the last chunk per resident warp is cut in
    // two halves
    int seq = Q_SEQ;
    int64_t const resident = (int64_t)num_sms() * KNN_BLOCKS_PER_SM * Q_WARPS;
    while ( seq > 1 && ( tgt.n + seq - 1 ) / seq < 4 * resident )
        seq /= 2;
    int64_t const tail_q = resident * seq;
    int64_t const n_big = tgt.n > tail_q ? ( tgt.n - tail_q ) / seq : 0;
    int const tail = seq > 1 ? seq / 2 : 1;
    int64_t const n_chunks = n_big + ( tgt.n - n_big * seq + tail - 1 ) / tail;
    int64_t const warps = n_chunks < resident ? n_chunks : resident;
    unsigned const blocks = blocks_for( warps, Q_WARPS );
    DeviceBuffer<unsigned> next( 1, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( next.get(), 0, sizeof( unsigned ), s ) );
    KnnChunks const ch{seq, n_big, next.get()};
    DeviceBuffer<Query> qrec( tgt.n, s );
    k_query_frame<<<blocks_for( tgt.n, 256 ), 256, 0, s>>>( tgt, order, tree.scene.get(), qrec.get() );
    check_launch( "k_query_frame" );
    if ( groups.tgt_grp )
        k_knn<true><<<blocks, Q_WARPS * 32, 0, s>>>( view_of( tree ), tgt, order, qrec.get(), k, ch, gv,
                                                     offset, idx, pos, status );
    else
        k_knn<false><<<blocks, Q_WARPS * 32, 0, s>>>( view_of( tree ), tgt, order, qrec.get(), k, ch, gv,
                                                      offset, idx, pos, status );
    check_launch( "k_knn" );
}

void radius_count( Lbvh const &tree, PointsView tgt, uint32_t const *order, double r,
                   GroupArgs const &groups, int64_t *counts, unsigned *status, cudaStream_t s )
{
    NvtxRange const nvtx_range( "DTK_radius_query" );
    if ( tgt.n == 0 )
        return;
    GroupView const gv{groups.src_off, groups.tgt_grp, groups.k, groups.r};
    if ( groups.tgt_grp )
        k_radius<false, true><<<blocks_for( tgt.n, R_WARPS ), R_WARPS * 32, 0, s>>>(
            view_of( tree ), tgt, order, r, gv, counts, nullptr, nullptr, status );
    else
        k_radius<false, false><<<blocks_for( tgt.n, R_WARPS ), R_WARPS * 32, 0, s>>>(
            view_of( tree ), tgt, order, r, gv, counts, nullptr, nullptr, status );
    check_launch( "k_radius(count)" );
}

void radius_fill( Lbvh const &tree, PointsView tgt, uint32_t const *order, double r,
                  GroupArgs const &groups, int32_t const *offset, int32_t *idx, unsigned *status,
                  cudaStream_t s )
{
    NvtxRange const nvtx_range( "DTK_radius_query" );
    if ( tgt.n == 0 )
        return;
    GroupView const gv{groups.src_off, groups.tgt_grp, groups.k, groups.r};
    if ( groups.tgt_grp )
        k_radius<true, true><<<blocks_for( tgt.n, R_WARPS ), R_WARPS * 32, 0, s>>>(
            view_of( tree ), tgt, order, r, gv, nullptr, offset, idx, status );
    else
        k_radius<true, false><<<blocks_for( tgt.n, R_WARPS ), R_WARPS * 32, 0, s>>>(
            view_of( tree ), tgt, order, r, gv, nullptr, offset, idx, status );
    check_launch( "k_radius(fill)" );
}

} // namespace dtk
