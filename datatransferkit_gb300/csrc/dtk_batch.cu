// Batched uneven MLS transfers (extension; the reference builds one operator
// per problem) and the setup planner shared with the single operator.
//
// All problems share one LBVH over their packed sources, built in
// problem-major Morton order: problem p's sources occupy one contiguous range
// of sorted positions, every tree node records the leaf range it covers, and
// a query only enters nodes and points of its own problem.  Targets are
// processed in problem-major Morton order.  The setup is planned on the
// device: a stable key sort splits the processing order into buckets of
// (basis, rbf, path), and a layout kernel cuts the buckets into tasks of 32
// targets (longest rows first).  One persistent launch runs every task: a
// warp gathers its targets' rows with G lanes a target (1 for kNN rows, the
// single operator's arithmetic; for radius rows, 0 to thousands of entries,
// G is tuned by timing candidates on a sample of the tasks at create), then
// runs the reference Jacobi one target a lane.  Mixed-form kNN rows run the
// fused mixed kernel per bucket instead.  The plan is kept: a re-setup on
// new coordinates with the same rows is the persistent launch alone,
// captured into a CUDA graph and replayed.
//
// Apply is one persistent launch over a schedule of warp tasks.  Rows are
// binned by length (bin b holds rows of at most 2^b entries); a task is up to
// 32/S rows of one bin that a warp reduces with S lanes per row.  S per bin
// comes from an autotuner that times the candidates on the actual data on
// the first apply; the schedule is then fixed (longest bins first, so that
// the slow tasks start early) and its launch can be captured into a CUDA
// graph and replayed.
#include "dtk_common.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

namespace dtk
{

namespace
{

constexpr int N_BASIS = 3, N_RBF = SETUP_RBFS, N_PATH = SETUP_PATHS;
constexpr int N_KEYS = SETUP_KEYS;
static_assert( N_KEYS == N_BASIS * N_RBF * N_PATH, "bucket keys" );

// Bucket key of every target in processing order, the targets themselves as
// sort values, and a histogram of the keys.
__global__ void k_plan_keys( int64_t n, uint32_t const *order, int32_t const *offset,
                             uint32_t const *tgt_grp, uint8_t const *basis_g, uint8_t const *rbf_g,
                             int basis, int rbf, bool split_all, uint32_t *keys, uint32_t *vals,
                             unsigned *hist )
{
    __shared__ unsigned h[N_KEYS];
    for ( int k = threadIdx.x; k < N_KEYS; k += blockDim.x )
        h[k] = 0;
    __syncthreads();
    int64_t const g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( g < n )
    {
        uint32_t const i = order[g];
        int const len = offset[i + 1] - offset[i];
        uint32_t const grp = tgt_grp ? tgt_grp[i] : 0u;
        int const b = basis_g ? basis_g[grp] : basis;
        int const r = rbf_g ? rbf_g[grp] : rbf;
        int const path = split_all ? ( len > 32 ? 2 : 1 ) : ( len > FUSED_MAX_ROW ? 2 : 0 );
        uint32_t const key = (uint32_t)( ( b * N_RBF + r ) * N_PATH + path );
        keys[g] = key;
        vals[g] = i;
        atomicAdd( &h[key], 1u );
    }
    __syncthreads();
    for ( int k = threadIdx.x; k < N_KEYS; k += blockDim.x )
        if ( h[k] )
            atomicAdd( &hist[k], h[k] );
}

// Task layout from the bucket histogram (one block): buckets of path 2 (the
// longest rows) first, then path 1, then path 0 (path 0 left out when
// `with_path0` is false), each bucket cut into tasks of 32 targets.  Writes
// the task count, the first task of each path and, per bucket, its first
// target in the bucketed list and its first task.
__global__ void k_task_layout( unsigned const *hist, bool with_path0, int64_t *n_tasks, int64_t *path_first,
                               int64_t *bucket_start, int64_t *bucket_task )
{
    if ( threadIdx.x != 0 )
        return;
    int64_t at = 0;
    for ( int k = 0; k < N_KEYS; ++k )
    {
        bucket_start[k] = at;
        at += hist[k];
    }
    int64_t t = 0;
    for ( int path = N_PATH - 1; path >= 0; --path )
    {
        path_first[path] = t;
        for ( int k = path; k < N_KEYS; k += N_PATH )
        {
            bucket_task[k] = t;
            if ( path > 0 || with_path0 )
                t += ( hist[k] + 31 ) / 32;
        }
    }
    path_first[N_PATH] = t;
    *n_tasks = t;
}

// The tasks (a grid over the largest possible count; the excess exits).
__global__ void k_fill_tasks( unsigned const *hist, int64_t const *n_tasks, int64_t const *bucket_start,
                              int64_t const *bucket_task, bool with_path0, int lanes0, int lanes1, int lanes2,
                              SetupTask *tasks )
{
    int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( t >= *n_tasks )
        return;
    // the bucket whose task range holds t (non-empty buckets are disjoint)
    int key = -1;
    for ( int k = 0; k < N_KEYS; ++k )
    {
        int const path = k % N_PATH;
        if ( hist[k] == 0 || ( path == 0 && !with_path0 ) )
            continue;
        int64_t const n_t = ( hist[k] + 31 ) / 32;
        if ( t >= bucket_task[k] && t < bucket_task[k] + n_t )
            key = k;
    }
    if ( key < 0 )
        return;
    int64_t const j = t - bucket_task[key];
    int const path = key % N_PATH;
    SetupTask x;
    x.first = (int32_t)( bucket_start[key] + 32 * j );
    int64_t const left = (int64_t)hist[key] - 32 * j;
    x.count = (uint8_t)( left < 32 ? left : 32 );
    x.key = (uint8_t)key;
    x.lanes = (uint8_t)( path == 2 ? lanes2 : path == 1 ? lanes1 : lanes0 );
    x.pad = 0;
    tasks[t] = x;
}

// Setup tuning: lanes a target for the gather phases of each path.  Path 0
// (kNN rows) keeps one lane a target, the arithmetic of the single
// operator's kernel; paths 1 and 2 are timed on a sample of their tasks.
std::mutex g_setup_tune_mutex;
std::map<std::tuple<int, int, int>, int> g_setup_tune_cache; // (path, precision, log2 tasks) -> lanes

} // namespace

SetupPlan::~SetupPlan() = default;

void plan_setup( SetupArgs const &a, int precision, uint8_t const *basis_of_group, uint8_t const *rbf_of_group,
                 uint32_t const *tgt_group, bool split_all, SetupPlan &plan, cudaStream_t s )
{
    int64_t const n = a.n_tgt;
    plan.n = n;
    plan.precision = precision;
    // mixed kNN rows (path 0 of the mixed form) run the fused mixed kernel
    // per bucket, the rest the persistent FP64 kernel
    plan.with_path0 = !( precision == DTK_MIXED && !split_all );
    plan.list.allocate( std::max<int64_t>( 1, n ), s );
    plan.hist.allocate( N_KEYS, s );
    plan.n_tasks.allocate( 1, s );
    plan.path_first.allocate( N_PATH + 1, s );
    plan.bucket_start.allocate( N_KEYS, s );
    plan.bucket_task.allocate( N_KEYS, s );
    plan.tasks.allocate( ( n + 31 ) / 32 + N_KEYS, s );
    plan.counter.allocate( 1, s );
    DTK_CUDA_OR_THROW( cudaMemsetAsync( plan.hist.get(), 0, N_KEYS * sizeof( unsigned ), s ) );
    if ( n )
    {
        DeviceBuffer<uint32_t> keys( n, s );
        k_plan_keys<<<(unsigned)( ( n + 255 ) / 256 ), 256, 0, s>>>( n, a.order, a.offset, tgt_group,
                                                                      basis_of_group, rbf_of_group, a.basis,
                                                                      a.rbf, split_all, keys.get(),
                                                                      plan.list.get(), plan.hist.get() );
        check_launch( "k_plan_keys" );
        // stable: each bucket keeps the processing order
        radix_sort_pairs( keys.get(), plan.list.get(), n, 8, s );
    }
    k_task_layout<<<1, 32, 0, s>>>( plan.hist.get(), plan.with_path0, plan.n_tasks.get(), plan.path_first.get(),
                                    plan.bucket_start.get(), plan.bucket_task.get() );
    check_launch( "k_task_layout" );
}

void fill_setup_tasks( SetupPlan &plan, cudaStream_t s )
{
    int64_t const most = ( plan.n + 31 ) / 32 + N_KEYS;
    k_fill_tasks<<<(unsigned)( ( most + 255 ) / 256 ), 256, 0, s>>>(
        plan.hist.get(), plan.n_tasks.get(), plan.bucket_start.get(), plan.bucket_task.get(), plan.with_path0,
        plan.lanes[0], plan.lanes[1], plan.lanes[2], plan.tasks.get() );
    check_launch( "k_fill_tasks" );
}

namespace
{

BatchSetupArgs batch_args( SetupArgs const &a, SetupPlan &plan, double *u_work )
{
    BatchSetupArgs b;
    b.nb = Neighbours{a.src, a.idx, a.pos, a.s2};
    b.tgt = a.tgt;
    b.offset = a.offset;
    b.list = plan.list.get();
    b.n_list = plan.n;
    b.tasks = plan.tasks.get();
    b.n_tasks = plan.n_tasks.get();
    b.rows_sorted = a.rows_sorted;
    b.coeff64 = a.coeff64;
    b.coeff32 = a.coeff32;
    b.underdetermined = a.underdetermined;
    b.rotations = a.rotations;
    b.status = a.status;
    b.counter = plan.counter.get();
    b.u_work = u_work;
    return b;
}

// Times the lane counts of paths 1 and 2 on a sample of their tasks (the
// first wave of each: one task a resident warp; the faster of two runs per
// candidate), keeps the fastest per path, and caches it by (path,
// precision, size class).  One synchronisation reads the task layout.
void tune_setup( SetupArgs const &a, SetupPlan &plan, double *u_work, cudaStream_t s )
{
    int fixed[N_PATH] = {0, 0, 0};
    fixed_setup_lanes( fixed[1], fixed[2] );
    if ( fixed[1] && fixed[2] )
    {
        plan.lanes[1] = fixed[1];
        plan.lanes[2] = fixed[2];
        return;
    }
    int64_t pf[N_PATH + 1];
    DTK_CUDA_OR_THROW( cudaMemcpyAsync( pf, plan.path_first.get(), sizeof( pf ), cudaMemcpyDeviceToHost, s ) );
    DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
    int64_t const wave = batch_setup_threads() / 32; // resident warps
    cudaEvent_t e0, e1;
    DTK_CUDA_OR_THROW( cudaEventCreate( &e0 ) );
    DTK_CUDA_OR_THROW( cudaEventCreate( &e1 ) );
    struct EvGuard
    {
        cudaEvent_t a, b;
        ~EvGuard()
        {
            cudaEventDestroy( a );
            cudaEventDestroy( b );
        }
    } guard{e0, e1};
    for ( int path = 1; path < N_PATH; ++path )
    {
        // tasks of this path: [pf[path], next path's first) (paths run 2, 1, 0)
        if ( fixed[path] )
        {
            plan.lanes[path] = fixed[path];
            continue;
        }
        int64_t const t0 = pf[path], t1 = path == 2 ? pf[1] : pf[0];
        int64_t const count = t1 - t0;
        if ( count <= 0 )
            continue;
        int size_class = 0;
        while ( ( int64_t( 1 ) << size_class ) < count )
            ++size_class;
        auto const key = std::make_tuple( path, plan.precision, size_class );
        {
            std::lock_guard<std::mutex> lock( g_setup_tune_mutex );
            auto const it = g_setup_tune_cache.find( key );
            if ( it != g_setup_tune_cache.end() )
            {
                plan.lanes[path] = it->second;
                plan.tuned[path] = true;
                continue;
            }
        }
        int64_t const sample = std::min<int64_t>( count, wave ); // one task a resident warp
        int const cands[2][3] = {{2, 4, 8}, {8, 16, 32}};
        float best = 3.4e38f;
        int best_lanes = plan.lanes[path];
        for ( int G : cands[path - 1] )
        {
            BatchSetupArgs b = batch_args( a, plan, u_work );
            b.t_begin = t0;
            b.t_end = t0 + sample;
            b.force_lanes = G;
            float ms[2];
            for ( int rep = 0; rep < 2; ++rep )
            {
                DTK_CUDA_OR_THROW( cudaEventRecord( e0, s ) );
                batch_setup( b, s );
                DTK_CUDA_OR_THROW( cudaEventRecord( e1, s ) );
                DTK_CUDA_OR_THROW( cudaEventSynchronize( e1 ) );
                DTK_CUDA_OR_THROW( cudaEventElapsedTime( &ms[rep], e0, e1 ) );
            }
            float const t = std::min( ms[0], ms[1] );
            if ( t < best )
            {
                best = t;
                best_lanes = G;
            }
        }
        plan.lanes[path] = best_lanes;
        plan.tuned[path] = true;
        std::lock_guard<std::mutex> lock( g_setup_tune_mutex );
        g_setup_tune_cache[key] = best_lanes;
    }
}

} // namespace

void run_setup_plan( SetupArgs const &a, int precision, uint8_t const *basis_of_group,
                     uint8_t const *rbf_of_group, uint32_t const *tgt_group, bool split_all,
                     cudaStream_t s, SetupPlan *keep, bool tune )
{
    SetupPlan local;
    SetupPlan &plan = keep ? *keep : local;
    plan_setup( a, precision, basis_of_group, rbf_of_group, tgt_group, split_all, plan, s );
    if ( a.n_tgt == 0 )
        return;
    if ( !plan.u_work.get() )
        plan.u_work.allocate( (size_t)jacobi_work_doubles( BS_MAX_M ) * batch_setup_threads(), s );
    // the tasks exist before any launch reads them (the tuner's samples
    // too); refilled with the tuned lane counts.  The statistics counters
    // collect the sample runs as well: zeroed after them
    fill_setup_tasks( plan, s );
    if ( tune )
    {
        tune_setup( a, plan, plan.u_work.get(), s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( a.underdetermined, 0, sizeof( unsigned long long ), s ) );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( a.rotations, 0, sizeof( unsigned long long ), s ) );
        fill_setup_tasks( plan, s );
    }
    run_planned_setup( a, plan, s );
}

void run_planned_setup( SetupArgs const &a, SetupPlan &plan, cudaStream_t s )
{
    if ( plan.n == 0 )
        return;
    BatchSetupArgs const b = batch_args( a, plan, plan.u_work.get() );
    batch_setup( b, s );
    if ( plan.with_path0 )
        return;
    // mixed-form kNN rows: the fused mixed kernel per (basis, rbf) bucket;
    // the bucket sizes come to the host once and are kept
    if ( plan.mixed_buckets.empty() )
    {
        unsigned h[N_KEYS];
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( h, plan.hist.get(), sizeof( h ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        int64_t start = 0;
        for ( int key = 0; key < N_KEYS; ++key )
        {
            if ( h[key] && key % N_PATH == 0 )
                plan.mixed_buckets.push_back( {key, start, (int64_t)h[key]} );
            start += h[key];
        }
        if ( plan.mixed_buckets.empty() )
            plan.mixed_buckets.push_back( {-1, 0, 0} ); // none: do not ask again
    }
    for ( auto const &bk : plan.mixed_buckets )
    {
        if ( bk.key < 0 )
            continue;
        SetupArgs b = a;
        b.basis = bk.key / N_PATH / N_RBF;
        b.rbf = bk.key / N_PATH % N_RBF;
        b.n_tgt = bk.count;
        b.order = plan.list.get() + bk.start;
        setup_mixed( b, s );
    }
}

namespace
{

__global__ void k_group_ids( int64_t const *off, int n_groups, int64_t n, uint32_t *out )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    int lo = 0, hi = n_groups; // largest g with off[g] <= i
    while ( hi - lo > 1 )
    {
        int const mid = ( lo + hi ) / 2;
        if ( off[mid] <= i )
            lo = mid;
        else
            hi = mid;
    }
    out[i] = (uint32_t)lo;
}

__global__ void k_narrow32( int64_t const *in, int32_t *out, int64_t n )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i <= n )
        out[i] = (int32_t)in[i];
}

// kNN row length of every target: min(k of its problem, sources of its problem)
__global__ void k_knn_rows( int64_t n, uint32_t const *tgt_grp, int64_t const *src_off, int32_t const *k,
                            int64_t *counts )
{
    int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    uint32_t const g = tgt_grp[i];
    int64_t const ns = src_off[g + 1] - src_off[g];
    counts[i] = k[g] < ns ? k[g] : ns;
}

// Apply bin of every target in processing order (bin b: rows of at most 2^b
// entries), the targets as sort values, and a histogram of the bins.
__global__ void k_bin_keys( int64_t n, uint32_t const *order, int32_t const *offset, uint32_t *keys,
                            uint32_t *vals, unsigned *hist )
{
    __shared__ unsigned h[32];
    if ( threadIdx.x < 32 )
        h[threadIdx.x] = 0;
    __syncthreads();
    int64_t const g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if ( g < n )
    {
        uint32_t const i = order[g];
        int const len = offset[i + 1] - offset[i];
        int const b = len <= 1 ? 0 : 32 - __clz( len - 1 );
        keys[g] = (uint32_t)b;
        vals[g] = i;
        atomicAdd( &h[b], 1u );
    }
    __syncthreads();
    if ( threadIdx.x < 32 && h[threadIdx.x] )
        atomicAdd( &hist[threadIdx.x], h[threadIdx.x] );
}

constexpr unsigned FULL = 0xffffffffu;
constexpr int APPLY_THREADS = 256;

// Task: x = first entry of its rows in the schedule's row list, y = lanes per
// row S (low 6 bits, a power of two) | number of rows (<= 32 / S) << 6.
template <bool F32>
__global__ void __launch_bounds__( APPLY_THREADS )
    k_apply_sched( int64_t n_tasks, int2 const *__restrict__ tasks, int32_t const *__restrict__ rows,
                   int32_t const *__restrict__ offset, int32_t const *__restrict__ idx,
                   void const *__restrict__ coeff, double const *__restrict__ values,
                   double *__restrict__ target )
{
    int const lane = threadIdx.x & 31;
    int64_t const warps = (int64_t)gridDim.x * ( APPLY_THREADS / 32 );
    for ( int64_t t = ( blockIdx.x * (int64_t)APPLY_THREADS + threadIdx.x ) >> 5; t < n_tasks; t += warps )
    {
        int2 const task = __ldg( tasks + t );
        int const S = task.y & 63, cnt = task.y >> 6;
        int const shift = __ffs( S ) - 1;
        int const r = lane >> shift, sub = lane & ( S - 1 );
        double acc = 0.0;
        int64_t row = -1;
        if ( r < cnt )
        {
            row = __ldg( rows + task.x + r );
            int const b = __ldg( offset + row ), e = __ldg( offset + row + 1 );
            for ( int j = b + sub; j < e; j += S )
            {
                double const c = F32 ? (double)__ldg( static_cast<float const *>( coeff ) + j )
                                     : __ldg( static_cast<double const *>( coeff ) + j );
                acc = fma( c, __ldg( values + __ldg( idx + j ) ), acc );
            }
        }
        for ( int o = S >> 1; o > 0; o >>= 1 ) // S is warp-uniform
            acc += __shfl_xor_sync( FULL, acc, o );
        if ( r < cnt && sub == 0 )
            target[row] = acc;
    }
}

inline int bin_of64( int64_t n )
{
    int b = 0;
    while ( ( int64_t( 1 ) << b ) < n )
        ++b;
    return b;
}

} // namespace
} // namespace dtk

using namespace dtk;

struct dtk_mls_batch_s
{
    HandleLife life;
    explicit dtk_mls_batch_s( cudaStream_t home )
        : life( home )
    {
    }
    int32_t n_problems = 0;
    int precision = DTK_FP64;
    int64_t n_src = 0, n_tgt = 0, nnz = 0;
    DeviceBuffer<int32_t> offset, idx;
    DeviceBuffer<double> coeff64;
    DeviceBuffer<float> coeff32;
    // row bins: rows of bin b (at most 2^b entries) at [bin_start[b], bin_start[b+1]) of `rows`
    static constexpr int NBINS = 32;
    std::vector<int64_t> bin_start;
    int lanes[NBINS] = {};
    DeviceBuffer<int32_t> rows;
    DeviceBuffer<int2> tasks;
    int64_t n_tasks = 0;
    bool tuned = false;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double const *g_src = nullptr;
    double *g_tgt = nullptr;
    int64_t underdetermined = 0, rotations = 0;
    float search_ms = 0.f, setup_ms = 0.f, host_ms = 0.f;
    // the setup's plan (bucketed targets, tasks, lane counts), kept for
    // re-setups on new coordinates with the same rows, and their graph
    SetupPlan plan;
    bool radius_mode = false;
    DeviceBuffer<unsigned> status;
    DeviceBuffer<unsigned long long> counters;
    cudaGraph_t setup_graph = nullptr;
    cudaGraphExec_t setup_exec = nullptr;
    double const *gs_src = nullptr, *gs_tgt = nullptr;
    int64_t setup_replays = 0;

    ~dtk_mls_batch_s()
    {
        life.retire( offset, idx, coeff64, coeff32, rows, tasks, status, counters, plan.list, plan.hist,
                     plan.n_tasks, plan.path_first, plan.bucket_start, plan.bucket_task, plan.tasks, plan.counter,
                     plan.u_work );
        if ( exec )
            cudaGraphExecDestroy( exec );
        if ( graph )
            cudaGraphDestroy( graph );
        if ( setup_exec )
            cudaGraphExecDestroy( setup_exec );
        if ( setup_graph )
            cudaGraphDestroy( setup_graph );
        if ( capture )
            cudaStreamDestroy( capture );
    }

    // schedule over the bins in `which` (longest first) with the given lanes
    std::vector<int2> schedule( std::vector<int> const &which, int const *lanes_of ) const
    {
        std::vector<int2> t;
        for ( int b : which )
        {
            int const S = lanes_of[b], per = 32 / S;
            for ( int64_t r = bin_start[b]; r < bin_start[b + 1]; r += per )
            {
                int const cnt = (int)std::min<int64_t>( per, bin_start[b + 1] - r );
                t.push_back( make_int2( (int)r, S | ( cnt << 6 ) ) );
            }
        }
        return t;
    }

    void launch( int2 const *t, int64_t n, double const *src_values, double *tgt_values, cudaStream_t s ) const
    {
        if ( n == 0 )
            return;
        int64_t const want = ( n * 32 + APPLY_THREADS - 1 ) / APPLY_THREADS;
        unsigned const blocks = (unsigned)std::max<int64_t>( 1, std::min<int64_t>( want, 8 * num_sms() ) );
        if ( coeff32.get() )
            k_apply_sched<true><<<blocks, APPLY_THREADS, 0, s>>>( n, t, rows.get(), offset.get(), idx.get(),
                                                                  coeff32.get(), src_values, tgt_values );
        else
            k_apply_sched<false><<<blocks, APPLY_THREADS, 0, s>>>( n, t, rows.get(), offset.get(), idx.get(),
                                                                   coeff64.get(), src_values, tgt_values );
        check_launch( "k_apply_sched" );
    }

    // Time each candidate lanes-per-row on each bin (median of 3 after one
    // warm-up), then upload the schedule of the winners.  Winners are kept
    // per process by (bin, coefficient type, order of magnitude of the bin's
    // row count), so later batches of a similar shape skip the timing.
    void tune( double const *src_values, double *tgt_values, cudaStream_t s )
    {
        static std::mutex cache_mutex;
        static std::map<std::tuple<int, bool, int>, int> cache;
        bool const f32 = coeff32.get() != nullptr;
        cudaEvent_t e0, e1;
        DTK_CUDA_OR_THROW( cudaEventCreate( &e0 ) );
        DTK_CUDA_OR_THROW( cudaEventCreate( &e1 ) );
        struct EvGuard
        {
            cudaEvent_t a, b;
            ~EvGuard()
            {
                cudaEventDestroy( a );
                cudaEventDestroy( b );
            }
        } guard{e0, e1};
        for ( int b = 0; b < NBINS; ++b )
        {
            if ( bin_start[b + 1] == bin_start[b] )
                continue;
            auto const key = std::make_tuple( b, f32, bin_of64( bin_start[b + 1] - bin_start[b] ) );
            {
                std::lock_guard<std::mutex> lock( cache_mutex );
                auto const it = cache.find( key );
                if ( it != cache.end() )
                {
                    lanes[b] = it->second;
                    continue;
                }
            }
            float best = 3.4e38f;
            int best_lanes = 1;
            for ( int S = 1; S <= 32; S <<= 1 )
            {
                if ( S > 1 && ( S >> 1 ) >= ( 1 << b ) )
                    break; // more lanes than entries
                int cand[NBINS];
                std::fill( cand, cand + NBINS, S );
                std::vector<int2> const t = schedule( {b}, cand );
                DeviceBuffer<int2> d( t.size(), s );
                DTK_CUDA_OR_THROW( cudaMemcpyAsync( d.get(), t.data(), t.size() * sizeof( int2 ),
                                                    cudaMemcpyHostToDevice, s ) );
                float ms[4];
                for ( int rep = 0; rep < 4; ++rep )
                {
                    DTK_CUDA_OR_THROW( cudaEventRecord( e0, s ) );
                    launch( d.get(), (int64_t)t.size(), src_values, tgt_values, s );
                    DTK_CUDA_OR_THROW( cudaEventRecord( e1, s ) );
                    DTK_CUDA_OR_THROW( cudaEventSynchronize( e1 ) );
                    DTK_CUDA_OR_THROW( cudaEventElapsedTime( &ms[rep], e0, e1 ) );
                }
                std::sort( ms + 1, ms + 4 );
                if ( ms[2] < best )
                {
                    best = ms[2];
                    best_lanes = S;
                }
            }
            lanes[b] = best_lanes;
            std::lock_guard<std::mutex> lock( cache_mutex );
            cache[key] = best_lanes;
        }
        std::vector<int> order;
        for ( int b = NBINS - 1; b >= 0; --b )
            if ( bin_start[b + 1] > bin_start[b] )
                order.push_back( b );
        std::vector<int2> const t = schedule( order, lanes );
        n_tasks = (int64_t)t.size();
        tasks.allocate( std::max<int64_t>( 1, n_tasks ), s );
        if ( n_tasks )
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( tasks.get(), t.data(), t.size() * sizeof( int2 ),
                                                cudaMemcpyHostToDevice, s ) );
        tuned = true;
    }
};

namespace
{

double ms_since( std::chrono::steady_clock::time_point t0 )
{
    return std::chrono::duration<double, std::milli>( std::chrono::steady_clock::now() - t0 ).count();
}

} // namespace

extern "C" {

dtk_status dtk_mls_batch_create( int32_t n_problems, const dtk_mls_options *opts,
                                 const int64_t *src_offsets, const double *src,
                                 const int64_t *tgt_offsets, const double *tgt,
                                 dtk_stream_t stream_, dtk_mls_batch_handle *out )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr, "output handle pointer is null" );
        *out = nullptr;
        DTK_REQUIRE_OR_THROW( n_problems >= 1, "n_problems must be >= 1" );
        DTK_REQUIRE_OR_THROW( opts && src_offsets && tgt_offsets, "null host array" );
        DTK_REQUIRE_OR_THROW( src_offsets[0] == 0 && tgt_offsets[0] == 0, "offsets must start at 0" );
        bool const radius_mode = opts[0].radius > 0.0;
        int const precision = opts[0].precision;
        DTK_REQUIRE_OR_THROW( precision == DTK_FP64 || precision == DTK_MIXED, "unknown precision" );
        std::vector<int32_t> kq( n_problems );
        std::vector<double> rq( n_problems );
        for ( int p = 0; p < n_problems; ++p )
        {
            dtk_mls_options const &o = opts[p];
            std::string const pre = "problem " + std::to_string( p ) + ": ";
            if ( o.comm_size > 1 )
                throw Error{DTK_ERR_UNSUPPORTED, pre + "only single-rank operators"};
            DTK_REQUIRE_OR_THROW( o.rbf >= DTK_WENDLAND0 && o.rbf <= DTK_BUHMANN4, pre + "unknown rbf" );
            DTK_REQUIRE_OR_THROW( o.basis >= DTK_CONSTANT3 && o.basis <= DTK_QUADRATIC3, pre + "unknown basis" );
            DTK_REQUIRE_OR_THROW( o.precision == precision, pre + "all problems of a batch share one precision form" );
            DTK_REQUIRE_OR_THROW( ( o.radius > 0.0 ) == radius_mode,
                                  pre + "all problems of a batch use kNN, or all use a radius search" );
            DTK_REQUIRE_OR_THROW( std::isfinite( o.radius ) && o.radius >= 0.0, pre + "bad radius" );
            DTK_REQUIRE_OR_THROW( o.k >= 0, pre + "k is negative" );
            kq[p] = o.k ? o.k : basis_size( o.basis );
            if ( !radius_mode && kq[p] > 32 )
                throw Error{DTK_ERR_UNSUPPORTED, pre + "kNN search supports k <= 32"};
            rq[p] = o.radius;
            // DTK_CHECK( !search_tree.empty() ) for every problem
            DTK_REQUIRE_OR_THROW( src_offsets[p + 1] > src_offsets[p], pre + "no source points" );
            DTK_REQUIRE_OR_THROW( tgt_offsets[p + 1] >= tgt_offsets[p], pre + "target offsets decrease" );
        }
        int64_t const n_src = src_offsets[n_problems], n_tgt = tgt_offsets[n_problems];
        DTK_REQUIRE_OR_THROW( n_src <= INT32_MAX && n_tgt < INT32_MAX, "too many points" );
        DTK_REQUIRE_OR_THROW( src != nullptr && ( n_tgt == 0 || tgt != nullptr ), "null points" );
        require_device_memory( src, "source points" );
        require_device_memory( n_tgt ? tgt : nullptr, "target points" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        auto h = std::make_unique<dtk_mls_batch_s>( s );
        TouchOnExit const touch{&h->life, s};
        h->n_problems = n_problems;
        h->precision = precision;
        h->n_src = n_src;
        h->n_tgt = n_tgt;
        PointsView const sv{src, n_src, 3, 1};
        PointsView const tv{tgt, n_tgt, 3, 1};
        double host_ms = 0.0;

        cudaEvent_t ev[3];
        for ( auto &e : ev )
            DTK_CUDA_OR_THROW( cudaEventCreate( &e ) );
        struct EvGuard
        {
            cudaEvent_t *e;
            ~EvGuard()
            {
                for ( int i = 0; i < 3; ++i )
                    cudaEventDestroy( e[i] );
            }
        } evg{ev};
        DeviceBuffer<unsigned> status( 1, s );
        DeviceBuffer<unsigned long long> counters( 3, s );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( status.get(), 0, sizeof( unsigned ), s ) );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( counters.get(), 0, 3 * sizeof( unsigned long long ), s ) );
        DTK_CUDA_OR_THROW( cudaEventRecord( ev[0], s ) );
        DeviceBuffer<int64_t> d_src_off( n_problems + 1, s ), d_tgt_off( n_problems + 1, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_src_off.get(), src_offsets, ( n_problems + 1 ) * 8,
                                            cudaMemcpyHostToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_tgt_off.get(), tgt_offsets, ( n_problems + 1 ) * 8,
                                            cudaMemcpyHostToDevice, s ) );
        DeviceBuffer<uint32_t> src_grp( n_src, s ), tgt_grp( std::max<int64_t>( 1, n_tgt ), s );
        k_group_ids<<<(unsigned)( ( n_src + 255 ) / 256 ), 256, 0, s>>>( d_src_off.get(), n_problems, n_src,
                                                                         src_grp.get() );
        check_launch( "k_group_ids(src)" );
        if ( n_tgt )
        {
            k_group_ids<<<(unsigned)( ( n_tgt + 255 ) / 256 ), 256, 0, s>>>( d_tgt_off.get(), n_problems,
                                                                             n_tgt, tgt_grp.get() );
            check_launch( "k_group_ids(tgt)" );
        }
        DeviceBuffer<int32_t> d_k( n_problems, s );
        DeviceBuffer<double> d_r( n_problems, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_k.get(), kq.data(), n_problems * 4, cudaMemcpyHostToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( d_r.get(), rq.data(), n_problems * 8, cudaMemcpyHostToDevice, s ) );

        // --- search over all problems at once ---
        Lbvh tree;
        DeviceBuffer<uint32_t> order;
        build_tree_and_order( sv, tv, tree, order, status.get(), s, src_grp.get(), tgt_grp.get(), n_problems );
        GroupArgs ga;
        ga.src_off = d_src_off.get();
        ga.tgt_grp = tgt_grp.get();
        ga.k = d_k.get();
        ga.r = d_r.get();
        h->offset.allocate( n_tgt + 1, s );
        {
            // row lengths: min(k_p, sources of p) for kNN, a count pass for radius
            DeviceBuffer<int64_t> counts( std::max<int64_t>( 1, n_tgt ), s ), offs( n_tgt + 1, s );
            if ( !radius_mode )
            {
                if ( n_tgt )
                {
                    k_knn_rows<<<(unsigned)( ( n_tgt + 255 ) / 256 ), 256, 0, s>>>(
                        n_tgt, tgt_grp.get(), d_src_off.get(), d_k.get(), counts.get() );
                    check_launch( "k_knn_rows" );
                }
            }
            else
                radius_count( tree, tv, order.get(), 0.0, ga, counts.get(), status.get(), s );
            exclusive_scan_i64( counts.get(), offs.get(), n_tgt, s );
            int64_t total = 0;
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( &total, offs.get() + n_tgt, 8, cudaMemcpyDeviceToHost, s ) );
            DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
            DTK_REQUIRE_OR_THROW( total <= INT32_MAX, "neighbour count exceeds int32 offsets" );
            h->nnz = total;
            k_narrow32<<<(unsigned)( ( n_tgt + 256 ) / 256 ), 256, 0, s>>>( offs.get(), h->offset.get(), n_tgt );
            check_launch( "k_narrow32" );
        }
        h->idx.allocate( std::max<int64_t>( 1, h->nnz ), s );
        if ( !radius_mode )
            knn_query( tree, tv, order.get(), 0, ga, h->offset.get(), h->idx.get(), status.get(), s );
        else
            radius_fill( tree, tv, order.get(), 0.0, ga, h->offset.get(), h->idx.get(), status.get(), s );
        tree = Lbvh();
        DTK_CUDA_OR_THROW( cudaEventRecord( ev[1], s ) );

        // --- setup, bucketed on the device by (basis, rbf, path) ---
        std::vector<uint8_t> basis_h( n_problems ), rbf_h( n_problems );
        for ( int p = 0; p < n_problems; ++p )
        {
            basis_h[p] = (uint8_t)opts[p].basis;
            rbf_h[p] = (uint8_t)opts[p].rbf;
        }
        DeviceBuffer<uint8_t> basis_g( n_problems, s ), rbf_g( n_problems, s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( basis_g.get(), basis_h.data(), n_problems, cudaMemcpyHostToDevice, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( rbf_g.get(), rbf_h.data(), n_problems, cudaMemcpyHostToDevice, s ) );
        SetupArgs a{};
        a.src = sv;
        a.tgt = tv;
        a.offset = h->offset.get();
        a.idx = h->idx.get();
        a.order = order.get();
        a.n_tgt = n_tgt;
        a.rows_sorted = !radius_mode;
        a.underdetermined = counters.get();
        a.rotations = counters.get() + 1;
        a.rotations32 = counters.get() + 2;
        a.status = status.get();
        if ( precision == DTK_FP64 )
        {
            h->coeff64.allocate( std::max<int64_t>( 1, h->nnz ), s );
            a.coeff64 = h->coeff64.get();
        }
        else
        {
            h->coeff32.allocate( std::max<int64_t>( 1, h->nnz ), s );
            a.coeff32 = h->coeff32.get();
        }
        auto const t1 = std::chrono::steady_clock::now();
        h->radius_mode = radius_mode;
        run_setup_plan( a, precision, basis_g.get(), rbf_g.get(), tgt_grp.get(), radius_mode, s, &h->plan,
                        true );
        host_ms += ms_since( t1 );
        DTK_CUDA_OR_THROW( cudaEventRecord( ev[2], s ) );

        // --- apply bins: rows grouped by length, processing order within a bin ---
        if ( n_tgt )
        {
            DeviceBuffer<uint32_t> keys( n_tgt, s );
            DeviceBuffer<unsigned> hist( dtk_mls_batch_s::NBINS, s );
            h->rows.allocate( n_tgt, s );
            DTK_CUDA_OR_THROW( cudaMemsetAsync( hist.get(), 0, dtk_mls_batch_s::NBINS * sizeof( unsigned ), s ) );
            k_bin_keys<<<(unsigned)( ( n_tgt + 255 ) / 256 ), 256, 0, s>>>(
                n_tgt, order.get(), h->offset.get(), keys.get(), reinterpret_cast<uint32_t *>( h->rows.get() ),
                hist.get() );
            check_launch( "k_bin_keys" );
            radix_sort_pairs( keys.get(), reinterpret_cast<uint32_t *>( h->rows.get() ), n_tgt, 8, s );
            unsigned hb[dtk_mls_batch_s::NBINS];
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( hb, hist.get(), sizeof( hb ), cudaMemcpyDeviceToHost, s ) );
            DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
            h->bin_start.assign( dtk_mls_batch_s::NBINS + 1, 0 );
            for ( int b = 0; b < dtk_mls_batch_s::NBINS; ++b )
                h->bin_start[b + 1] = h->bin_start[b] + hb[b];
        }
        else
            h->bin_start.assign( dtk_mls_batch_s::NBINS + 1, 0 );

        unsigned st = 0;
        unsigned long long cnt[3] = {0, 0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( cnt, counters.get(), sizeof( cnt ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop hit its cap"};
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "search or setup reported an internal error"};
        h->underdetermined = (int64_t)cnt[0];
        h->rotations = (int64_t)cnt[1];
        DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->search_ms, ev[0], ev[1] ) );
        DTK_CUDA_OR_THROW( cudaEventElapsedTime( &h->setup_ms, ev[1], ev[2] ) );
        h->host_ms = (float)host_ms;
        *out = h.release();
    } );
}

dtk_status dtk_mls_batch_apply( dtk_mls_batch_handle h, const double *src_values, double *tgt_values,
                                int32_t use_graph, dtk_stream_t stream_ )
{
    return guarded( [&] {
        NvtxRange const nvtx_range( "DTK_compute_values" );
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        DTK_REQUIRE_OR_THROW( src_values != nullptr && ( h->n_tgt == 0 || tgt_values != nullptr ),
                              "null values" );
        require_device_memory( src_values, "src_values" );
        require_device_memory( tgt_values, "tgt_values" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        if ( !h->tuned )
            h->tune( src_values, tgt_values, s );
        if ( !use_graph )
        {
            h->launch( h->tasks.get(), h->n_tasks, src_values, tgt_values, s );
            return;
        }
        if ( !h->exec || h->g_src != src_values || h->g_tgt != tgt_values )
        {
            if ( h->exec )
            {
                cudaGraphExecDestroy( h->exec );
                h->exec = nullptr;
            }
            if ( h->graph )
            {
                cudaGraphDestroy( h->graph );
                h->graph = nullptr;
            }
            if ( !h->capture )
                DTK_CUDA_OR_THROW( cudaStreamCreateWithFlags( &h->capture, cudaStreamNonBlocking ) );
            DTK_CUDA_OR_THROW( cudaStreamBeginCapture( h->capture, cudaStreamCaptureModeThreadLocal ) );
            h->launch( h->tasks.get(), h->n_tasks, src_values, tgt_values, h->capture );
            DTK_CUDA_OR_THROW( cudaStreamEndCapture( h->capture, &h->graph ) );
            DTK_CUDA_OR_THROW( cudaGraphInstantiate( &h->exec, h->graph, 0 ) );
            h->g_src = src_values;
            h->g_tgt = tgt_values;
        }
        DTK_CUDA_OR_THROW( cudaGraphLaunch( h->exec, s ) );
    } );
}

dtk_status dtk_mls_batch_resetup( dtk_mls_batch_handle h, const double *src, const double *tgt,
                                  dtk_stream_t stream_ )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        DTK_REQUIRE_OR_THROW( src != nullptr && ( h->n_tgt == 0 || tgt != nullptr ), "null points" );
        require_device_memory( src, "source points" );
        require_device_memory( h->n_tgt ? tgt : nullptr, "target points" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        if ( h->n_tgt == 0 )
            return;
        if ( !h->status.get() )
        {
            h->status.allocate( 1, s );
            h->counters.allocate( 3, s );
        }
        SetupArgs a{};
        a.src = PointsView{src, h->n_src, 3, 1};
        a.tgt = PointsView{tgt, h->n_tgt, 3, 1};
        a.offset = h->offset.get();
        a.idx = h->idx.get();
        a.order = nullptr;
        a.n_tgt = h->n_tgt;
        a.rows_sorted = false; // rows kept from other coordinates need not be sorted any more
        a.coeff64 = h->coeff64.get();
        a.coeff32 = h->coeff32.get();
        a.underdetermined = h->counters.get();
        a.rotations = h->counters.get() + 1;
        a.rotations32 = h->counters.get() + 2;
        a.status = h->status.get();
        auto enqueue = [&]( cudaStream_t q ) {
            DTK_CUDA_OR_THROW( cudaMemsetAsync( h->status.get(), 0, sizeof( unsigned ), q ) );
            DTK_CUDA_OR_THROW( cudaMemsetAsync( h->counters.get(), 0, 3 * sizeof( unsigned long long ), q ) );
            run_planned_setup( a, h->plan, q );
        };
        // one graph: the statistics reset and the persistent setup launch (and
        // the fused mixed kernel per mixed kNN bucket), captured once per pair
        // of point arrays and replayed
        if ( !h->setup_exec || h->gs_src != src || h->gs_tgt != tgt )
        {
            if ( h->setup_exec )
            {
                cudaGraphExecDestroy( h->setup_exec );
                h->setup_exec = nullptr;
            }
            if ( h->setup_graph )
            {
                cudaGraphDestroy( h->setup_graph );
                h->setup_graph = nullptr;
            }
            if ( !h->capture )
                DTK_CUDA_OR_THROW( cudaStreamCreateWithFlags( &h->capture, cudaStreamNonBlocking ) );
            DTK_CUDA_OR_THROW( cudaStreamBeginCapture( h->capture, cudaStreamCaptureModeThreadLocal ) );
            try
            {
                enqueue( h->capture );
            }
            catch ( ... )
            {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture( h->capture, &g );
                if ( g )
                    cudaGraphDestroy( g );
                throw;
            }
            DTK_CUDA_OR_THROW( cudaStreamEndCapture( h->capture, &h->setup_graph ) );
            DTK_CUDA_OR_THROW( cudaGraphInstantiate( &h->setup_exec, h->setup_graph, 0 ) );
            h->gs_src = src;
            h->gs_tgt = tgt;
        }
        DTK_CUDA_OR_THROW( cudaGraphLaunch( h->setup_exec, s ) );
        ++h->setup_replays;
        unsigned st = 0;
        unsigned long long cnt[3] = {0, 0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( &st, h->status.get(), sizeof( st ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( cnt, h->counters.get(), sizeof( cnt ), cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( st & DEV_TIMEOUT )
            throw Error{DTK_ERR_TIMEOUT, "a bounded device loop hit its cap"};
        if ( st )
            throw Error{DTK_ERR_INTERNAL, "the setup reported an internal error"};
        h->underdetermined = (int64_t)cnt[0];
        h->rotations = (int64_t)cnt[1];
    } );
}

dtk_status dtk_mls_batch_get_config( dtk_mls_batch_handle h, int32_t *setup_lanes, int32_t *apply_lanes,
                                     int64_t *setup_graph_replays )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( setup_lanes )
            for ( int p = 0; p < 3; ++p )
                setup_lanes[p] = h->plan.lanes[p];
        if ( apply_lanes )
            for ( int b = 0; b < dtk_mls_batch_s::NBINS; ++b )
                apply_lanes[b] = h->tuned && h->bin_start[b + 1] > h->bin_start[b] ? h->lanes[b] : 0;
        if ( setup_graph_replays )
            *setup_graph_replays = h->setup_replays;
    } );
}

dtk_status dtk_mls_batch_get_csr( dtk_mls_batch_handle h, const int32_t **offset, const int32_t **indices,
                                  const void **coeff, int64_t *nnz, int32_t *coeff_is_fp32 )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        bool const f32 = h->coeff32.get() != nullptr;
        if ( offset )
            *offset = h->offset.get();
        if ( indices )
            *indices = h->idx.get();
        if ( coeff )
            *coeff = f32 ? (const void *)h->coeff32.get() : (const void *)h->coeff64.get();
        if ( nnz )
            *nnz = h->nnz;
        if ( coeff_is_fp32 )
            *coeff_is_fp32 = f32 ? 1 : 0;
    } );
}

dtk_status dtk_mls_batch_get_stage_times( dtk_mls_batch_handle h, float *search_ms, float *setup_ms,
                                          float *host_ms )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr, "handle is null" );
        if ( search_ms )
            *search_ms = h->search_ms;
        if ( setup_ms )
            *setup_ms = h->setup_ms;
        if ( host_ms )
            *host_ms = h->host_ms;
    } );
}

dtk_status dtk_mls_batch_destroy( dtk_mls_batch_handle h )
{
    return guarded( [&] { delete h; } );
}

} // extern "C"
