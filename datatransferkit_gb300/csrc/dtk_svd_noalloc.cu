// Batched pseudo-inverse that allocates no device memory (dtk_svd_pinv_noalloc).
//
// For callers that cannot call cudaMalloc -- code under a fixed device-memory
// budget, inside a framework whose allocator owns the device, or that cannot
// take an allocation's implicit synchronisation -- this entry point runs the
// batched Jacobi pseudo-inverse kernel on a work area that is a static device
// array of this file instead of a stream-ordered allocation.  The array
// (DTK_SVD_NOALLOC_MAX_DOUBLES doubles plus four counter slots) exists on
// every GPU that loads the library, until the process exits.  Host code
// cannot use the array's name as a device address: its address is looked up
// with cudaGetSymbolAddress on the first call with that device current, and
// cached.  Later calls look it up again whenever `stream` is not capturing
// (so the cache follows a device reset), and use the cached address while
// it is.  Every call shares the array, so calls that overlap on the GPU
// race; each call clears the counters it reads.
#include "dtk_common.cuh"

#include <map>
#include <mutex>
#include <string>

namespace
{

constexpr int kCounterSlots = 4; // [0] underdetermined count, [1] status word

static __device__ __align__( 256 ) double g_svd_scratch[kCounterSlots + DTK_SVD_NOALLOC_MAX_DOUBLES];

std::mutex g_mutex;
std::map<int, double *> g_addr; // device -> device address of g_svd_scratch

double *scratch_address( cudaStream_t s )
{
    int dev = 0;
    DTK_CUDA_OR_THROW( cudaGetDevice( &dev ) );
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    bool const capturing = cudaStreamIsCapturing( s, &cap ) != cudaSuccess ||
                           cap != cudaStreamCaptureStatusNone;
    if ( capturing )
        cudaGetLastError(); // an implicit-capture query error is not ours to keep
    std::lock_guard<std::mutex> lock( g_mutex );
    auto it = g_addr.find( dev );
    if ( capturing )
    {
        if ( it == g_addr.end() )
            throw dtk::Error{DTK_ERR_INVALID_ARG,
                             "the first dtk_svd_pinv_noalloc call on a device must come before "
                             "any stream capture (it looks up the work area's address)"};
        return it->second;
    }
    double *ptr = nullptr;
    DTK_CUDA_OR_THROW( cudaGetSymbolAddress( (void **)&ptr, g_svd_scratch ) );
    g_addr[dev] = ptr;
    return ptr;
}

} // namespace

extern "C" dtk_status dtk_svd_pinv_noalloc( int32_t n, int64_t count, const double *a, double *pinv,
                                            int64_t *underdetermined, dtk_stream_t stream_ )
{
    return dtk::guarded( [&] {
        DTK_REQUIRE_OR_THROW( n >= 1 && n <= 64, "matrix size must be in [1, 64]" );
        DTK_REQUIRE_OR_THROW( count >= 0, "count is negative" );
        int64_t const per_matrix = 3 * (int64_t)n * n;
        // bound count before forming 3 n^2 count, which could overflow
        DTK_REQUIRE_OR_THROW( count <= DTK_SVD_NOALLOC_MAX_DOUBLES / per_matrix,
                              "3 * n * n * count exceeds the static work area of " +
                                  std::to_string( DTK_SVD_NOALLOC_MAX_DOUBLES ) +
                                  " doubles (at most " +
                                  std::to_string( DTK_SVD_NOALLOC_MAX_DOUBLES / per_matrix ) +
                                  " matrices of this size); use dtk_svd_pinv" );
        DTK_REQUIRE_OR_THROW( count == 0 || ( a && pinv ), "null matrix pointer" );
        if ( count )
        {
            dtk::require_device_memory( a, "a" );
            dtk::require_device_memory( pinv, "pinv" );
        }
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        double *base = scratch_address( s );
        auto *under = reinterpret_cast<unsigned long long *>( base );
        auto *status = reinterpret_cast<unsigned *>( base + 1 );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( base, 0, kCounterSlots * sizeof( double ), s ) );
        dtk::svd_pinv_batched_work( n, count, a, pinv, base + kCounterSlots, under, status, s );
        unsigned long long counters[2] = {0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( counters, base, sizeof( counters ),
                                            cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( (unsigned)counters[1] & dtk::DEV_TIMEOUT )
            throw dtk::Error{DTK_ERR_TIMEOUT, "a bounded device loop (Jacobi rotations) hit its cap"};
        if ( underdetermined )
            *underdetermined = (int64_t)counters[0];
    } );
}
