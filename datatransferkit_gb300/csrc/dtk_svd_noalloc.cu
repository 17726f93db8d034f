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
// with cudaGetSymbolAddress once per device, on the first call with that
// device current, and cached.  Every call shares the array, so calls that
// overlap on the GPU race; each call clears the counters it reads.
#include "dtk_common.cuh"

#include <map>
#include <mutex>
#include <new>
#include <string>

namespace
{

constexpr int kCounterSlots = 4; // [0] underdetermined count, [1] status word

static __device__ __align__( 256 ) double g_svd_scratch[kCounterSlots + DTK_SVD_NOALLOC_MAX_DOUBLES];

std::mutex g_mutex;
std::map<int, double *> g_addr; // device -> device address of g_svd_scratch

double *scratch_address()
{
    int dev = 0;
    DTK_CUDA_OR_THROW( cudaGetDevice( &dev ) );
    std::lock_guard<std::mutex> lock( g_mutex );
    auto it = g_addr.find( dev );
    if ( it != g_addr.end() )
        return it->second;
    double *ptr = nullptr;
    DTK_CUDA_OR_THROW( cudaGetSymbolAddress( (void **)&ptr, g_svd_scratch ) );
    g_addr[dev] = ptr;
    return ptr;
}

} // namespace

extern "C" dtk_status dtk_svd_pinv_noalloc( int32_t n, int64_t count, const double *a, double *pinv,
                                            int64_t *underdetermined, dtk_stream_t stream_ )
{
    try
    {
        DTK_REQUIRE_OR_THROW( n >= 1 && n <= 64, "matrix size must be in [1, 64]" );
        DTK_REQUIRE_OR_THROW( count >= 0, "count is negative" );
        DTK_REQUIRE_OR_THROW( count == 0 || ( a && pinv ), "null matrix pointer" );
        int64_t const need = 3 * (int64_t)n * n * count;
        DTK_REQUIRE_OR_THROW( need <= DTK_SVD_NOALLOC_MAX_DOUBLES,
                              "3 * n * n * count = " + std::to_string( need ) +
                                  " doubles exceeds the static work area of " +
                                  std::to_string( DTK_SVD_NOALLOC_MAX_DOUBLES ) +
                                  " doubles; use dtk_svd_pinv" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        double *base = scratch_address();
        auto *under = reinterpret_cast<unsigned long long *>( base );
        auto *status = reinterpret_cast<unsigned *>( base + 1 );
        DTK_CUDA_OR_THROW( cudaMemsetAsync( base, 0, kCounterSlots * sizeof( double ), s ) );
        dtk::svd_pinv_batched_work( n, count, a, pinv, base + kCounterSlots, under, status, s );
        unsigned long long counters[2] = {0, 0};
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( counters, base, sizeof( counters ),
                                            cudaMemcpyDeviceToHost, s ) );
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        if ( (unsigned)counters[1] & dtk::DEV_TIMEOUT )
            throw dtk::Error{DTK_ERR_TIMEOUT, "a Jacobi iteration hit its iteration cap"};
        if ( underdetermined )
            *underdetermined = (int64_t)counters[0];
        return DTK_OK;
    }
    catch ( dtk::Error const &e )
    {
        dtk::set_error( e.msg );
        return e.status;
    }
    catch ( std::bad_alloc const & )
    {
        dtk::set_error( "host allocation failed" );
        return DTK_ERR_OOM;
    }
    catch ( std::exception const &e )
    {
        dtk::set_error( e.what() );
        return DTK_ERR_INTERNAL;
    }
}
