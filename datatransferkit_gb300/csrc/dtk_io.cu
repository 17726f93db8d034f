// The operator product on disk and on the wire (extension): the CSR that
// setup produces -- offset, source indices, coefficients, the members of
// DataTransferKit::MovingLeastSquaresOperator
// (packages/Meshfree/src/DTK_MovingLeastSquaresOperator_decl.hpp:56-62) -- in a
// flat little-endian byte layout, so that apply can be reused across restarts
// and shipped to other processes without repeating the search and the setup.
//
// Layout (all little-endian):
//   bytes  0..7   magic "DTKMLS01"
//          8..11  uint32 format version (1)
//         12..15  uint32 flags: bit 0 = coefficients are FP32 (mixed form)
//         16..39  int64 n_src, n_tgt, nnz
//         40..55  int32 rbf, basis, k, precision
//         56..63  double radius
//   then  int32 offset[n_tgt + 1], int32 indices[nnz],
//         coefficients[nnz] (double, or float when flag bit 0),
//   then  uint64 checksum of every preceding byte (64-bit FNV-1a over 8-byte
//         little-endian words, the tail zero-padded).
// Import validates the magic, version, sizes, offsets (monotone, from 0 to
// nnz), index range and checksum, and rejects anything else with
// DTK_ERR_INVALID_ARG.
#include "dtk_common.cuh"
#include "dtk_handle.cuh"

#include <cstring>
#include <memory>
#include <vector>

namespace dtk
{
namespace
{

constexpr char MAGIC[8] = {'D', 'T', 'K', 'M', 'L', 'S', '0', '1'};
constexpr uint32_t VERSION = 1;
constexpr int64_t HEADER = 64;

uint64_t checksum( unsigned char const *p, int64_t n )
{
    uint64_t h = 1469598103934665603ull;
    int64_t i = 0;
    for ( ; i + 8 <= n; i += 8 )
    {
        uint64_t w;
        std::memcpy( &w, p + i, 8 );
        h = ( h ^ w ) * 1099511628211ull;
    }
    if ( i < n )
    {
        uint64_t w = 0;
        std::memcpy( &w, p + i, (size_t)( n - i ) );
        h = ( h ^ w ) * 1099511628211ull;
    }
    return h;
}

bool little_endian()
{
    uint32_t const one = 1;
    unsigned char b;
    std::memcpy( &b, &one, 1 );
    return b == 1;
}

int64_t payload_bytes( int64_t n_tgt, int64_t nnz, bool f32 )
{
    return 4 * ( n_tgt + 1 ) + 4 * nnz + ( f32 ? 4 : 8 ) * nnz;
}

} // namespace
} // namespace dtk

using namespace dtk;

extern "C" {

dtk_status dtk_mls_export_size( dtk_mls_handle h, int64_t *bytes )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr && bytes != nullptr, "null argument" );
        *bytes = HEADER + payload_bytes( h->n_tgt, h->nnz, h->coeff32.get() != nullptr ) + 8;
    } );
}

dtk_status dtk_mls_export( dtk_mls_handle h, void *host_buffer, int64_t bytes, dtk_stream_t stream_ )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( h != nullptr && host_buffer != nullptr, "null argument" );
        if ( !little_endian() )
            throw Error{DTK_ERR_UNSUPPORTED, "the product format is little-endian"};
        bool const f32 = h->coeff32.get() != nullptr;
        int64_t const need = HEADER + payload_bytes( h->n_tgt, h->nnz, f32 ) + 8;
        DTK_REQUIRE_OR_THROW( bytes >= need, "buffer smaller than dtk_mls_export_size" );
        unsigned char *p = static_cast<unsigned char *>( host_buffer );
        std::memset( p, 0, HEADER );
        std::memcpy( p, MAGIC, 8 );
        uint32_t const flags = f32 ? 1u : 0u;
        std::memcpy( p + 8, &VERSION, 4 );
        std::memcpy( p + 12, &flags, 4 );
        int64_t const sizes[3] = {h->n_src, h->n_tgt, h->nnz};
        std::memcpy( p + 16, sizes, 24 );
        int32_t const o[4] = {h->opts.rbf, h->opts.basis, h->opts.k, h->opts.precision};
        std::memcpy( p + 40, o, 16 );
        std::memcpy( p + 56, &h->opts.radius, 8 );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        TouchOnExit const touch{&h->life, s};
        int64_t at = HEADER;
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( p + at, h->offset.get(), 4 * ( h->n_tgt + 1 ),
                                            cudaMemcpyDeviceToHost, s ) );
        at += 4 * ( h->n_tgt + 1 );
        if ( h->nnz )
        {
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( p + at, h->idx.get(), 4 * h->nnz, cudaMemcpyDeviceToHost, s ) );
            at += 4 * h->nnz;
            void const *c = f32 ? (void const *)h->coeff32.get() : (void const *)h->coeff64.get();
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( p + at, c, ( f32 ? 4 : 8 ) * h->nnz, cudaMemcpyDeviceToHost, s ) );
            at += ( f32 ? 4 : 8 ) * h->nnz;
        }
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        uint64_t const sum = checksum( p, at );
        std::memcpy( p + at, &sum, 8 );
    } );
}

dtk_status dtk_mls_import( const void *host_buffer, int64_t bytes, dtk_stream_t stream_, dtk_mls_handle *out )
{
    return guarded( [&] {
        DTK_REQUIRE_OR_THROW( out != nullptr && host_buffer != nullptr, "null argument" );
        *out = nullptr;
        if ( !little_endian() )
            throw Error{DTK_ERR_UNSUPPORTED, "the product format is little-endian"};
        unsigned char const *p = static_cast<unsigned char const *>( host_buffer );
        DTK_REQUIRE_OR_THROW( bytes >= HEADER + 4 + 8, "buffer too short for a product" );
        DTK_REQUIRE_OR_THROW( std::memcmp( p, MAGIC, 8 ) == 0, "not an MLS operator product (bad magic)" );
        uint32_t version, flags;
        std::memcpy( &version, p + 8, 4 );
        std::memcpy( &flags, p + 12, 4 );
        DTK_REQUIRE_OR_THROW( version == VERSION, "unsupported product format version" );
        DTK_REQUIRE_OR_THROW( ( flags & ~1u ) == 0, "unknown product flags" );
        bool const f32 = flags & 1u;
        int64_t sizes[3];
        std::memcpy( sizes, p + 16, 24 );
        int64_t const n_src = sizes[0], n_tgt = sizes[1], nnz = sizes[2];
        DTK_REQUIRE_OR_THROW( n_src > 0 && n_src <= INT32_MAX && n_tgt >= 0 && n_tgt < INT32_MAX && nnz >= 0 &&
                                  nnz <= INT32_MAX,
                              "product sizes out of range" );
        int64_t const need = HEADER + payload_bytes( n_tgt, nnz, f32 ) + 8;
        DTK_REQUIRE_OR_THROW( bytes == need, "product size does not match its header" );
        uint64_t sum;
        std::memcpy( &sum, p + need - 8, 8 );
        DTK_REQUIRE_OR_THROW( checksum( p, need - 8 ) == sum, "product checksum mismatch" );
        cudaStream_t s = reinterpret_cast<cudaStream_t>( stream_ );
        auto h = std::make_unique<dtk_mls_s>( s );
        dtk_mls_default_options( &h->opts );
        int32_t o[4];
        std::memcpy( o, p + 40, 16 );
        h->opts.rbf = o[0];
        h->opts.basis = o[1];
        h->opts.k = o[2];
        h->opts.precision = o[3];
        std::memcpy( &h->opts.radius, p + 56, 8 );
        h->n_src = n_src;
        h->n_tgt = n_tgt;
        h->nnz = nnz;
        h->m = basis_size( h->opts.basis );
        // offsets: monotone from 0 to nnz; uniform rows take the vector apply
        std::vector<int32_t> off( n_tgt + 1 );
        std::memcpy( off.data(), p + HEADER, 4 * ( n_tgt + 1 ) );
        DTK_REQUIRE_OR_THROW( off[0] == 0 && off[n_tgt] == nnz, "product offsets do not span the entries" );
        int64_t const row = n_tgt ? nnz / n_tgt : 0;
        bool uniform = n_tgt > 0 && row * n_tgt == nnz;
        for ( int64_t i = 0; i < n_tgt; ++i )
        {
            DTK_REQUIRE_OR_THROW( off[i + 1] >= off[i], "product offsets decrease" );
            uniform = uniform && off[i + 1] - off[i] == row;
        }
        int32_t const *idx = reinterpret_cast<int32_t const *>( p + HEADER + 4 * ( n_tgt + 1 ) );
        for ( int64_t j = 0; j < nnz; ++j )
        {
            int32_t v;
            std::memcpy( &v, idx + j, 4 );
            DTK_REQUIRE_OR_THROW( v >= 0 && v < n_src, "product index out of range" );
        }
        h->uniform_row = uniform ? (int)row : 0;
        h->mean_row = n_tgt ? (int)( ( nnz + n_tgt - 1 ) / n_tgt ) : 0;
        TouchOnExit const touch{&h->life, s};
        h->offset.allocate( n_tgt + 1, s );
        h->idx.allocate( std::max<int64_t>( 1, nnz ), s );
        DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->offset.get(), off.data(), 4 * ( n_tgt + 1 ), cudaMemcpyHostToDevice, s ) );
        unsigned char const *c = p + HEADER + 4 * ( n_tgt + 1 ) + 4 * nnz;
        if ( f32 )
            h->coeff32.allocate( std::max<int64_t>( 1, nnz ), s );
        else
            h->coeff64.allocate( std::max<int64_t>( 1, nnz ), s );
        if ( nnz )
        {
            DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->idx.get(), idx, 4 * nnz, cudaMemcpyHostToDevice, s ) );
            if ( f32 )
                DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->coeff32.get(), c, 4 * nnz, cudaMemcpyHostToDevice, s ) );
            else
                DTK_CUDA_OR_THROW( cudaMemcpyAsync( h->coeff64.get(), c, 8 * nnz, cudaMemcpyHostToDevice, s ) );
        }
        // the caller may release its buffer on return
        DTK_CUDA_OR_THROW( cudaStreamSynchronize( s ) );
        *out = h.release();
    } );
}

} // extern "C"
