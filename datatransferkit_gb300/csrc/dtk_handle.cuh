// The operator handle behind dtk_mls_handle (internal).
//
// Mirrors the data members of DataTransferKit::MovingLeastSquaresOperator
// (packages/Meshfree/src/DTK_MovingLeastSquaresOperator_decl.hpp:56-62): the
// CSR offset, the source indices and the coefficients, plus the source count.
// The reference's `_ranks` array is absent: on one rank every rank is 0 and
// the fetch is a local gather fused into apply.
#pragma once

#include "dtk_common.cuh"

struct dtk_mls_s
{
    dtk::HandleLife life; // first: its event outlives the buffers' frees
    dtk_mls_options opts;
    explicit dtk_mls_s( cudaStream_t home )
        : life( home )
    {
    }
    int64_t n_src = 0, n_tgt = 0, nnz = 0;
    int m = 0;
    int uniform_row = 0; // > 0 for kNN rows
    int mean_row = 0;
    dtk::DeviceBuffer<int32_t> offset, idx;
    dtk::DeviceBuffer<double> coeff64;
    dtk::DeviceBuffer<float> coeff32;
    dtk::DeviceBuffer<uint32_t> order;            // Morton order of targets
    // kNN operators: the entries' sorted positions in the source tree
    // (parallel to idx) and the tree's position -> index map, for the apply
    dtk::DeviceBuffer<int32_t> pos;
    dtk::DeviceBuffer<uint32_t> perm;
    dtk::DeviceBuffer<double> src_copy, tgt_copy; // packed n x 3 (keep_points)
    // transpose of the CSR (source -> its entries, ascending), built on the
    // first adjoint call
    dtk::DeviceBuffer<int32_t> t_offset, t_entry;
    int64_t underdetermined = 0;
    int64_t rotations = 0, rotations32 = 0;
    float search_ms = 0.f, setup_ms = 0.f;
    float build_ms = 0.f, query_ms = 0.f; // the search split: tree build + query sort, kNN/radius queries

    ~dtk_mls_s()
    {
        life.retire( offset, idx, coeff64, coeff32, order, pos, perm, src_copy, tgt_copy, t_offset, t_entry );
    }
};
