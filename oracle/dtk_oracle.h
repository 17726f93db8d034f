/*
 * CPU oracle for the moving-least-squares (MLS) transfer path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU product
 * is compared against and the timed CPU baseline of the benchmark.  Nothing
 * in the product (datatransferkit_gb300/, include/) links, loads or calls it.
 *
 * It restates, in plain FP64 C++ with OpenMP over targets, the algorithm of
 *   packages/Meshfree/src/DTK_MovingLeastSquaresOperator_def.hpp:24-141
 *   packages/Meshfree/src/DTK_DetailsMovingLeastSquaresOperatorImpl.hpp:49-336
 *   packages/Meshfree/src/DTK_DetailsSVDImpl.hpp:29-302
 *   packages/Meshfree/src/DTK_CompactlySupportedRadialBasisFunctions.hpp:22-147
 *   packages/Meshfree/src/DTK_MultivariatePolynomialBasis.hpp:98-125
 * and the neighbour contract of the (un-vendored) ArborX nearest / radius
 * queries used at DTK_MovingLeastSquaresOperator_def.hpp:47-60:
 *   row i = the min(k, n_src) smallest (d2, source index) pairs in
 *   lexicographic order, ascending, d2 = (dx*dx + dy*dy) + dz*dz with
 *   dx = s.x - t.x, every operation rounded separately (no FMA).
 *   Radius rows hold every source with sqrt(d2) <= r, in the same order.
 *
 * All point arrays are row-major n x 3 doubles (point stride 3).
 * Parity of the restatement is pinned against the reference's own numerics
 * headers compiled with a project-written API shim (oracle/ref_driver.cpp)
 * and against the reference's known-answer tests (tests/test_oracle_*.py).
 */
#ifndef DTK_ORACLE_H
#define DTK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int dtk_oracle_max_threads(void);
void dtk_oracle_set_threads(int n);

/* Exact kNN over a uniform-grid index.  offset: n_tgt+1, idx/d2: n_tgt *
 * min(k, n_src).  d2 may be NULL.  Returns 0, or -1 on bad arguments. */
int dtk_oracle_knn(const double *src, int64_t n_src, const double *tgt,
                   int64_t n_tgt, int k, int32_t *offset, int32_t *idx,
                   double *d2);
/* Same contract by exhaustive search (small cases, cross-check). */
int dtk_oracle_knn_brute(const double *src, int64_t n_src, const double *tgt,
                         int64_t n_tgt, int k, int32_t *offset, int32_t *idx,
                         double *d2);
/* Radius search, two phases: count fills offset (n_tgt+1) and returns nnz;
 * fill writes idx/d2 (nnz) given that offset. */
int64_t dtk_oracle_radius_count(const double *src, int64_t n_src,
                                const double *tgt, int64_t n_tgt, double r,
                                int32_t *offset);
int dtk_oracle_radius_fill(const double *src, int64_t n_src, const double *tgt,
                           int64_t n_tgt, double r, const int32_t *offset,
                           int32_t *idx, double *d2);

/* MLS setup numerics for given CSR connectivity (offset, idx).
 * Writes coeff[nnz]; radius[n_tgt] and row0[n_tgt*m] when non-NULL.
 * Returns the number of rank-deficient (underdetermined) moment matrices,
 * or -1 on bad arguments. */
int64_t dtk_oracle_mls_coefficients(const double *src, const double *tgt,
                                    int64_t n_tgt, const int32_t *offset,
                                    const int32_t *idx, int rbf, int basis,
                                    double *coeff, double *radius,
                                    double *row0);
/* target[i] = sum_j coeff[j] * values[idx[j]] (DTK apply on one rank). */
int dtk_oracle_apply(int64_t n_tgt, const int32_t *offset, const int32_t *idx,
                     const double *coeff, const double *values,
                     double *target);
/* Transpose of apply: grad[s] = sum over entries j with idx[j]==s of
 * coeff[j]*cot[row(j)], summed in ascending entry order. */
int dtk_oracle_apply_transpose(int64_t n_tgt, int64_t n_src,
                               const int32_t *offset, const int32_t *idx,
                               const double *coeff, const double *cot,
                               double *grad);
/* d/d(source coordinates) of L where dL/d(target) = cot, connectivity fixed.
 * grad_xyz: n_src x 3, accumulated (caller zeroes). */
int dtk_oracle_coord_grad(const double *src, int64_t n_src, const double *tgt,
                          int64_t n_tgt, const int32_t *offset,
                          const int32_t *idx, int rbf, int basis,
                          const double *values, const double *cot,
                          double *grad_xyz);

/* Batched Jacobi pseudo-inverse of count n x n row-major matrices, exactly
 * the DTK SVDFunctor algorithm.  Returns the underdetermined count. */
int64_t dtk_oracle_svd_pinv(int n, int64_t count, const double *a,
                            double *pinv);

void dtk_oracle_rbf(int rbf, const double *x, int64_t n, double *out);
int dtk_oracle_basis_size(int basis);
void dtk_oracle_basis(int basis, const double *pts, int64_t n, double *out);

#ifdef __cplusplus
}
#endif
#endif
