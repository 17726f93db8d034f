"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the DataTransferKit sources are present: the reference's MLS
numerics headers (DTK_DetailsMovingLeastSquaresOperatorImpl.hpp,
DTK_DetailsSVDImpl.hpp, DTK_CompactlySupportedRadialBasisFunctions.hpp,
DTK_MultivariatePolynomialBasis.hpp) are compiled unchanged against the
project's API shim (oracle/ref_shim, oracle/ref_driver.cpp) and run on seeded
inputs.  The neighbour connectivity comes from the oracle's exact kNN (the
reference's ArborX search is not vendored).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import cpu, ref  # noqa: E402
from datatransferkit_gb300 import synthetic as syn  # noqa: E402

BASIS_SIZE = {0: 1, 1: 4, 2: 10}


def mls_case(name, src, tgt, values, rbf, basis, k):
    off, idx, d2 = cpu.knn(src, tgt, k)
    coeff, under = ref.mls_coefficients(src, tgt, off, idx, rbf, basis)
    target = ref.apply(off, idx, coeff, values)
    np.savez_compressed(HERE / f"{name}.npz", src=src, tgt=tgt, values=values, offset=off,
                        idx=idx, d2=d2, coeff=coeff, target=target, underdetermined=under,
                        rbf=rbf, basis=basis, k=k)
    print(f"{name}: nnz={len(idx)} under={under}")


def main():
    if not ref.available():
        raise SystemExit("the reference sources are not available here")
    # Known-answer layouts of tstMeshfreeOperators.cpp (Wendland<0>, k = basis size)
    for basis in (0, 1, 2):
        m = BASIS_SIZE[basis]
        f = syn.polynomial_of_basis(m)
        src, tgt = syn.cluster_problem(10, m, 0.5, seed=11)
        mls_case(f"kat_same_npoints_b{basis}", src, tgt, f(src), 0, basis, m)
        src = syn.grid_points((40, 40, 1), (0.0, 0.0, 0.0))
        tgt = syn.grid_points((1, 1, 1), (19.0, 19.0, 0.0))
        mls_case(f"kat_grid_b{basis}", src, tgt, f(src), 0, basis, m)
        src = syn.grid_points((40, 1, 1), (0.0, 0.0, 0.0))
        tgt = syn.grid_points((39, 1, 1), (0.5, 0.0, 0.0))
        mls_case(f"kat_line_b{basis}", src, tgt, f(src), 0, basis, m)
        src, tgt = syn.cluster_problem(10, 1, 0.5, seed=12)
        mls_case(f"kat_single_point_b{basis}", src, tgt, f(src), 0, basis, m)
    # corner case of tstMeshfreeOperatorsSimpleProblem.cpp:116-130
    mls_case("kat_corner", np.array([[1.0, 1, 1], [2.0, 2, 2]]), np.array([[1.5, 1.5, 1.5]]),
             np.array([255.0, 255.0]), 0, 1, 4)
    # Small clouds of the benchmark workloads (plain_cpu layout, reduced size)
    src = syn.uniform_points(3000, 1)
    tgt = syn.uniform_points(1000, 2)
    mls_case("uniform_w2_q_k20", src, tgt, syn.smooth_field(src), 1, 2, 20)
    mls_case("uniform_w4_q_k32", src, tgt, syn.smooth_field(src), 2, 2, 32)
    mls_case("uniform_w0_l_k4", src, tgt, syn.smooth_field(src), 0, 1, 4)
    # SVD known answers (tstSVD.cpp:67-150 layouts, own seeded inputs)
    rng = np.random.default_rng(13)
    full = rng.uniform(-1000, 1000, (10, 32, 32))
    pf, uf = ref.svd_pinv(full)
    deficient = rng.uniform(-1000, 1000, (10, 40, 40))
    deficient[:, :, 3] = 0.0
    pd, ud = ref.svd_pinv(deficient)
    np.savez_compressed(HERE / "svd.npz", full=full, full_pinv=pf, full_under=uf,
                        deficient=deficient, deficient_pinv=pd, deficient_under=ud)
    print(f"svd: under full={uf} deficient={ud}")
    # RBF and basis values
    x = np.arange(10) / 10.0
    rbf_vals = np.stack([ref.rbf(r, x) for r in range(9)])
    pts = np.array([[0.0, 0, 0], [0.0, 1, 2], [1.5, -2.0, 0.25]])
    np.savez_compressed(HERE / "rbf_basis.npz", x=x, rbf=rbf_vals, pts=pts,
                        b0=ref.basis(0, pts), b1=ref.basis(1, pts), b2=ref.basis(2, pts))
    print("rbf_basis: ok")


if __name__ == "__main__":
    main()
