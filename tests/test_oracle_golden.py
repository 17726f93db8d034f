"""The CPU oracle against golden fixtures produced by the reference's own numerics.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs
DataTransferKit's MLS numerics headers compiled unchanged (against the
project's API shim).  The oracle restatement reproduces them bit for bit on
this host; the tolerance below only absorbs libm differences between hosts.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import cpu

GOLDEN = Path(__file__).resolve().parent / "golden"
MLS_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if p.stem not in ("svd", "rbf_basis"))


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


@pytest.mark.parametrize("name", MLS_CASES)
def test_mls_golden(name):
    g = load(name)
    off, idx, d2 = cpu.knn(g["src"], g["tgt"], int(g["k"]))
    assert np.array_equal(off, g["offset"]) and np.array_equal(idx, g["idx"])
    coeff, rad, _, under = cpu.mls_coefficients(g["src"], g["tgt"], off, idx, int(g["rbf"]),
                                                int(g["basis"]))
    assert under == int(g["underdetermined"])
    scale = np.maximum(np.abs(g["coeff"]).max(), 1e-300)
    assert np.abs(coeff - g["coeff"]).max() <= 1e-13 * scale
    target = cpu.apply(off, idx, coeff, g["values"])
    tscale = np.maximum(np.abs(g["target"]).max(), 1e-300)
    assert np.abs(target - g["target"]).max() <= 1e-13 * tscale


def test_svd_golden():
    g = load("svd")
    p, u = cpu.svd_pinv(g["full"])
    assert u == int(g["full_under"])
    assert np.abs(p - g["full_pinv"]).max() <= 1e-13 * np.abs(g["full_pinv"]).max()
    p, u = cpu.svd_pinv(g["deficient"])
    assert u == int(g["deficient_under"]) == 10
    assert np.abs(p - g["deficient_pinv"]).max() <= 1e-13 * np.abs(g["deficient_pinv"]).max()


def test_rbf_basis_golden():
    g = load("rbf_basis")
    for r in range(9):
        v = cpu.rbf(r, g["x"])
        ref = g["rbf"][r]
        both_nan = np.isnan(v) & np.isnan(ref)
        assert np.all(both_nan | (np.abs(v - ref) <= 1e-15 * np.maximum(1, np.abs(ref))))
    for b in range(3):
        assert np.array_equal(cpu.basis(b, g["pts"]), g[f"b{b}"])


def test_oracle_is_bit_exact_with_reference_numerics_here():
    """Where the reference sources exist, compare with them directly."""
    from oracle import ref
    if not ref.available():
        pytest.skip("reference sources not present on this host")
    rng = np.random.default_rng(21)
    src = rng.random((2000, 3))
    tgt = rng.random((400, 3))
    for basis in (0, 1, 2):
        for rbf in range(9):
            off, idx, _ = cpu.knn(src, tgt, 16)
            c1, _, _, u1 = cpu.mls_coefficients(src, tgt, off, idx, rbf, basis)
            c2, u2 = ref.mls_coefficients(src, tgt, off, idx, rbf, basis)
            assert u1 == u2
            assert np.array_equal(c1, c2), (basis, rbf)
    a = rng.uniform(-1000, 1000, (4, 24, 24))
    p1, _ = cpu.svd_pinv(a)
    p2, _ = ref.svd_pinv(a)
    assert np.array_equal(p1, p2)
