"""The workloads' own configurations, at their stated sizes, on the full sets.

* Plain transfer, 10,000 sources / 10,000 targets U[0,1]^3 (seeds 1, 2),
  Quadratic3, Wendland<2>, k = 20, f = sin(2 pi x) cos(2 pi y) + z^2: neighbour
  rows bit-exact against the oracle; coefficients and target values within
  max(1e-12, 100 x the oracle's rounding spread); the approximation error
  against f at the targets is stated (2.97e-3 relative L2 by the oracle).
* FP64 form at scale, 2M sources U[0,1]^3 (seed 3), 126^3 jittered-grid
  targets (seed 4), Quadratic3, Wendland<2>, k = 32: all 2,000,376 neighbour
  rows bit-exact and all target values within 1e-12 relative L2.
* Adjoint, 1M sources / 1M targets U[0,1]^3 (seeds 8, 9), Quadratic3,
  Wendland<2>, k = 32, L = 1/2 ||T f - g||^2, g = f + 0.05 cos(4 pi z): the
  source-value gradient against the oracle's transpose (1e-12), the
  coordinate gradient against the oracle's analytic adjoint (relative L2
  5e-8, every entry within 2e-7 of the largest: the oracle differentiates the
  reference's Jacobi pseudo-inverse, whose deviation from the exact one grows
  with the density), and
  central finite differences (h = 1e-6) on 64 random unit directions (seed
  10) with the connectivity frozen to the operator's rows.  The forwards of
  the finite differences run on the GPU (an accurate FP64 forward in torch:
  radius-scaled moments and a direct solve, the smooth function the
  coordinate adjoint differentiates), about 0.2 s each instead of minutes on
  the host.
"""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn
from oracle import cpu

pytestmark = pytest.mark.gpu
Q = dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)
TOL = 1e-12


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def transfer(src, tgt, vals, rbf, k, precision="fp64", keep_points=False):
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), rbf, Q, k=k, precision=precision,
                                        keep_points=keep_points)
    out = torch.full((len(tgt),), np.nan, dtype=torch.float64, device="cuda")
    op.apply(dev(vals), out)
    return out.cpu().numpy(), op


def test_plain_10k_exact_config():
    src, tgt = syn.uniform_points(10_000, 1), syn.uniform_points(10_000, 2)
    f = syn.smooth_field(src)
    ref = cpu.mls_transfer(src, tgt, f, 1, 2, k=20)
    sc, st = cpu.rounding_spread(src, tgt, ref["offset"], ref["idx"], 1, 2, f, ref["coeff"])
    tol_c, tol_t = max(TOL, 100 * sc), max(TOL, 100 * st)
    y, op = transfer(src, tgt, f, dtk.Wendland(2), 20)
    off, idx, coeff = (t.cpu().numpy() for t in op.csr())
    assert np.array_equal(off, ref["offset"]) and np.array_equal(idx, ref["idx"])
    for i in range(len(tgt)):
        a, b = coeff[off[i]:off[i + 1]], ref["coeff"][off[i]:off[i + 1]]
        assert np.abs(a - b).max() <= tol_c * np.abs(b).max(), i
    err = rel_l2(y, ref["target"])
    assert err <= tol_t, err
    assert op.underdetermined == ref["underdetermined"] == 0
    approx = rel_l2(y, syn.smooth_field(tgt))
    print(f"\nplain 10k: rel L2 vs oracle {err:.2e} (bound {tol_t:.1e}); vs f at the targets {approx:.4e}")
    assert abs(approx - rel_l2(ref["target"], syn.smooth_field(tgt))) <= 1e-9
    assert approx < 4e-3
    # the mixed form on the same configuration
    ym, _ = transfer(src, tgt, f, dtk.Wendland(2), 20, precision="mixed")
    assert rel_l2(ym, ref["target"]) <= 1e-6


def test_fp64_2m_jittered_grid_full_set():
    src = syn.uniform_points(2_000_000, 3)
    tgt = syn.jittered_grid(126, 4)
    f = syn.smooth_field(src)
    y, op = transfer(src, tgt, f, dtk.Wendland(2), 32)
    off, idx, coeff = (t.cpu().numpy() for t in op.csr())
    r_off, r_idx, _ = cpu.knn(src, tgt, 32)
    assert len(tgt) == 2_000_376
    assert np.array_equal(off, r_off)
    bad = np.flatnonzero((idx != r_idx).reshape(len(tgt), 32).any(1))
    assert bad.size == 0, f"{bad.size} rows differ, first {bad[:5]}"
    r_coeff, _, _, under = cpu.mls_coefficients(src, tgt, r_off, r_idx, 1, 2)
    ref = cpu.apply(r_off, r_idx, r_coeff, f)
    err = rel_l2(y, ref)
    print(f"\nFP64 2M full set: {len(tgt)} rows bit-exact, rel L2 vs oracle {err:.2e}")
    assert err <= TOL
    assert op.underdetermined == under


def _torch_forward(src, tgt, idx, k, values):
    """Accurate FP64 forward with frozen connectivity (Quadratic3, Wendland<2>)."""
    n_t = tgt.shape[0]
    X = src[idx].view(n_t, k, 3) - tgt[:, None, :]
    rho = X.square().sum(-1).sqrt()
    R = 1.1 * torch.clamp(rho.max(1).values, min=10 * np.finfo(float).eps)
    Xh = X / R[:, None, None]
    x = rho / R[:, None]
    phi = (1 - x) ** 4 * (4 * x + 1)
    a, b, c = Xh.unbind(-1)
    P = torch.stack([torch.ones_like(a), a, b, c, a * a, a * b, a * c, b * b, b * c, c * c], -1)
    A = torch.einsum("tka,tkb->tab", P * phi[..., None], P)
    e0 = torch.zeros(n_t, 10, 1, dtype=torch.float64, device=src.device)
    e0[:, 0] = 1.0
    sol = torch.linalg.solve(A, e0)
    coef = phi * (P @ sol)[..., 0]
    return (coef * values[idx].view(n_t, k)).sum(1)


def test_adjoint_1m_against_oracle_and_finite_differences():
    n, k, h = 1_000_000, 32, 1e-6
    src, tgt = syn.uniform_points(n, 8), syn.uniform_points(n, 9)
    f = syn.smooth_field(src)
    g = syn.smooth_field(tgt) + 0.05 * np.cos(4 * np.pi * tgt[:, 2])
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), dtk.Wendland(2), Q, k=k,
                                        keep_points=True)
    off_t, idx_t, _ = op.csr()
    idx_l = idx_t.long()
    src_t, tgt_t, f_t, g_t = dev(src), dev(tgt), dev(f), dev(g)
    y = _torch_forward(src_t, tgt_t, idx_l, k, f_t)
    cot = y - g_t
    gv, gc = op.apply_adjoint(cot, f_t, coords=True)
    # central finite differences, connectivity frozen
    gen = torch.Generator(device="cuda").manual_seed(10)
    scale = float(gc.norm())
    worst_abs, worst_rel = 0.0, 0.0
    for _ in range(64):
        d = torch.randn(n, 3, dtype=torch.float64, device="cuda", generator=gen)
        d /= d.norm()
        yp = _torch_forward(src_t + h * d, tgt_t, idx_l, k, f_t)
        ym = _torch_forward(src_t - h * d, tgt_t, idx_l, k, f_t)
        # L(+) - L(-) = sum (yp - ym)(yp + ym - 2 g) / 2, without the cancellation
        fd = float(((yp - ym) * (yp + ym - 2 * g_t)).sum()) / (4 * h)
        gd = float((gc * d).sum())
        worst_abs = max(worst_abs, abs(fd - gd) / scale)
        worst_rel = max(worst_rel, abs(fd - gd) / abs(gd))
    print(f"\nadjoint 1M: max |FD - <grad,d>| / ||grad|| = {worst_abs:.2e}, "
          f"max relative to |<grad,d>| = {worst_rel:.2e}")
    # against the oracle (same connectivity)
    off, idx = off_t.cpu().numpy(), idx_t.cpu().numpy()
    coeff, _, _, _ = cpu.mls_coefficients(src, tgt, off, idx, 1, 2)
    cot_h = cot.cpu().numpy()
    gv_ref = cpu.apply_transpose(off, idx, coeff, cot_h, n)
    gv_err = float(np.abs(gv.cpu().numpy() - gv_ref).max() / np.abs(gv_ref).max())
    gc_ref = cpu.coord_grad(src, tgt, off, idx, 1, 2, f, cot_h)
    gc_h = gc.cpu().numpy()
    # the oracle differentiates the reference's Jacobi pseudo-inverse, whose
    # deviation from the exact one (absolute DBL_EPSILON stop on unscaled
    # moments) grows with the point density (1.1e-8 relative L2 measured
    # here); the GPU adjoint differentiates the accurate one, which the
    # finite differences check
    l2 = rel_l2(gc_h, gc_ref)
    worst = float(np.abs(gc_h - gc_ref).max() / np.abs(gc_ref).max())
    print(f"adjoint 1M vs the oracle: values {gv_err:.2e} of max; coordinates rel L2 {l2:.2e}, "
          f"max {worst:.2e} of max")
    assert worst_abs <= 1e-6
    assert worst_rel <= 1e-4
    assert gv_err <= 1e-12
    assert l2 <= 5e-8
    assert worst <= 2e-7
