"""Accurate FP64 forward of the MLS transfer with frozen connectivity, in numpy
(scaled moments, direct solve), for central finite-difference checks of the
adjoint.  Test helper, not part of the product."""
import numpy as np

RBF = {
    1: (lambda x: (1 - x) ** 4 * (4 * x + 1)),            # Wendland<2>
    2: (lambda x: (1 - x) ** 6 * (35 * x * x + 18 * x + 3)),  # Wendland<4>
}


def basis(X, basis_id):
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    one = np.ones_like(x)
    if basis_id == 0:
        return one[..., None]
    if basis_id == 1:
        return np.stack([one, x, y, z], -1)
    return np.stack([one, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z], -1)


def forward(src, tgt, idx, k, values, rbf_id, basis_id):
    """Target values for rows of exactly k neighbours idx (n_t*k,)."""
    n_t = len(tgt)
    X = src[idx].reshape(n_t, k, 3) - tgt[:, None, :]
    rho = np.sqrt((X ** 2).sum(-1))
    R = 1.1 * np.maximum(10 * np.finfo(float).eps, rho.max(1))
    Xh = X / R[:, None, None]
    phi = RBF[rbf_id](rho / R[:, None])
    P = basis(Xh, basis_id)
    A = np.einsum('tk,tka,tkb->tab', phi, P, P)
    e0 = np.zeros((n_t, P.shape[-1], 1))
    e0[:, 0, 0] = 1.0
    a = np.linalg.solve(A, e0)[..., 0]
    c = phi * np.einsum('tka,ta->tk', P, a)
    return (c * values[idx].reshape(n_t, k)).sum(1)


def loss(src, tgt, idx, k, values, g, rbf_id, basis_id):
    y = forward(src, tgt, idx, k, values, rbf_id, basis_id)
    return 0.5 * float(((y - g) ** 2).sum())


def fd_coord_directional(src, tgt, idx, k, values, g, rbf_id, basis_id, d, h=1e-6):
    lp = loss(src + h * d, tgt, idx, k, values, g, rbf_id, basis_id)
    lm = loss(src - h * d, tgt, idx, k, values, g, rbf_id, basis_id)
    return (lp - lm) / (2 * h)
