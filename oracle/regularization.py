"""CPU restatement of the inversion pieces that consume the DC path (oracle only).

* WeightedLeastSquares (Smallness + SmoothnessFirstOrder, all cells active):
  ``simpeg/regularization/base.py:13-466, 758-1207, 1540-``;
  R = alpha_s diag(V) + sum_j alpha_j G_j^T diag(w_j) G_j, where G_j is the
  cell gradient on interior j-faces ((m_b - m_a) / centre distance; zero on
  boundary faces) and w_j the mean volume of the two cells of the face;
  alpha_j = (length_scale_j * smallest cell width)^2 with length_scale 1.
* L2DataMisfit: ``simpeg/data_misfit.py:238-343``.
* InexactGaussNewton direction with the UpdatePreconditioner Jacobi:
  ``simpeg/optimization.py:1345-1415``, ``simpeg/directives/_directives.py:2180-2260``.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _grad_1d(h):
    n = len(h)
    if n < 2:
        return sp.csr_matrix((0, n))
    d = 0.5 * (h[1:] + h[:-1])
    return sp.diags([-1.0 / d, 1.0 / d], [0, 1], shape=(n - 1, n), format="csr")


def _avg_1d(n):
    if n < 2:
        return sp.csr_matrix((0, n))
    return sp.diags([0.5 * np.ones(n - 1), 0.5 * np.ones(n - 1)], [0, 1], shape=(n - 1, n), format="csr")


def regularization_matrix(mesh, alpha_s=1.0):
    hx, hy, hz = [np.asarray(w, dtype=np.float64) for w in mesh.h]
    nx, ny, nz = len(hx), len(hy), len(hz)
    V = np.kron(hz, np.kron(hy, hx))
    base = min(hx.min(), hy.min(), hz.min())
    a = base ** 2
    Ix, Iy, Iz = sp.eye(nx), sp.eye(ny), sp.eye(nz)
    Gx = sp.kron(Iz, sp.kron(Iy, _grad_1d(hx)))
    Gy = sp.kron(Iz, sp.kron(_grad_1d(hy), Ix))
    Gz = sp.kron(_grad_1d(hz), sp.kron(Iy, Ix))
    Ax = sp.kron(Iz, sp.kron(Iy, _avg_1d(nx)))
    Ay = sp.kron(Iz, sp.kron(_avg_1d(ny), Ix))
    Az = sp.kron(_avg_1d(nz), sp.kron(Iy, Ix))
    R = alpha_s * sp.diags(V)
    for G, A in ((Gx, Ax), (Gy, Ay), (Gz, Az)):
        R = R + a * (G.T @ sp.diags(A @ V) @ G)
    return R.tocsr(), V, a


def gauss_newton_direction(orc, m, dobs, W, beta, R, cg_maxiter=10):
    """p = PCG(H, -g) with H v = 2 J^T W^2 J v + 2 beta R v, g = 2 J^T W^2 r + 2 beta R m."""
    orc.set_model(m)
    f = orc.fields()
    w2 = np.asarray(W) ** 2
    r = orc.dpred(f=f) - dobs
    g = 2 * orc.Jtvec(m, w2 * r, f=f) + 2 * beta * (R @ m)
    jtj = orc.getJtJdiag(m, W=sp.diags(np.asarray(W)), f=f)
    dA = jtj + beta * 2 * R.diagonal()
    Minv = np.where(dA != 0, 1.0 / np.where(dA != 0, dA, 1.0), 0.0)

    def H(v):
        return 2 * orc.Jtvec(m, w2 * orc.Jvec(m, v, f=f), f=f) + 2 * beta * (R @ v)

    b = -g
    x = np.zeros_like(b)
    res = b.copy()
    z = Minv * res
    p = z.copy()
    rz = res @ z
    for _ in range(cg_maxiter):
        q = H(p)
        alpha = rz / (p @ q)
        x = x + alpha * p
        res = res - alpha * q
        z = Minv * res
        rz_new = res @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, g, jtj
