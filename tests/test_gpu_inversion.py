"""Inversion pieces on the GPU vs the CPU oracle: regulariser apply, misfit
gradient, JtJ diagonal and a 10-iteration inexact Gauss-Newton direction."""

import numpy as np
import pytest

from oracle.dc3d import OracleDC3DNodal
from oracle.regularization import gauss_newton_direction, regularization_matrix
from simpeg_gb300 import maps
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import Simulation3DNodal, receivers, sources
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu


def _case():
    mesh = TensorMesh([[(10.0, 3, -1.3), (10.0, 10), (10.0, 3, 1.3)], [(10.0, 3, -1.3), (10.0, 8), (10.0, 3, 1.3)],
                       [(10.0, 3, -1.3), (10.0, 6)]], origin="CCN")
    xs = np.arange(-40.0, 41.0, 10.0)
    srcs = []
    for i in range(4):
        M = np.c_[xs[i + 2:i + 5], np.zeros(3), np.zeros(3)]
        N = np.c_[xs[i + 3:i + 6], np.zeros(3), np.zeros(3)]
        srcs.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[xs[i], 0, 0], np.r_[xs[i + 1], 0, 0]))
    survey = Survey(srcs)
    rng = np.random.default_rng(4)
    m_true = np.log(10 ** rng.uniform(-2.5, -1.5, mesh.n_cells))
    m0 = np.full(mesh.n_cells, np.log(10 ** -2.0))
    return mesh, survey, m_true, m0, rng


def test_regulariser_apply_matches_oracle(cuda):
    import torch

    from simpeg_gb300.inversion import WeightedLeastSquares

    mesh, survey, m_true, m0, rng = _case()
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh))
    reg = WeightedLeastSquares(mesh, sim)
    R, V, a = regularization_matrix(mesh)
    v = rng.standard_normal(mesh.n_cells)
    out = reg.R(torch.from_numpy(v).cuda()).cpu().numpy()
    np.testing.assert_allclose(out, R @ v, rtol=1e-12, atol=1e-12 * np.abs(R @ v).max())
    np.testing.assert_allclose(reg.diag_deriv2().cpu().numpy(), 2 * R.diagonal(), rtol=1e-12)
    assert np.isclose(reg.alpha_x, a)


def test_gauss_newton_direction_matches_oracle(cuda):
    import torch

    from simpeg_gb300.inversion import L2DataMisfit, WeightedLeastSquares, inexact_gauss_newton_direction

    mesh, survey, m_true, m0, rng = _case()
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m_true)
    dobs = orc.dpred()
    W = 1.0 / (0.05 * np.abs(dobs) + 1e-6)
    beta = 1e-2
    R, _, _ = regularization_matrix(mesh)
    p0, g0, jtj0 = gauss_newton_direction(orc, m0, dobs, W, beta, R, cg_maxiter=10)
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    dmis = L2DataMisfit(sim, dobs, W=W)
    reg = WeightedLeastSquares(mesh, sim)
    p, info = inexact_gauss_newton_direction(dmis, reg, beta, m0, cg_maxiter=10)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(info["g"].cpu().numpy(), g0) < 1e-6
    assert rel(info["jtj_diag"].cpu().numpy(), jtj0) < 1e-6
    assert rel(p.cpu().numpy(), p0) < 1e-6


def test_inexact_gauss_newton_minimiser(cuda):
    """The minimiser on the DC problem: with the UpdatePreconditioner Jacobi and 10 CG iterations its
    first search direction is the Gauss-Newton direction above, and three iterations with the Armijo
    line search decrease phi = phi_d + beta phi_m at every step."""
    from simpeg_gb300.inversion import (BaseInvProblem, InexactGaussNewton, L2DataMisfit, WeightedLeastSquares,
                                        inexact_gauss_newton_direction, jacobi_preconditioner)

    mesh, survey, m_true, m0, rng = _case()
    orc = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    orc.set_model(m_true)
    dobs = orc.dpred()
    W = 1.0 / (0.05 * np.abs(dobs) + 1e-6)
    beta = 1e-2
    sim = Simulation3DNodal(mesh, survey=survey, sigmaMap=maps.ExpMap(mesh), rtol=1e-11)
    dmis = L2DataMisfit(sim, dobs, W=W)
    reg = WeightedLeastSquares(mesh, sim)
    p_ref, _ = inexact_gauss_newton_direction(dmis, reg, beta, m0, cg_maxiter=10)
    prob = BaseInvProblem(dmis, reg, beta)
    opt = InexactGaussNewton(maxIter=1, cg_maxiter=10, cg_rtol=0.0,
                             approxHinv=jacobi_preconditioner(dmis, reg, beta, m0))
    opt.minimize(prob.evalFunction, m0)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(opt.searchDirection.cpu().numpy(), p_ref.cpu().numpy()) < 1e-10
    opt = InexactGaussNewton(maxIter=3, cg_maxiter=5, approxHinv=jacobi_preconditioner(dmis, reg, beta, m0))
    opt.remember("f")
    m = opt.minimize(prob.evalFunction, m0)
    f = opt.recall("f") + [prob.evalFunction(m, return_g=False, return_H=False)]
    assert all(b < a for a, b in zip(f, f[1:])), f
