"""GPUSolver (the simpeg Solver plug-in) against SciPy SuperLU on assembled DC matrices."""

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle.dc3d import OracleDC3DNodal
from simpeg_gb300.mesh import TensorMesh
from simpeg_gb300.resistivity import sources
from simpeg_gb300.resistivity.survey import Survey

pytestmark = pytest.mark.gpu


def _A(seed=0):
    mesh = TensorMesh([[(10.0, 2, -1.3), (10.0, 8), (10.0, 2, 1.3)], [(10.0, 9)], [(10.0, 2, -1.3), (10.0, 6)]],
                      origin="CCN")
    rng = np.random.default_rng(seed)
    o = OracleDC3DNodal(mesh, Survey([sources.Pole([], np.r_[0.0, 0.0, 0.0])]),
                        sigma=10 ** rng.uniform(-3, -1, mesh.n_cells))
    return o.getA()


@pytest.mark.parametrize("k", [1, 3, 40])
def test_gpu_solver_matches_superlu(cuda, k):
    from simpeg_gb300.solver import GPUSolver

    A = _A()
    rng = np.random.default_rng(1)
    B = rng.standard_normal((A.shape[0], k))
    Ainv = GPUSolver(A, rtol=1e-12)
    X = Ainv * (B[:, 0] if k == 1 else B)
    X0 = spla.splu(A.tocsc()).solve(B)
    if k == 1:
        X0 = X0[:, 0]
    assert np.linalg.norm(X - X0) / np.linalg.norm(X0) < 1e-9
    Ainv.clean()


def test_gpu_solver_api_and_errors(cuda):
    from simpeg_gb300.solver import GPUSolver, get_default_solver, set_default_solver

    A = _A(1)
    s = GPUSolver(A)
    assert s.shape == A.shape and s.T is s
    with pytest.raises(ValueError):
        s * np.ones(A.shape[0] + 1)
    with pytest.raises(NotImplementedError):
        GPUSolver(A + 0.5 * __import__("scipy.sparse", fromlist=["eye"]).eye(A.shape[0], k=1))
    assert get_default_solver() is GPUSolver
    with pytest.raises(TypeError):
        set_default_solver(object)
