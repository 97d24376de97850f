"""GPU ``Simulation3DCellCentered``: simpeg's cell-centred DC forward/sensitivity API on the CUDA engine.

Drop-in for ``simpeg.electromagnetics.static.resistivity.Simulation3DCellCentered``
(``simpeg/electromagnetics/static/resistivity/simulation.py:321-480``): the same
constructor arguments (``bc_type`` "Dirichlet", "Neumann", "Robin" or "Mixed"),
the same ``fields / dpred / Jvec / Jtvec / getJ / getJtJdiag / getA / getADeriv``
signatures and data ordering as the nodal simulation it shares its plumbing
with.  The unknowns are the cell-centre potentials; ``A = Div MfRhoI Grad`` is
never assembled: it is a seven-point stencil on the grid of cell centres
(``dc_set_model_cc``) solved by the same multigrid-PCG engine, sources sit at
the nearest cell centre (``sources.py:79-81``) and receivers interpolate from
the cell centres (``receivers.py:414``).  The operator depends on the
resistivity, so the model derivative handed to the kernels is ``d rho / d m``
(``rhoMap``'s derivative, or ``-sigma' / sigma^2`` through ``sigmaMap``).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from ..engine import CCEngine
from .fields import Fields3DCellCentered
from .simulation import Simulation3DNodal

__all__ = ["Simulation3DCellCentered"]


class Simulation3DCellCentered(Simulation3DNodal):
    """3D cell-centred DC problem on a tensor mesh, solved on the GPU.

    Extra keyword arguments as :class:`Simulation3DNodal` (``precision``, ``rtol``,
    ``maxit``, ``device``, ``engine_opts``)."""

    _solutionType = "phiSolution"
    _formulation = "HJ"
    fieldsPair = Fields3DCellCentered
    _grid = "CC"
    _bc_types = ("Robin", "Neumann", "Dirichlet")

    def _make_engine(self, eo):
        # Neumann: the engine reproduces the reference's row-0 pin (simulation.py:365-373)
        return CCEngine(self.mesh, self.bc_type, self.surface_faces, **eo)

    def _engine_set_property(self, sigma_dev):
        """The operator is built from the resistivity."""
        self.engine.set_model(1.0 / sigma_dev)

    def _sigma_deriv(self):
        """d rho / d m (diagonal as an array, else sparse): -diag(1 / sigma^2) d sigma / d m."""
        d = super()._sigma_deriv()
        if d is None:
            return None
        s = np.asarray(self.sigma, dtype=np.float64)
        if isinstance(d, np.ndarray):
            return -d / (s * s)
        return (sp.diags(-1.0 / (s * s)) @ d).tocsr()

    def _property_deriv_dev(self, d_sigma_dev):
        rho = self.engine.rho
        return -d_sigma_dev * rho * rho

    @property
    def rhoDeriv(self):
        d = self._sigma_deriv()
        if d is None:
            return None
        return sp.diags(d) if isinstance(d, np.ndarray) else d

    def _jtj_diag_reciprocity(self, w):
        return None  # the electrode-reciprocity kernel is nodal: getJtJdiag forms J

    def getJtJdiag(self, m, W=None, f=None):
        """diag(J^T W^T W J) (``simulation.py:137-154``) from the batched-adjoint J."""
        return super().getJtJdiag(m, W=W, f=f)
