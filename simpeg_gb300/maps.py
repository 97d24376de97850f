"""Model -> conductivity maps used on the DC path.

Mirrors the maps the reference path uses (``simpeg/maps/_base.py`` IdentityMap,
``simpeg/maps/_property_maps.py:18-112`` ExpMap, ReciprocalMap, and ``map * map``
composition).  Every map here has a diagonal derivative, which is what the GPU
sensitivity kernels consume (``sigmaDeriv`` enters ``getADeriv`` only as
``diag(dsigma/dm)``).  Maps from an installed simpeg are also accepted by the
simulation: their ``deriv`` is then applied on the host as a sparse matrix.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

__all__ = ["IdentityMap", "ExpMap", "ReciprocalMap", "ComboMap"]


class IdentityMap:
    def __init__(self, mesh=None, nP=None, **kwargs):
        if nP is None and mesh is not None:
            nP = mesh.n_cells if hasattr(mesh, "n_cells") else int(mesh.nC)
        self._nP = nP

    @property
    def nP(self):
        return self._nP if self._nP is not None else "*"

    @property
    def shape(self):
        return (self.nP, self.nP)

    def _transform(self, m):
        return np.asarray(m, dtype=np.float64).ravel()

    def transform_dev(self, m):
        """The map applied to a device (torch) model vector, elementwise."""
        return m

    def diag_deriv(self, m):
        """Diagonal of d(map(m))/dm."""
        return np.ones(np.asarray(m).size)

    def deriv(self, m, v=None):
        d = sp.diags(self.diag_deriv(m))
        return d @ v if v is not None else d

    def inverse(self, D):
        return np.asarray(D, dtype=np.float64).ravel()

    def _check(self, m):
        m = np.asarray(m, dtype=np.float64).ravel()
        if isinstance(self.nP, int) and m.size != self.nP:
            raise ValueError(f"model has {m.size} entries, map expects {self.nP}")
        return m

    def __mul__(self, other):
        if isinstance(other, IdentityMap):
            return ComboMap([self, other])
        return self._transform(self._check(other))

    def __rmul__(self, other):
        raise TypeError("maps apply from the left: use map * m")

    @property
    def is_linear(self):
        return True


class ExpMap(IdentityMap):
    """sigma = exp(m) (natural log model); derivative diag(exp(m))."""

    def _transform(self, m):
        return np.exp(np.asarray(m, dtype=np.float64).ravel())

    def transform_dev(self, m):
        return m.exp()

    def diag_deriv(self, m):
        return np.exp(np.asarray(m, dtype=np.float64).ravel())

    def inverse(self, D):
        return np.log(np.asarray(D, dtype=np.float64).ravel())

    @property
    def is_linear(self):
        return False


class ReciprocalMap(IdentityMap):
    """sigma = 1/m; derivative diag(-1/m**2)."""

    def _transform(self, m):
        return 1.0 / np.asarray(m, dtype=np.float64).ravel()

    def transform_dev(self, m):
        return 1.0 / m

    def diag_deriv(self, m):
        m = np.asarray(m, dtype=np.float64).ravel()
        return -1.0 / m**2

    def inverse(self, D):
        return 1.0 / np.asarray(D, dtype=np.float64).ravel()

    @property
    def is_linear(self):
        return False


class ComboMap(IdentityMap):
    """maps[0] * maps[1] * ... applied right to left; derivative by the chain rule."""

    def __init__(self, maps):
        flat = []
        for m in maps:
            flat.extend(m.maps if isinstance(m, ComboMap) else [m])
        self.maps = flat
        nPs = [m.nP for m in flat if isinstance(m.nP, int)]
        super().__init__(nP=nPs[-1] if nPs else None)

    def _transform(self, m):
        x = np.asarray(m, dtype=np.float64).ravel()
        for mp in reversed(self.maps):
            x = mp._transform(x)
        return x

    def transform_dev(self, m):
        for mp in reversed(self.maps):
            m = mp.transform_dev(m)
        return m

    def diag_deriv(self, m):
        x = np.asarray(m, dtype=np.float64).ravel()
        d = np.ones_like(x)
        for mp in reversed(self.maps):
            d = mp.diag_deriv(x) * d
            x = mp._transform(x)
        return d

    @property
    def is_linear(self):
        return all(m.is_linear for m in self.maps)
