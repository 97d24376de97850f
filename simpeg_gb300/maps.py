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

__all__ = ["IdentityMap", "ExpMap", "ReciprocalMap", "ComboMap", "InjectActiveCells"]


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

    def diag_deriv_dev(self, m):
        """Diagonal of d(map(m))/dm for a device (torch) model vector."""
        return m.new_ones(m.shape)

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

    def diag_deriv_dev(self, m):
        return m.exp()

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

    def diag_deriv_dev(self, m):
        return -1.0 / (m * m)

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
        """Diagonal of the derivative when every map in the chain has a diagonal one;
        NotImplementedError otherwise (the derivative is then ``deriv``)."""
        if not all(getattr(mp, "is_diagonal", True) for mp in self.maps):
            raise NotImplementedError("the chain contains a map without a diagonal derivative")
        x = np.asarray(m, dtype=np.float64).ravel()
        d = np.ones_like(x)
        for mp in reversed(self.maps):
            d = mp.diag_deriv(x) * d
            x = mp._transform(x)
        return d

    def diag_deriv_dev(self, m):
        """:meth:`diag_deriv` for a device model vector (chains of diagonal maps)."""
        if not self.is_diagonal:
            raise NotImplementedError("the chain contains a map without a diagonal derivative")
        d = m.new_ones(m.shape)
        for mp in reversed(self.maps):
            d = mp.diag_deriv_dev(m) * d
            m = mp.transform_dev(m)
        return d

    def deriv(self, m, v=None):
        """Chain rule with sparse matrices (any maps)."""
        if all(getattr(mp, "is_diagonal", True) for mp in self.maps):
            return super().deriv(m, v)
        x = np.asarray(m, dtype=np.float64).ravel()
        D = None
        for mp in reversed(self.maps):
            Dm = sp.csr_matrix(mp.deriv(x))
            D = Dm if D is None else (Dm @ D)
            x = mp._transform(x)
        return D @ v if v is not None else D

    @property
    def is_diagonal(self):
        return all(getattr(mp, "is_diagonal", True) for mp in self.maps)

    @property
    def is_linear(self):
        return all(m.is_linear for m in self.maps)


class InjectActiveCells(IdentityMap):
    """Model on the active cells, a fixed value on the others (``simpeg/maps/_injection.py``):
    ``out[active] = m``, ``out[~active] = value_inactive``; derivative the (nC, nActive)
    injection matrix.  Its derivative is not diagonal: a simulation applies it on the host."""

    is_diagonal = False

    def __init__(self, mesh, active_cells=None, value_inactive=0.0, **kwargs):
        nC = mesh.n_cells if hasattr(mesh, "n_cells") else int(mesh.nC)
        act = np.ones(nC, dtype=bool) if active_cells is None else np.asarray(active_cells)
        if act.dtype != bool:
            idx = act.astype(np.int64)
            act = np.zeros(nC, dtype=bool)
            act[idx] = True
        if act.size != nC:
            raise ValueError(f"active_cells has {act.size} entries, the mesh {nC} cells")
        self.active_cells = act
        self.nC = nC
        self.value_inactive = value_inactive
        self._P = sp.csr_matrix((np.ones(int(act.sum())), (np.flatnonzero(act), np.arange(int(act.sum())))),
                                shape=(nC, int(act.sum())))
        super().__init__(nP=int(act.sum()))

    @property
    def value_inactive(self):
        return self._value_inactive

    @value_inactive.setter
    def value_inactive(self, value):
        v = np.asarray(value, dtype=np.float64)
        n_inact = int((~self.active_cells).sum())
        if v.size not in (1, n_inact):
            raise ValueError("value_inactive must be a scalar or one value per inactive cell")
        self._value_inactive = np.broadcast_to(v.ravel(), (n_inact,)).copy()

    @property
    def shape(self):
        return (self.nC, self.nP)

    def _transform(self, m):
        out = np.empty(self.nC)
        out[self.active_cells] = np.asarray(m, dtype=np.float64).ravel()
        out[~self.active_cells] = self._value_inactive
        return out

    def transform_dev(self, m):
        import torch

        act = torch.as_tensor(self.active_cells, device=m.device)
        out = torch.empty(self.nC, dtype=m.dtype, device=m.device)
        out[act] = m
        out[~act] = torch.as_tensor(self._value_inactive, dtype=m.dtype, device=m.device)
        return out

    def diag_deriv(self, m):
        raise NotImplementedError("InjectActiveCells has no diagonal derivative")

    def deriv(self, m, v=None):
        return self._P @ v if v is not None else self._P

    def inverse(self, D):
        return np.asarray(D, dtype=np.float64).ravel()[self.active_cells]

    @property
    def is_linear(self):
        return True
