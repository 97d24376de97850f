"""DC receivers: potential (Pole) and potential-difference (Dipole) data.

Mirrors ``simpeg/electromagnetics/static/resistivity/receivers.py``:
``BaseRx.eval``/``evalDeriv`` (``:156-244``) project the nodal potential with
``P`` (``Dipole.getP`` = interp(M) - interp(N), ``:379-424``; ``Pole.getP`` =
interp(M), ``:461-498``) and divide by the geometric factor for
``data_type="apparent_resistivity"``.  On the GPU path ``P`` is never formed;
the projection is an electrode gather (see ``electrodes.py``).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

__all__ = ["BaseRx", "Pole", "Dipole"]

_VOLT = ("volt", "potential", "potentials", "v", "voltage", "voltages")
_APPRES = (
    "apparent_resistivity",
    "apparent resistivity",
    "appresistivity",
    "apparentresistivity",
    "apparent-resistivity",
)
_APPCHG = (
    "apparent_chargeability",
    "apparent chargeability",
    "appchargeability",
    "apparentchargeability",
    "apparent-chargeability",
)


def _loc2d(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a[None, :]
    if a.ndim != 2:
        raise ValueError("locations must be (n, dim)")
    return a


class BaseRx:
    def __init__(self, locations, data_type="volt", orientation=None, projField="phi",
                 storeProjections=False):
        self.locations = locations
        self.data_type = data_type
        if orientation is not None:
            raise NotImplementedError("only potential (phi) receivers are on the GPU path")
        self.orientation = None
        if projField != "phi":
            raise NotImplementedError("only projField='phi' is on the GPU path")
        self.projField = "phi"
        self.storeProjections = storeProjections
        self._geometric_factor = {}
        self._Ps = {}

    @property
    def data_type(self):
        return self._data_type

    @data_type.setter
    def data_type(self, var):
        v = str(var).lower()
        if v in _VOLT:
            self._data_type = "volt"
        elif v in _APPRES:
            self._data_type = "apparent_resistivity"
        elif v in _APPCHG:
            self._data_type = "apparent_chargeability"
        else:
            raise ValueError(f"data_type {var!r} not in volt / apparent_resistivity / apparent_chargeability")

    @property
    def geometric_factor(self):
        return self._geometric_factor

    # ------------------------------------------------------------ host projections
    def getP(self, mesh, projected_grid="N", transpose=False):
        """(nD, nN) interpolation of the potential at the receiver electrodes
        (``receivers.py:379-424,461-498``): the trilinear node weights of M, minus those of
        N for a dipole.  Only nodal potentials (``projected_grid`` "N") are on this path;
        the simulation itself uses the same weights as device tables."""
        if projected_grid not in ("N", "nodes"):
            raise NotImplementedError("only nodal potentials ('N') are on the GPU path")
        from .electrodes import rx_projection

        P = self._Ps.get(id(mesh)) if self.storeProjections else None
        if P is None:
            P = rx_projection(mesh, self)
            if self.storeProjections:
                self._Ps[id(mesh)] = P
        return P.toarray().T if transpose else P

    def _factor(self, src):
        if self.data_type != "apparent_resistivity":
            return None
        try:
            return 1.0 / np.asarray(self.geometric_factor[src], dtype=np.float64)
        except KeyError:
            raise KeyError(
                "Receiver geometric factor has not been set, please execute survey.set_geometric_factor()")

    def eval(self, src, mesh, f):
        """Data of this receiver for source ``src`` from the fields ``f`` (``receivers.py:156-192``):
        ``P phi``, divided by the geometric factor for apparent resistivity."""
        v = self.getP(mesh) @ np.asarray(f[src, "phiSolution"])
        fac = self._factor(src)
        return v if fac is None else fac * v

    def evalDeriv(self, src, mesh, f, v=None, adjoint=False):
        """Derivative of ``eval`` with respect to the potential (``receivers.py:194-244``): the
        (scaled) projection itself when ``v`` is None (its transpose with ``adjoint``), else its
        product with ``v``."""
        P = self.getP(mesh)
        fac = self._factor(src)
        if v is None:
            if fac is not None:
                P = sp.diags(fac) @ P
            return P.T if adjoint else P
        if not adjoint:
            out = P @ v
            return out if fac is None else fac * out
        if fac is not None:
            v = fac * v
        return P.T @ v


class Pole(BaseRx):
    """Potential at electrode M."""

    def __init__(self, locations, **kwargs):
        super().__init__(locations=locations, **kwargs)

    @property
    def locations(self):
        return self._locations

    @locations.setter
    def locations(self, value):
        self._locations = _loc2d(value)

    @property
    def nD(self):
        return self._locations.shape[0]

    @property
    def locations_m(self):
        return self._locations

    @property
    def locations_n(self):
        return None


class Dipole(BaseRx):
    """Potential difference between electrodes M and N."""

    def __init__(self, locations_m=None, locations_n=None, locations=None, **kwargs):
        if locations_m is not None or locations_n is not None:
            if locations_n is None or locations_m is None:
                raise ValueError("For a dipole receiver both locations_m and locations_n must be set")
            if locations is not None:
                raise ValueError(
                    "Cannot set both locations and locations_m, locations_n. Please provide "
                    "either locations=(locations_m, locations_n) or both locations_m, locations_n"
                )
            locations = [locations_m, locations_n]
        if locations is None:
            raise AttributeError("Receiver cannot be instantiated without assigning 'locations'.")
        kwargs.pop("threshold", None)
        super().__init__(locations=locations, **kwargs)

    @property
    def locations(self):
        return self._locations

    @locations.setter
    def locations(self, locs):
        if len(locs) != 2:
            raise ValueError(
                "locations must be a list or tuple of length 2: [locations_m, locations_n]. "
                f"The input locations has length {len(locs)}"
            )
        m, n = _loc2d(locs[0]), _loc2d(locs[1])
        if m.shape != n.shape:
            raise ValueError(
                f"locations_m (shape: {m.shape}) and locations_n (shape: {n.shape}) need to be the same size"
            )
        self._locations = [m, n]

    @property
    def locations_m(self):
        return self._locations[0]

    @property
    def locations_n(self):
        return self._locations[1]

    @property
    def nD(self):
        return self._locations[0].shape[0]
