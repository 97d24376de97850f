"""CPU restatement of the nodal IP simulation (oracle only -- test infrastructure).

Follows ``simpeg/electromagnetics/static/induced_polarization/simulation.py``:

* ``sigmaDeriv = -diag(sigma) etaDeriv``            ``simulation.py:36-38``
* ``_scale`` (1 / DC voltage for apparent-chargeability data)  ``:44-61``
* ``fields`` / ``dpred`` / ``forward = Jvec(m, m)``  ``:89-112,129-130``
* ``Jvec = scale * DC Jvec``, ``Jtvec = DC Jtvec(scale * v)``  ``:126-134``
* ``getJtJdiag`` from J with weights ``scale^2`` (times ``W^2``)  ``:114-124``

on top of the DC oracle (``oracle/dc3d.py``, and ``oracle/cc3d.py`` for the
cell-centred form) at the fixed conductivity.
"""

from __future__ import annotations

import numpy as np

from .dc3d import OracleDC3DNodal


class OracleIP3DNodal(OracleDC3DNodal):
    """IP data as the linearised DC response to eta at fixed sigma (direct solves)."""

    def __init__(self, mesh, survey, sigma, eta_map=None, **kwargs):
        super().__init__(mesh, survey, sigma=sigma, **kwargs)
        self.eta_map = eta_map
        self._f = None

    def set_model(self, m):
        # A depends on sigma only: keep the factorisation across model updates
        self.model = None if m is None else np.asarray(m, dtype=np.float64).ravel()

    def sigma_deriv_diag(self):
        de = np.ones(self.ops.nC) if self.eta_map is None else self.eta_map.diag_deriv(self.model)
        return -self._sigma_fixed * de

    def dc_fields(self):
        if self._f is None:
            self._f = self._solve(self.getRHS())
        return self._f

    def scale(self):
        f = self.dc_fields()
        out = []
        for i, src in enumerate(self.survey.source_list):
            for rx in src.receiver_list:
                if rx.data_type == "apparent_chargeability":
                    P = self._rx_P(rx)
                    out.append(1.0 / (P @ f[:, i]))
                else:
                    out.append(np.ones(rx.nD))
        return np.hstack(out)

    def _rx_P(self, rx):
        from .dc3d import _rx_projection

        return _rx_projection(self.ops, rx)

    def Jvec(self, m, v, f=None):
        self.set_model(m)
        return self.scale() * super().Jvec(m, v, f=self.dc_fields())

    def Jtvec(self, m, v, f=None):
        self.set_model(m)
        return super().Jtvec(m, self.scale() * np.asarray(v, dtype=np.float64), f=self.dc_fields())

    def dpred(self, m=None, f=None):
        return self.Jvec(m, m)

    def getJtJdiag(self, m, W=None, f=None):
        self.set_model(m)
        J = self.getJ(m, f=self.dc_fields())
        w = self.scale() if W is None else self.scale() * np.asarray(W, dtype=np.float64)
        return ((w ** 2)[:, None] * J * J).sum(axis=0)


from .cc3d import OracleDC3DCellCentered  # noqa: E402


class OracleIP3DCellCentered(OracleDC3DCellCentered):
    """Cell-centred IP (``induced_polarization/simulation.py:160-163``): the linearised cell-centred
    DC response at fixed sigma with ``rhoDeriv = diag(rho) etaDeriv`` (``simulation.py:40-42``)."""

    def __init__(self, mesh, survey, sigma, eta_map=None, **kwargs):
        super().__init__(mesh, survey, sigma=sigma, **kwargs)
        self.eta_map = eta_map
        self._f = None

    def set_model(self, m):
        self.model = None if m is None else np.asarray(m, dtype=np.float64).ravel()

    def rho_deriv_diag(self):
        de = np.ones(self.ops.nC) if self.eta_map is None else self.eta_map.diag_deriv(self.model)
        return self._rho_fixed * de

    def dc_fields(self):
        if self._f is None:
            self._f = self._solve(self.getRHS())
        return self._f

    def scale(self):
        """1 / (DC voltage) for apparent-chargeability data, 1 otherwise, per receiver in survey order."""
        f = self.dc_fields()
        out = []
        k = 0
        projs = self._projections()
        for src in self.survey.source_list:
            for rx in src.receiver_list:
                i, P, _ = projs[k]
                k += 1
                if rx.data_type == "apparent_chargeability":
                    out.append(1.0 / (P @ f[:, i]))
                else:
                    out.append(np.ones(rx.nD))
        return np.hstack(out)

    def Jvec(self, m, v, f=None):
        self.set_model(m)
        return self.scale() * super().Jvec(m, v, f=self.dc_fields())

    def Jtvec(self, m, v, f=None):
        self.set_model(m)
        return super().Jtvec(m, self.scale() * np.asarray(v, dtype=np.float64), f=self.dc_fields())

    def dpred(self, m=None, f=None):
        return self.Jvec(m, m)
