"""GPU ``Simulation3DNodal`` and ``Simulation3DCellCentered`` for induced polarization.

Drop-in for ``simpeg.electromagnetics.static.induced_polarization.Simulation3DNodal``
(``simpeg/electromagnetics/static/induced_polarization/simulation.py:15-167``).
The IP data are the linearised DC response to a chargeability model eta at a
fixed conductivity sigma:

* ``sigmaDeriv = -diag(sigma) etaDeriv`` (``simulation.py:36-38``), so every
  sensitivity product is the DC one (matrix-free stencil, multigrid-PCG solves
  on the GPU) with that derivative;
* ``Jvec = scale * DC Jvec``, ``Jtvec = DC Jtvec(scale * v)`` (``:126-134``),
  where ``scale`` is 1 / (DC voltage) for ``apparent_chargeability`` data and
  1 otherwise (``_scale``, ``:44-61``);
* ``dpred(m) = forward(m) = Jvec(m, m)`` (``:89-112,129-130``);
* ``getJtJdiag`` with the weights ``scale^2`` (times ``W^2``) (``:114-124``),
  evaluated by electrode reciprocity without forming J.

The DC fields at sigma are solved once and kept (or taken from ``_f``): a
model update changes nothing on the device (the reference's
``_delete_on_model_update`` is empty, ``:136-139``).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from ..maps import IdentityMap
from ..resistivity.simulation import Simulation3DNodal as _DCSimulation3DNodal
from ..resistivity.simulation_cc import Simulation3DCellCentered as _DCSimulation3DCellCentered

__all__ = ["Simulation3DNodal", "Simulation3DCellCentered"]


class _Weights:
    def __init__(self, w):
        self._w = np.asarray(w, dtype=np.float64)

    def diagonal(self):
        return self._w


class Simulation3DNodal(_DCSimulation3DNodal):
    """3D nodal IP problem on a tensor mesh, solved on the GPU.

    ``Ainv`` (a DC simulation's factorisation in the reference) is accepted and
    not needed: there is no factorisation to share.  ``_f`` may be the
    :class:`~simpeg_gb300.resistivity.Fields3DNodal` of a DC simulation at the
    same conductivity (with the same survey and mesh).  The remaining keyword
    arguments are those of the DC simulation (``precision``, ``rtol``, ...)."""

    def __init__(self, mesh, survey=None, sigma=None, rho=None, eta=None, etaMap=None, Ainv=None, _f=None,
                 **kwargs):
        for k in ("sigmaMap", "rhoMap"):
            if kwargs.pop(k, None) is not None:
                raise TypeError(f"{k} is fixed to the identity in an IP simulation")
        if sigma is None and rho is None:
            raise ValueError("an IP simulation needs the conductivity sigma (or resistivity rho)")
        super().__init__(mesh, survey=survey, sigma=sigma, rho=rho, **kwargs)
        self._eta = None if eta is None else np.asarray(eta, dtype=np.float64)
        self.etaMap = etaMap
        self._f = _f
        self._scale_dev = None
        self._pred = None

    # ------------------------------------------------------------ properties
    @property
    def eta(self):
        if self._eta is not None:
            return self._eta
        if self.etaMap is None:
            raise AttributeError("Neither a value nor mapping for eta has been set")
        if self._model is None:
            raise AttributeError("A `model` is required for physical property eta")
        return self.etaMap * self._model

    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, m):
        # the IP forward is linear in eta: fields, J and its diagonal do not depend on the model
        if m is None:
            self._model = None
            return
        m = np.asarray(m, dtype=np.float64).ravel()
        nP = getattr(self.etaMap, "nP", "*") if self.etaMap is not None else "*"
        if isinstance(nP, (int, np.integer)) and m.size != nP:
            raise ValueError(f"model must have {nP} parameters, got {m.size}")
        if self._model is not None and self._model.shape == m.shape and np.array_equal(self._model, m):
            return
        self._model = m.copy()
        self._dsig_cache = None

    def _sigma_deriv(self):
        """Diagonal of d sigma / d m = -sigma * d eta / d m (``simulation.py:36-38``)."""
        mp = self.etaMap if self.etaMap is not None else IdentityMap()
        s = self.sigma
        if hasattr(mp, "diag_deriv") and getattr(mp, "is_diagonal", True):
            m = self._model if self._model is not None else np.zeros(self.nC)
            return -s * mp.diag_deriv(m)
        D = mp.deriv(self._model)
        if sp.issparse(D):
            D = D.tocsr()
            if D.shape[0] == D.shape[1] and D.nnz == np.count_nonzero(D.diagonal()):
                return -s * np.asarray(D.diagonal(), dtype=np.float64)
        return sp.diags(-s) @ D

    # ------------------------------------------------------------ DC fields and the data scale
    def _dc_fields(self):
        if self._f is None:
            self._ensure_model()
            self._f = _DCSimulation3DNodal.fields(self, None)
        return self._f

    def _fields_for(self, m, f):
        return f if f is not None else self._dc_fields()

    @property
    def _scale(self):
        """1 / (DC voltage) for apparent-chargeability data, 1 otherwise (``simulation.py:44-61``)."""
        return self._scale_t().cpu().numpy()

    def _scale_t(self):
        if self._scale_dev is None:
            nD = self.survey.nD
            is_chg = np.zeros(nD, dtype=bool)
            i0 = 0
            for src in self.survey.source_list:
                for rx in src.receiver_list:
                    if rx.data_type == "apparent_chargeability":
                        is_chg[i0:i0 + rx.nD] = True
                    i0 += rx.nD
            scale = np.ones(nD)
            if is_chg.any():
                f = self._dc_fields()
                d = self._mini_survey_data(self._gather(f.phi_dev).cpu().numpy())
                scale[is_chg] = 1.0 / d[is_chg]
            self._scale_dev = torch.from_numpy(scale).to(self.device)
        return self._scale_dev

    # ------------------------------------------------------------ simulation API
    def fields(self, m=None, calcJ=True):
        """DC fields at sigma (solved once) and the IP prediction at m (``simulation.py:89-97``)."""
        f = self._dc_fields()
        if m is not None:
            self._pred = self.forward(m, f=f)
        return f

    def forward(self, m, f=None):
        return np.asarray(self.Jvec(m, m, f=f))

    def dpred(self, m=None, f=None):
        """IP data at m (``simulation.py:99-112``).  With ``f`` given, the prediction is
        evaluated with those fields (the reference returns the prediction of its last
        ``fields`` call instead)."""
        if m is None:
            m = self.model
        if f is None:
            self.fields(m)
            return self._pred
        return self.forward(m, f=f)

    def Jvec(self, m, v, f=None):
        return self._scale * super().Jvec(m, v, f=f)

    def Jtvec(self, m, v, f=None):
        if hasattr(v, "dobs"):
            v = v.dobs
        return super().Jtvec(m, np.asarray(v, dtype=np.float64) * self._scale, f=f)

    def getJtJdiag(self, m, W=None, f=None):
        """diag(J^T diag(scale W)^2 J) (``simulation.py:114-124``), by electrode reciprocity."""
        if self._gtgdiag is None:
            w = self._scale if W is None else self._scale * np.asarray(W.diagonal(), dtype=np.float64)
            self._gtgdiag = super().getJtJdiag(m, W=_Weights(w), f=f)
        return self._gtgdiag

    # ------------------------------------------------------------ device-resident products
    def jvec_dev(self, v_dev, f=None):
        return self._scale_t() * super().jvec_dev(v_dev, f=f)

    def jtvec_dev(self, w_dev, f=None):
        return super().jtvec_dev(self._scale_t() * w_dev, f=f)


class Simulation3DCellCentered(Simulation3DNodal, _DCSimulation3DCellCentered):
    """3D cell-centred IP problem on a tensor mesh, solved on the GPU
    (``induced_polarization/simulation.py:160-163``): the IP logic of
    :class:`Simulation3DNodal` on the cell-centred DC operator, whose property is the
    resistivity: ``rhoDeriv = diag(rho) etaDeriv`` (``simulation.py:40-42``)."""

    def _sigma_deriv(self):
        """d rho / d m = rho * d eta / d m."""
        mp = self.etaMap if self.etaMap is not None else IdentityMap()
        r = 1.0 / np.asarray(self.sigma, dtype=np.float64)
        if hasattr(mp, "diag_deriv") and getattr(mp, "is_diagonal", True):
            m = self._model if self._model is not None else np.zeros(self.nC)
            return r * mp.diag_deriv(m)
        D = mp.deriv(self._model)
        if sp.issparse(D):
            D = D.tocsr()
            if D.shape[0] == D.shape[1] and D.nnz == np.count_nonzero(D.diagonal()):
                return r * np.asarray(D.diagonal(), dtype=np.float64)
        return sp.diags(r) @ D

    def _dc_fields(self):
        if self._f is None:
            self._ensure_model()
            self._f = _DCSimulation3DCellCentered.fields(self, None)
        return self._f
