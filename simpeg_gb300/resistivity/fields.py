"""Device-backed ``Fields3DNodal``.

Mirrors ``simpeg/electromagnetics/static/resistivity/fields.py:186-257`` and
the ``Fields`` store of ``simpeg/fields.py:7-345``: the nodal potential of
every source, indexed ``f[src, "phiSolution"]`` / ``f[:, "phi"]``, and the
fields derived from it on request: ``e = -G phi`` and ``j = MeI MeSigma e`` on
the edges, ``charge`` on the nodes and ``charge_density`` on the cells
(``dc_edge_fields`` / ``dc_node_charge`` kernels).  The store stays on the GPU
as a ``(nSrc, nN)`` float64 tensor (column-major (nN, nSrc)); indexing copies
the requested columns to the host as numpy arrays.
"""

from __future__ import annotations

import numpy as np


_DERIVED = ("e", "j", "charge", "charge_density")


class Fields3DNodal:
    knownFields = {"phiSolution": "N"}
    aliasFields = {
        "phi": ["phiSolution", "N", "_phi"],
        "j": ["phiSolution", "E", "_j"],
        "e": ["phiSolution", "E", "_e"],
        "charge_density": ["phiSolution", "CC", "_charge_density"],
        "charge": ["phiSolution", "N", "_charge"],
    }

    def __init__(self, simulation, phi_dev):
        self.simulation = simulation
        self.phi_dev = phi_dev

    @property
    def survey(self):
        sim = self.simulation
        return sim._mini_survey if sim._mini_survey is not None else sim.survey

    def _src_index(self, src):
        sl = self.survey.source_list
        if isinstance(src, slice):
            return list(range(len(sl)))[src]
        if isinstance(src, (list, tuple)):
            return [self._src_index(s) for s in src]
        for i, s in enumerate(sl):
            if s is src:
                return i
        raise KeyError("source is not part of the survey")

    def _GLoc(self, fieldType):
        """Grid location of a field (``fields.py:205-211``)."""
        if fieldType == "phi":
            return "N"
        if fieldType in ("e", "j"):
            return "E"
        raise KeyError("Field type must be phi, e, j")

    def _derived(self, idx, name):
        """Derived field of the sources idx (list) on the device, (len(idx), n) (``fields.py:214-253``)."""
        from scipy.constants import epsilon_0

        eng = self.simulation.engine
        phi = self.phi_dev[idx]
        if name in ("e", "j"):
            e, j = eng.edge_fields(phi, e=name == "e", j=name == "j")
            return e if name == "e" else j
        e, _ = eng.edge_fields(phi, e=True, j=False)
        q, rho = eng.node_charge(e, epsilon_0, density=name == "charge_density")
        return q if name == "charge" else rho

    def __getitem__(self, key):
        if not isinstance(key, tuple) or len(key) != 2:
            raise KeyError("index as f[src, 'phiSolution']")
        src, name = key
        if name not in ("phiSolution", "phi") + _DERIVED:
            raise KeyError(f"{name!r} is not a field of Fields3DNodal ({', '.join(('phi',) + _DERIVED)})")
        idx = self._src_index(src)
        if name in _DERIVED:
            out = self._derived(idx if isinstance(idx, list) else [idx], name).cpu().numpy()
            return out.T.copy() if isinstance(idx, list) else out[0]
        if isinstance(idx, list):
            return self.phi_dev[idx].cpu().numpy().T.copy()
        return self.phi_dev[idx].cpu().numpy()

    def __setitem__(self, key, value):
        import torch

        src, name = key
        if name not in ("phiSolution", "phi"):
            raise KeyError(name)
        idx = self._src_index(src)
        v = torch.as_tensor(np.asarray(value, dtype=np.float64), device=self.phi_dev.device)
        if isinstance(idx, list):
            self.phi_dev[idx] = v.T
        else:
            self.phi_dev[idx] = v


class Fields3DCellCentered(Fields3DNodal):
    """Device-backed ``Fields3DCellCentered`` (``resistivity/fields.py:75-185``): the cell-centred
    potential of every source, and on request ``e = MfI Grad phi`` and ``j = MfRhoI Grad phi`` on
    the faces (x|y|z faces, each Fortran-ordered) and ``charge = eps0 Div e``,
    ``charge_density = charge / V`` on the cells (``dc_cc_face_fields`` / ``dc_cc_charge``)."""

    knownFields = {"phiSolution": "CC"}
    aliasFields = {
        "phi": ["phiSolution", "CC", "_phi"],
        "j": ["phiSolution", "F", "_j"],
        "e": ["phiSolution", "F", "_e"],
        "charge": ["phiSolution", "CC", "_charge"],
        "charge_density": ["phiSolution", "CC", "_charge_density"],
    }

    def _GLoc(self, fieldType):
        if fieldType == "phi":
            return "CC"
        if fieldType in ("e", "j"):
            return "F"
        raise KeyError("Field type must be phi, e, j")

    def _derived(self, idx, name):
        from scipy.constants import epsilon_0

        eng = self.simulation.engine
        phi = self.phi_dev[idx]
        if name in ("e", "j"):
            e, j = eng.face_fields(phi, e=name == "e", j=name == "j")
            return e if name == "e" else j
        e, _ = eng.face_fields(phi, e=True, j=False)
        q, qd = eng.cell_charge(e, epsilon_0, density=name == "charge_density")
        return q if name == "charge" else qd
