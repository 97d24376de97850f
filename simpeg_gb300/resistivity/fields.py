"""Device-backed ``Fields3DNodal``.

Mirrors ``simpeg/electromagnetics/static/resistivity/fields.py:186-257`` and
the ``Fields`` store of ``simpeg/fields.py:7-345``: the nodal potential of
every source, indexed ``f[src, "phiSolution"]`` / ``f[:, "phi"]``.  The store
stays on the GPU as a ``(nSrc, nN)`` float64 tensor (column-major (nN, nSrc));
indexing copies the requested columns to the host as numpy arrays.
"""

from __future__ import annotations

import numpy as np


class Fields3DNodal:
    knownFields = {"phiSolution": "N"}
    aliasFields = {"phi": ["phiSolution", "N", "_phi"]}

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

    def __getitem__(self, key):
        if not isinstance(key, tuple) or len(key) != 2:
            raise KeyError("index as f[src, 'phiSolution']")
        src, name = key
        if name not in ("phiSolution", "phi"):
            raise KeyError(f"field {name!r} is not stored on the GPU path (phi / phiSolution only)")
        idx = self._src_index(src)
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
