"""DC survey: the flat data layout over (source, receiver) pairs.

Mirrors ``simpeg/survey.py:416-626`` (``nD``, ``get_all_slices``: data ordered
by source in ``source_list``, then receiver in ``receiver_list``, then row) and
``simpeg/electromagnetics/static/resistivity/survey.py:13-300`` (ABMN
locations; ``set_geometric_factor`` per
``simpeg/electromagnetics/static/utils/static_utils.py:260-305``).
"""

from __future__ import annotations

import numpy as np

from . import receivers as Rx
from . import sources as Src

__all__ = ["Survey", "geometric_factor"]


class Survey:
    def __init__(self, source_list, survey_geometry="surface", **kwargs):
        if kwargs.pop("survey_type", None) is not None:
            raise TypeError("Argument 'survey_type' has been removed.")
        if kwargs:
            raise TypeError(f"unexpected arguments {sorted(kwargs)}")
        self.source_list = list(source_list)
        if survey_geometry not in ("surface", "borehole", "general"):
            raise ValueError("survey_geometry must be surface, borehole or general")
        self.survey_geometry = survey_geometry

    @property
    def survey_type(self):
        """Removed in the reference (``survey.py:57-72``): sources and receivers carry their type."""
        raise AttributeError("'survey_type' has been removed.")

    @property
    def source_locations(self):
        """[A locations, B locations] of every source, in order (``survey.py:150-166``)."""
        return [np.vstack([np.atleast_2d(src.location_a) for src in self.source_list]),
                np.vstack([np.atleast_2d(src.location_b) for src in self.source_list])]

    @property
    def nSrc(self):
        return len(self.source_list)

    @property
    def vnD(self):
        return np.array([src.nD for src in self.source_list], dtype=int)

    @property
    def nD(self):
        return int(self.vnD.sum())

    def get_all_slices(self):
        slices = {}
        end = 0
        for src in self.source_list:
            for rx in src.receiver_list:
                start = end
                end += rx.nD
                slices[(src, rx)] = slice(start, end)
        return slices

    def get_slice(self, source, receiver):
        s = self.get_all_slices().get((source, receiver))
        if s is None:
            raise KeyError(f"Source '{source}' and receiver '{receiver}' pair is not part of the survey.")
        return s

    def _abmn(self):
        a, b, m, n = [], [], [], []
        for src in self.source_list:
            for rx in src.receiver_list:
                k = rx.nD
                if isinstance(src, Src.Dipole):
                    a.append(np.repeat(src.location[0][None], k, 0))
                    b.append(np.repeat(src.location[1][None], k, 0))
                else:
                    a.append(np.repeat(src.location[0][None], k, 0))
                    b.append(np.repeat(src.location[0][None], k, 0))
                if isinstance(rx, Rx.Dipole):
                    m.append(rx.locations[0])
                    n.append(rx.locations[1])
                else:
                    m.append(rx.locations)
                    n.append(rx.locations)
        return [np.vstack(v) for v in (a, b, m, n)]

    @property
    def locations_a(self):
        return self._abmn()[0]

    @property
    def locations_b(self):
        return self._abmn()[1]

    @property
    def locations_m(self):
        return self._abmn()[2]

    @property
    def locations_n(self):
        return self._abmn()[3]

    @property
    def unique_electrode_locations(self):
        return np.unique(np.vstack(self._abmn()), axis=0)

    def set_geometric_factor(self, space_type="halfspace"):
        g = geometric_factor(self, space_type=space_type)
        slices = self.get_all_slices()
        for src in self.source_list:
            for rx in src.receiver_list:
                if rx.data_type == "apparent_resistivity":
                    rx._geometric_factor[src] = g[slices[src, rx]]
        return g

    def __repr__(self):
        return f"Survey(#sources: {self.nSrc}; #data: {self.nD})"


def geometric_factor(survey, space_type="halfspace"):
    """G = (1/C)(1/AM - 1/BM - 1/AN + 1/BN), C = 2*pi (half space) or 4*pi (whole space).

    Pole electrodes sit at infinity, so their terms vanish.
    """
    st = space_type.lower().replace("-", "").replace("_", "").replace(" ", "")
    if st in ("halfspace", "half"):
        fac = 2.0
    elif st in ("wholespace", "whole"):
        fac = 4.0
    else:
        raise TypeError("'space_type must be 'whole space' | 'half space'")
    out = []
    for src in survey.source_list:
        a = src.location[0]
        b = src.location[1] if isinstance(src, Src.Dipole) else np.full_like(a, np.inf)
        for rx in src.receiver_list:
            if isinstance(rx, Rx.Dipole):
                m, n = rx.locations
            else:
                m = rx.locations
                n = np.full_like(m, -np.inf)
            with np.errstate(divide="ignore"):
                am = np.linalg.norm(a - m, axis=1)
                bm = np.linalg.norm(b - m, axis=1)
                an = np.linalg.norm(a - n, axis=1)
                bn = np.linalg.norm(b - n, axis=1)
                out.append(1 / am - 1 / bm - 1 / an + 1 / bn)
    return np.hstack(out) / (fac * np.pi)
