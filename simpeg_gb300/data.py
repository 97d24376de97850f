"""Observed/synthetic data containers (``simpeg/data.py:11-391``, subset)."""

from __future__ import annotations

import numpy as np


class Data:
    def __init__(self, survey, dobs=None, relative_error=None, noise_floor=None, standard_deviation=None):
        self.survey = survey
        self.dobs = np.asarray(dobs, dtype=np.float64) if dobs is not None else np.full(survey.nD, np.nan)
        self.relative_error = relative_error
        self.noise_floor = noise_floor
        self._std = standard_deviation

    @property
    def nD(self):
        return self.dobs.size

    @property
    def standard_deviation(self):
        if self._std is not None:
            return np.asarray(self._std, dtype=np.float64)
        std = np.zeros(self.nD)
        if self.relative_error is not None:
            std = std + (np.asarray(self.relative_error) * np.abs(self.dobs)) ** 2
        if self.noise_floor is not None:
            std = std + np.asarray(self.noise_floor) ** 2
        return np.sqrt(std)


class SyntheticData(Data):
    def __init__(self, survey, dobs=None, dclean=None, **kwargs):
        super().__init__(survey, dobs=dobs, **kwargs)
        self.dclean = np.asarray(dclean, dtype=np.float64) if dclean is not None else None
