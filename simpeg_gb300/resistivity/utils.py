"""Survey utilities: pole-pole miniaturisation.

Restates ``_mini_pole_pole`` (``simpeg/electromagnetics/static/resistivity/
utils.py:75-128``): every datum AM - AN - BM + BN of a dipole survey is a sum
of pole-pole potentials.  The unique electrodes are numbered with
``np.unique(axis=0)``, each (A, M) pair is sorted (reciprocity: G(A,M) = G(M,A)),
the unique pairs become pole sources with pole receivers, and integer inverse
maps reassemble the dipole data (bit-exact integer work).
"""

from __future__ import annotations

import numpy as np

from . import receivers, sources
from .survey import Survey


def WennerSrcList(n_electrodes, a_spacing, in2D=False, plotIt=False):
    """Dipole sources of a Wenner array (``resistivity/utils.py:13-74``): electrodes
    ``a_spacing`` apart on a line centred on x = 0; for every spacing s = 1, 2, ... and first
    electrode j with j + 3 s < n_electrodes, source A = e_j, B = e_(j+3s) with one dipole
    receiver M = e_(j+s), N = e_(j+2s).  Locations are (x, 0, 0), or (x, 0) with ``in2D``."""
    if plotIt:
        raise NotImplementedError("plotting is not part of this package")
    n = int(n_electrodes)
    x = a_spacing * np.arange(n) - a_spacing * (n - 1) / 2.0

    def loc(i):
        return np.r_[x[i], 0.0] if in2D else np.r_[x[i], 0.0, 0.0]

    out = []
    for s in range(1, n):
        for j in range(n - 3 * s):
            rx = receivers.Dipole(loc(j + s)[None, :], loc(j + 2 * s)[None, :])
            out.append(sources.Dipole([rx], loc(j), loc(j + 3 * s)))
    return out


def mini_pole_pole(survey, verbose=False):
    A = survey.locations_a
    B = survey.locations_b
    M = survey.locations_m
    N = survey.locations_n
    elecs, inverse = np.unique(np.r_[A, B, M, N], axis=0, return_inverse=True)
    inverse = np.asarray(inverse).ravel()
    inv_A, inv_B, inv_M, inv_N = inverse.reshape(4, -1)
    dipole_tx = inv_A != inv_B
    dipole_rx = inv_M != inv_N
    AM = np.sort(np.c_[inv_A, inv_M])
    AN = np.sort(np.c_[inv_A[dipole_rx], inv_N[dipole_rx]])
    BM = np.sort(np.c_[inv_B[dipole_tx], inv_M[dipole_tx]])
    BN = np.sort(np.c_[inv_B[dipole_tx & dipole_rx], inv_N[dipole_tx & dipole_rx]])
    upp, pp_inv = np.unique(np.r_[AM, AN, BM, BN], axis=0, return_inverse=True)
    pp_inv = np.asarray(pp_inv).ravel()
    nAM, nAN, nBM = len(AM), len(AN), len(BM)
    inv_AM = pp_inv[:nAM]
    inv_AN = pp_inv[nAM:nAM + nAN]
    inv_BM = pp_inv[nAM + nAN:nAM + nAN + nBM]
    inv_BN = pp_inv[nAM + nAN + nBM:]
    if verbose:
        print(f"There are {upp.shape[0]} unique pole-pole combinations.")
    unique_sources = []
    # group the sorted unique pairs by their first electrode
    starts = np.flatnonzero(np.r_[True, upp[1:, 0] != upp[:-1, 0]]) if len(upp) else np.zeros(0, int)
    ends = np.r_[starts[1:], len(upp)]
    for s0, s1 in zip(starts, ends):
        rxs = receivers.Pole(elecs[upp[s0:s1, 1]])
        unique_sources.append(sources.Pole([rxs], elecs[upp[s0, 0]]))
    return [dipole_rx, dipole_tx], [inv_AM, inv_AN, inv_BM, inv_BN], Survey(unique_sources)
