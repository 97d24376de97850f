"""Closed-form DC potentials (oracle only -- test infrastructure).

Restates ``simpeg/electromagnetics/analytics/DC.py:5-97``: the potential of a
point current I in a uniform medium of conductivity sigma is
``I / (4 pi sigma r)`` (whole space) and twice that on the surface of a half
space.  Used as the analytic pin of ``tests/em/static/test_DC_analytic.py:10-81``.
"""

from __future__ import annotations

import numpy as np


def _r(a, pts):
    pts = np.atleast_2d(pts)
    return np.sqrt(((pts - np.asarray(a)[None, :]) ** 2).sum(axis=1))


def pole_dipole(a, m, n, sigma, current=1.0, earth_type="wholespace"):
    """phi(M) - phi(N) for a + pole at a."""
    f = current / (4 * np.pi * sigma)
    phi = f * (1 / _r(a, m) - 1 / _r(a, n))
    return 2 * phi if earth_type == "halfspace" else phi


def pole_pole(a, m, sigma, current=1.0, earth_type="wholespace"):
    f = current / (4 * np.pi * sigma)
    phi = f / _r(a, m)
    return 2 * phi if earth_type == "halfspace" else phi


def dipole_dipole(a, b, m, n, sigma, current=1.0, earth_type="wholespace"):
    return pole_dipole(a, m, n, sigma, current, earth_type) - pole_dipole(b, m, n, sigma, current, earth_type)
