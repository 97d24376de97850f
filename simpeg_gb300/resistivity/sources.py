"""DC sources: the electrode/current description of a right-hand side.

Mirrors ``simpeg/electromagnetics/static/resistivity/sources.py:9-270``:
``Pole(receiver_list, location)`` carries one electrode with current ``+I``;
``Dipole(receiver_list, location_a, location_b)`` carries ``[+I, -I]``.  The
discretisation of a source to the nodal right-hand side (``BaseSrc.eval``,
``sources.py:64-88``: trilinear node interpolation weighted by the currents)
happens on the GPU through :func:`simpeg_gb300.resistivity.electrodes.electrode_table`.
"""

from __future__ import annotations

import numpy as np

__all__ = ["BaseSrc", "Pole", "Multipole", "Dipole"]


def _as_locations(loc):
    a = np.asarray(loc, dtype=np.float64)
    if a.ndim == 1:
        a = a[None, :]
    if a.ndim != 2:
        raise ValueError("location must be a (n, dim) array")
    return a


class BaseSrc:
    """Base DC source: ``location`` is ``(n_electrodes, dim)``, ``current`` per electrode."""

    def __init__(self, receiver_list, location, current=1.0):
        self.receiver_list = list(receiver_list) if receiver_list is not None else []
        self.location = location
        self.current = current

    @property
    def location(self):
        return self._location

    @location.setter
    def location(self, value):
        self._location = _as_locations(value)

    @property
    def current(self):
        return self._current

    @current.setter
    def current(self, value):
        c = np.atleast_1d(np.asarray(value, dtype=np.float64)).ravel()
        if len(c) > 1 and len(c) != self.location.shape[0]:
            raise ValueError(
                "Current must be constant or equal to the number of specified source "
                f"locations. saw {len(c)} current sources and {self.location.shape[0]} locations."
            )
        self._current = c

    @property
    def nD(self):
        return int(sum(rx.nD for rx in self.receiver_list))

    @property
    def vnD(self):
        return np.array([rx.nD for rx in self.receiver_list], dtype=int)

    def electrode_currents(self):
        """(n_electrodes,) currents, broadcasting a scalar current."""
        c = self.current
        if len(c) == 1 and self.location.shape[0] > 1:
            c = np.full(self.location.shape[0], c[0])
        return c

    def eval(self, sim):
        """Source term on the mesh nodes (``sources.py:64-88``, nodal formulation):
        ``q = sum_k I_k interp_N(location_k)`` as a host array (nN,).  The simulation builds
        the same term on the device from its electrode tables."""
        if getattr(sim, "_formulation", "EB") != "EB":
            raise NotImplementedError("only the nodal (EB) formulation is on the GPU path")
        from .electrodes import interp_weights

        idx, w = interp_weights(sim.mesh, self.location)
        q = np.zeros(sim.mesh.n_nodes)
        np.add.at(q, idx.ravel(), (self.electrode_currents()[:, None] * w).ravel())
        return q

    def evalDeriv(self, sim):
        """The source term does not depend on the model (``sources.py:90-104``)."""
        return 0.0


class Pole(BaseSrc):
    """Single current electrode A with current ``+I``."""

    def __init__(self, receiver_list, location=None, current=1.0):
        if location is None:
            raise TypeError("Pole source needs a location")
        super().__init__(receiver_list, location, current=current)
        if len(self.location) != 1:
            raise ValueError(
                f"Pole sources only have a single location, not {len(self.location)}"
            )

    @property
    def location_a(self):
        return self.location[0]

    @property
    def location_b(self):
        return np.full_like(self.location[0], np.nan)

    def __repr__(self):
        return f"Pole(a: {self.location[0]})"


class Multipole(BaseSrc):
    """Any number of current electrodes, one current each (``sources.py:107-132``)."""

    def __init__(self, receiver_list=None, location=None, current=1.0):
        if location is None:
            raise TypeError("Multipole source needs the electrode locations")
        super().__init__(receiver_list, location, current=current)

    @property
    def location_a(self):
        return self.location

    @property
    def location_b(self):
        return np.full_like(self.location, np.nan)


class Dipole(BaseSrc):
    """Current dipole A (+I), B (-I)."""

    def __init__(self, receiver_list, location_a=None, location_b=None, location=None, current=1.0):
        if location is None and location_a is None and location_b is None:
            raise TypeError(
                "Found 'location', 'location_a' and 'location_b' as None. Please specify "
                "'location', or 'location_a' and 'location_b' when defining a dipole source."
            )
        if location is not None and (location_a is not None or location_b is not None):
            raise TypeError(
                "Found 'location_a' and/or 'location_b' as not None values. When passing a "
                "not None value for 'location', 'location_a' and 'location_b' should be None."
            )
        if location is None:
            if location_a is None or location_b is None:
                raise TypeError("both 'location_a' and 'location_b' must be given")
            location = [location_a, location_b]
        if len(location) != 2:
            raise ValueError(
                "location must be a list or tuple of length 2: [location_a, location_b]. "
                f"The input location has length {len(location)}"
            )
        loc = np.vstack([np.asarray(location[0], float).ravel(), np.asarray(location[1], float).ravel()])
        super().__init__(receiver_list, loc, current=[current, -current])

    @property
    def location_a(self):
        return self.location[0]

    @property
    def location_b(self):
        return self.location[1]

    def __repr__(self):
        return f"Dipole(a: {self.location_a}; b: {self.location_b})"
