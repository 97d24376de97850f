"""Induced polarization on the GPU (mirror of ``simpeg.electromagnetics.static.induced_polarization``).

The IP problem reuses the DC machinery: receivers, sources and surveys are the
resistivity ones, and the nodal simulation is the DC simulation at a fixed
conductivity with the chargeability as the model; the cell-centred one is the
cell-centred DC simulation the same way.
"""

from ..resistivity import receivers, sources, utils
from ..resistivity.survey import Survey
from .simulation import Simulation3DCellCentered, Simulation3DNodal
from .survey import from_dc_to_ip_survey

__all__ = ["Simulation3DNodal", "Simulation3DCellCentered", "Survey", "from_dc_to_ip_survey", "receivers", "sources", "utils"]
