"""Nodal and cell-centred DC resistivity on the GPU (mirror of ``simpeg.electromagnetics.static.resistivity``)."""

from . import receivers, sources
from .fields import Fields3DCellCentered, Fields3DNodal
from .simulation import Simulation3DNodal
from .simulation_cc import Simulation3DCellCentered
from .survey import Survey, geometric_factor
from .utils import WennerSrcList, mini_pole_pole

__all__ = ["receivers", "sources", "Survey", "Simulation3DNodal", "Simulation3DCellCentered", "Fields3DNodal",
           "Fields3DCellCentered", "geometric_factor",
           "mini_pole_pole", "WennerSrcList"]
