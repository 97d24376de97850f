"""Nodal DC resistivity on the GPU (mirror of ``simpeg.electromagnetics.static.resistivity``)."""

from . import receivers, sources
from .fields import Fields3DNodal
from .simulation import Simulation3DNodal
from .survey import Survey, geometric_factor
from .utils import WennerSrcList, mini_pole_pole

__all__ = ["receivers", "sources", "Survey", "Simulation3DNodal", "Fields3DNodal", "geometric_factor",
           "mini_pole_pole", "WennerSrcList"]
