"""simpeg_gb300: simpeg's 3D nodal DC-resistivity forward/sensitivity path on GB300.

Public API mirrors simpeg (``resistivity.Simulation3DNodal``, ``resistivity.sources``,
``resistivity.receivers``, ``resistivity.Survey``, ``maps.ExpMap``,
``induced_polarization.Simulation3DNodal``, ``meta.MetaSimulation``...).  The compute
path is the CUDA engine ``libdcgpu.so`` (C ABI in ``include/dcgpu.h``).
"""

from . import induced_polarization, maps, meta, resistivity
from .mesh import TensorMesh

__all__ = ["TensorMesh", "maps", "resistivity", "induced_polarization", "meta"]
__version__ = "0.1.0"
