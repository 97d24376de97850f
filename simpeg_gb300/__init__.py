"""simpeg_gb300: simpeg's 3D nodal DC-resistivity forward/sensitivity path on GB300.

Public API mirrors simpeg (``resistivity.Simulation3DNodal``, ``resistivity.sources``,
``resistivity.receivers``, ``resistivity.Survey``, ``maps.ExpMap``...).  The compute
path is the CUDA engine ``libdcgpu.so`` (C ABI in ``include/dcgpu.h``).
"""

from . import maps, resistivity
from .mesh import TensorMesh

__all__ = ["TensorMesh", "maps", "resistivity"]
__version__ = "0.1.0"
