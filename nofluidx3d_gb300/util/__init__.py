from nofluidx3d_gb300.util.Bridge import Bridge
from nofluidx3d_gb300.util.IO import writeVTK

__all__ = ["Bridge", "writeVTK"]
