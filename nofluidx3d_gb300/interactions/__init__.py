from nofluidx3d_gb300.interactions.FiniteStrainViscoplastic import FiniteStrainViscoplastic
from nofluidx3d_gb300.interactions.Interaction import Interaction
from nofluidx3d_gb300.interactions.Plane import Plane
from nofluidx3d_gb300.interactions.Sphere import Sphere
from nofluidx3d_gb300.interactions.SphereIntegral import SphereIntegral
from nofluidx3d_gb300.interactions.Substrate import Substrate
from nofluidx3d_gb300.interactions.Tetra import Tetra
from nofluidx3d_gb300.interactions.VelocityVerlet import VelocityVerlet
from nofluidx3d_gb300.interactions.VelocityVerlet2 import VelocityVerlet2

__all__ = ["FiniteStrainViscoplastic", "Interaction", "Plane", "Sphere", "SphereIntegral", "Substrate", "Tetra",
           "VelocityVerlet", "VelocityVerlet2"]
