"""Lumped-mass damped velocity Verlet, mirroring nofluidx3d/Interactions.py:818-836
(InteractionVelocityVerlet2) and kernels/velocityVerlet2.cl: nodal masses density * sum of V0/4
over the node's tetrahedra (SimulationLegacy.py:911-924, density 1 there), the old-force buffer
holding the previous acceleration. Register it last, like VelocityVerlet."""

from .Interaction import Interaction


class VelocityVerlet2(Interaction):
    def __init__(self, numPoints, damping=0.1, density=1.0):
        self.damping = damping
        self.density = density

    def build(self):
        self.scope = self.simulation.numPoints
        self.simulation.handle.set_integrator_lumped(self.damping, self.density)
