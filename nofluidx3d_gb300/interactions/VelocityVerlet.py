"""Damped velocity-Verlet integrator, mirroring nofluidx3d/interactions/VelocityVerlet.py:22-50
and kernels/Interactions/VelocityVerlet.cl. The reference hard-codes the damping xi = 0.005
(VelocityVerlet.cl:11); it is the keyword `damping` here with that default."""

from .Interaction import Interaction


class VelocityVerlet(Interaction):
    def __init__(self, numPoints, fixTopBottom=False, damping=0.005):
        self.fixTopBottom = fixTopBottom
        self.damping = damping

    def build(self):
        self.scope = self.simulation.numPoints
        self.simulation.handle.set_integrator(self.damping, self.fixTopBottom)
