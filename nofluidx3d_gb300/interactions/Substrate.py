"""Rigid substrate below the cell, mirroring nofluidx3d/interactions/Substrate.py:18-37 and
kernels/Interactions/Substrate.cl: f_y += k * max(wallPosition - y, 0)."""

from .. import _lib
from .Interaction import Interaction


class Substrate(Interaction):
    def __init__(self, wallPosition, forceConst):
        self.wallPosition = wallPosition
        self.forceConst = forceConst
        self.contactId = None

    def build(self):
        self.scope = self.simulation.numPoints
        self.contactId = self.simulation.handle.add_contact(_lib.CONTACT_SUBSTRATE, self.forceConst, 0.0,
                                                            self.wallPosition, 0.0, float("inf"))
