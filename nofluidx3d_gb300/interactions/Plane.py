"""Flat indenter from above, mirroring nofluidx3d/interactions/Plane.py:18-41 and
kernels/Interactions/Plane.cl: f_y -= k * max(y - wallFunc(t), 0)."""

from .. import _lib
from ._moving import MovingContact


class Plane(MovingContact):
    kind = _lib.CONTACT_PLANE

    def __init__(self, wallFunc, forceConst):
        self.wallFunc = wallFunc
        self.forceConst = forceConst
        self.globalTime = 0
        self.contactId = None

    def _func(self):
        return self.wallFunc
