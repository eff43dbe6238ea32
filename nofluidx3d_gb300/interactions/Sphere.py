"""Spherical indenter centred at (0, sphereFunc(t), 0), mirroring
nofluidx3d/interactions/Sphere.py:18-43 and kernels/Interactions/Sphere.cl:
f += k * max(radius - |r|, 0) * r/|r|."""

from .. import _lib
from ._moving import MovingContact


class Sphere(MovingContact):
    kind = _lib.CONTACT_SPHERE

    def __init__(self, radius, sphereFunc, forceConst):
        self.radius = radius
        self.sphereFunc = sphereFunc
        self.forceConst = forceConst
        self.globalTime = 0
        self.contactId = None

    def _func(self):
        return self.sphereFunc

    def _radius(self) -> float:
        return float(self.radius)
