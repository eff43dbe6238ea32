"""Spherical indenter whose contact force is integrated over every tetra, mirroring
nofluidx3d/Interactions.py:601-637 (InteractionSphereIntegral) and
kernels/InteractionSphereIntegral.cl:22-85: a repulsive density exp(-forceConst (|x - c| - radius))
(x - c)/|x - c| with c = (0, sphereFunc(t), 0), integrated with a four-point Gauss rule per
tetra and distributed to its corners."""

from .. import _lib
from ._moving import MovingContact


class SphereIntegral(MovingContact):
    kind = _lib.CONTACT_SPHERE_INTEGRAL

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
