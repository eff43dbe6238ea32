"""Per-tetra hyperelastic force plugin, mirroring nofluidx3d/interactions/Tetra.py:23-92.

Material constants as the reference bakes them into tetra.cl (:79-84, :97-102, :118-121):
mu = E/(2(1+nu)), mu1 = r mu, mu2 = (1-r) mu, kappa = E/(3(1-2nu)). Neo-Hookean is
Mooney-Rivlin with ratio 1 (Tetra.py:77-78). The reference edge vectors and volumes
(Tetra.py:49-64) are computed by the library from the mesh given to the simulation.
"""

from enum import Enum, auto

from .. import _lib
from .Interaction import Interaction


class Tetra(Interaction):
    class materialModel(Enum):
        SAINT_VENANT_KIRCHHOFF_KELLNBERGER = auto()
        SVKK = SAINT_VENANT_KIRCHHOFF_KELLNBERGER
        SAINT_VENANT_KIRCHHOFF = auto()
        SVK = SAINT_VENANT_KIRCHHOFF
        NEO_HOOKEAN = auto()
        NH = NEO_HOOKEAN
        MOONEY_RIVLIN = auto()
        MR = MOONEY_RIVLIN

    _MODEL_CODE = {
        "SAINT_VENANT_KIRCHHOFF_KELLNBERGER": _lib.MODEL_SVKK,
        "SAINT_VENANT_KIRCHHOFF": _lib.MODEL_SVK,
        "NEO_HOOKEAN": _lib.MODEL_MR,
        "MOONEY_RIVLIN": _lib.MODEL_MR,
    }

    def __init__(self, referenceCell, youngsModulus, poissonRatio, mooneyRivlinRatio=1, model=materialModel.NEO_HOOKEAN):
        self.referenceCell = referenceCell
        self.youngsModulus = youngsModulus
        self.poissonRatio = poissonRatio
        self.mooneyRivlinRatio = mooneyRivlinRatio
        self.model = model

    def build(self):
        self.scope = self.simulation.numTetra
        code = self._MODEL_CODE[self.model.name]
        ratio = 1.0 if self.model is self.materialModel.NEO_HOOKEAN else self.mooneyRivlinRatio
        self.simulation.handle.set_tetra(code, self.youngsModulus, self.poissonRatio, ratio)
        self.referenceCell = None
