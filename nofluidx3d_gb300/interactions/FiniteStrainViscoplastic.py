"""Finite-strain viscoplastic material plugin: the reference's
InteractionFiniteStrainViscoplastic (nofluidx3d/Interactions.py:248-349, kernel
kernels/InteractionFiniteStrainViscoplastic.cl) exposed through the new plugin API. It replaces
the Tetra plugin: elastic Mooney-Rivlin stress of Fe = F Fp^-1 plus the power-law flow rule
eps_dot = plasticFlowRate * (sigma_vm / sigma0)^flowExponent,
sigma0 = yieldStress * (1 + eps/hardeningThreshhold)^hardeningExponent."""

from .Interaction import Interaction


class FiniteStrainViscoplastic(Interaction):
    def __init__(self, shearModulus1, shearModulus2, bulkModulus, viscoplasticFlowExponent, viscoplasticYieldStress,
                 viscoplasticFlowRate, hardeningThreshhold, hardeningExponent):
        self.par = (shearModulus1, shearModulus2, bulkModulus, viscoplasticFlowExponent, viscoplasticYieldStress,
                    viscoplasticFlowRate, hardeningThreshhold, hardeningExponent)

    def build(self):
        self.scope = self.simulation.numTetra
        self.simulation.handle.set_viscoplastic(self.par)
