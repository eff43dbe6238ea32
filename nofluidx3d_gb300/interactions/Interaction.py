"""Interaction plugin base, mirroring nofluidx3d/interactions/Interaction.py:15-40.

Lifecycle as in the reference: register(simulation) -> createBuffers() -> build() -> setArgs(),
then per step beforeTimeStep(t) and enqueue(). The difference: a plugin no longer launches its
own kernel. It hands its parameters to the simulation's nfx_sim handle in build()/setArgs(), and
Simulation.timeStep()/run() advance all of them with one fused step. enqueue() is therefore a
no-op, kept so code that calls it still runs. prepareSteps(t0, n) is called before a block of n
steps starting at time t0 so plugins with host-side per-step data (position callables) can
upload it for the whole block.
"""


class Interaction:
    def __init__(self, scope=None):
        self.scope = scope
        self.knl = None

    def register(self, simulation):
        self.simulation = simulation
        self.createBuffers()
        self.build()
        self.setArgs()

    def createBuffers(self):
        pass

    def build(self):
        pass

    def setArgs(self):
        pass

    def beforeTimeStep(self, globalTime):
        pass

    def prepareSteps(self, t0: int, n: int):
        pass

    def enqueue(self):
        """The step is fused: Simulation.timeStep() launches it once for all plugins."""
        return None
