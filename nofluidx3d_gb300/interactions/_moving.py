"""Shared logic of the moving indenters (Plane, Sphere).

The reference calls the position callable on the host every step and passes the value as a
kernel argument (interactions/Plane.py:32-41, Sphere.py:33-43). Here a callable that carries
an `nfx_schedule = (p0, v, tmove)` attribute (position p0 - v*min(t, tmove), as the
Simulation's own wallFunc/sphereFunc do) runs on the device; any other callable is evaluated
on the host for every step of a block and uploaded as a per-step position table, which keeps
arbitrary callables exact.
"""

import numpy as np

from .Interaction import Interaction


class MovingContact(Interaction):
    kind = -1

    def _func(self):
        raise NotImplementedError

    def _radius(self) -> float:
        return 0.0

    def build(self):
        self.scope = self.simulation.numPoints
        f = self._func()
        sched = getattr(f, "nfx_schedule", None)
        if sched is not None:
            p0, v, tmove = sched
            self.tableMode = False
        else:
            p0, v, tmove = float(f(0)), 0.0, float("inf")
            self.tableMode = True
        self.contactId = self.simulation.handle.add_contact(self.kind, self.forceConst, self._radius(), p0, v, tmove)

    def beforeTimeStep(self, globalTime):
        self.globalTime = globalTime

    def prepareSteps(self, t0: int, n: int):
        if not self.tableMode:
            return
        f = self._func()
        # one extra entry: the readout after the block evaluates the position at t0 + n
        pos = np.array([f(t) for t in range(t0, t0 + n + 1)], dtype=np.float64)
        self.simulation.handle.set_contact_table(self.contactId, t0, pos)
