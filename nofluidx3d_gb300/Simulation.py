"""Simulation driver, mirroring nofluidx3d/Simulation.py:34-290.

Same JSON configuration, unit conversion, interaction set-up and output loop as the reference;
the difference is underneath: the shared buffers live in one nfx_sim handle (a CellSim) on the
GPU, plugins hand it their parameters, and timeStep()/run() advance the whole fused step through
the C ABI. Output frames are legacy-VTK files; non-finite positions raise FloatingPointError
instead of exit().

`con` is a path to the reference's JSON config or an already-parsed dict with the same keys.
`cell` optionally supplies the TetraCell directly (e.g. a generated Kuhn sphere through
TetraCell.from_arrays) instead of reading CELL.InitVTK, which avoids a text VTK round trip for
meshes of millions of tetrahedra.
"""

from __future__ import annotations

import json
import os
import time

import numpy as np

from .core import CellSim
from .interactions import (FiniteStrainViscoplastic, Plane, Sphere, SphereIntegral, Substrate, Tetra, VelocityVerlet,
                           VelocityVerlet2)
from .TetraCell import TetraCell
from .util.Bridge import Bridge
from .util.IO import writeVTK


def _linear_schedule(p0: float, v: float, tmove: float):
    """The reference's wallFunc/sphereFunc shape (Simulation.py:117-132, :173-183), tagged so the
    position runs on the device."""

    def f(time):
        if time <= tmove:
            return p0 - v * time
        return p0 - v * tmove

    f.nfx_schedule = (p0, v, tmove)
    return f


class Simulation:
    def __init__(self, con, verbose: bool = True, cell: TetraCell | None = None):
        if isinstance(con, dict):
            self.parameters = con
        else:
            with open(con) as configfile:
                self.parameters = json.load(configfile)
        self.verbose = verbose
        device = int(self.parameters.get("gpu", 0))

        # conversion constants (Simulation.py:41-53)
        rho = 1.0
        self.rho0 = self.parameters["RhoSI"] / rho
        self.L0 = self.parameters["CELL"]["RadiusSI"] / self.parameters["CELL"]["RadiusSIM"]
        E = 1e-2
        self.p0 = self.parameters["CELL"]["YoungsModulusSI"] / E
        self.V0 = np.sqrt(self.p0 / self.rho0)
        self.T0 = self.L0 / self.V0
        self._print(f"V0={self.V0}")
        self._print(f"T0={self.T0}")

        self.Nsteps = int(round(self.parameters["SimulationTimeSI"] / self.T0))
        self.VTKInterval = int(round(self.Nsteps / self.parameters["VTKFramesTotal"]))
        self.vtkfilespath = self.parameters["OutputDir"] + "vtkfiles/frame"
        os.makedirs(self.parameters["OutputDir"] + "vtkfiles", exist_ok=True)

        if cell is not None:
            self.cell = cell
        else:
            self.cell = TetraCell(self.parameters["CELL"]["InitVTK"], radius=self.parameters["CELL"]["RadiusSIM"],
                                  recenter=True)
        self.numPoints = self.cell.points[:, 0].size
        self.numTetra = self.cell.tetras[:, 0].size
        self._print(f"Particle mesh consists of {self.numPoints} vertices and {self.numTetra} tetrahedrons")
        self.interactions = []
        self.time = 0

        # the device state (shared buffers of Simulation.py:82-90)
        self.handle = CellSim(device)
        self.handle.set_mesh(self.cell.points, self.cell.tetras)
        # per-tetra fields are refreshed by the last step of every output interval
        self.handle.set_record(-1, max(self.VTKInterval, 1), 0)
        self.points = Bridge(self.cell.points.reshape(3 * self.numPoints, order="F"), np.float64,
                             read=lambda a: self.handle.points_soa(out=a), write=lambda a: self.handle.set_points(a))
        self.tetras = Bridge(self.cell.tetras.reshape(4 * self.numTetra, order="F"), np.uint32)
        # VelocityVerlet.cl zeroes the force buffer at the end of every step (:33-35)
        self.force = Bridge(np.zeros(self.numPoints * 3), np.float64, read=lambda a: a.fill(0.0))
        self.vonMises = Bridge(np.zeros(self.numTetra), np.float64,
                               read=lambda a: a.__setitem__(slice(None), self.handle.tet_field(0)))
        self.pressure = Bridge(np.zeros(self.numTetra), np.float64,
                               read=lambda a: a.__setitem__(slice(None), self.handle.tet_field(1)))

        self.recordedQuantities = []

        def currentTime():
            return self.time

        self.recordedQuantities.append(currentTime)

    def _print(self, *a, **k):
        if self.verbose:
            print(*a, **k)

    def register(self, interaction):
        interaction.register(self)
        self.interactions.append(interaction)

    def setInteractionSubstrate(self):
        wallPosition = -(self.parameters["CELL"]["RadiusSIM"] + self.parameters["InitialDistance"])
        forceConst = 0.1
        self.register(Substrate(wallPosition, forceConst))

    def _move_params(self):
        v = self.parameters["VelocitySI"] / self.V0
        tmove = self.parameters["MoveTimeSI"] / self.T0
        return v, tmove

    def setInteractionPlane(self, record=True):
        p0 = self.parameters["CELL"]["RadiusSIM"] + self.parameters["InitialDistance"]
        v, tmove = self._move_params()
        wallFunc = _linear_schedule(p0, v, tmove)
        forceConst = 0.1
        plane = Plane(wallFunc, forceConst)
        self.register(plane)

        def indentationSI():
            return (wallFunc(0) - wallFunc(self.time)) * self.L0

        def forceSI():
            return self.handle.indenter_force(plane.contactId) * (self.p0 * self.L0**2)

        if record:
            self.recordedQuantities.append(indentationSI)
            self.recordedQuantities.append(forceSI)
        return plane

    def setInteractionSphere(self, record=True, isSpherical=True):
        radius = self.parameters["SphereRadiusSI"] / self.L0
        if isSpherical:
            start = self.parameters["CELL"]["RadiusSIM"] + radius + self.parameters["InitialDistance"]
        else:
            start = self.cell.mesh.points[3][1] + radius + self.parameters["InitialDistance"]
        v, tmove = self._move_params()
        sphereFunc = _linear_schedule(start, v, tmove)
        forceConst = 0.1
        sphere = Sphere(radius, sphereFunc, forceConst)
        self.register(sphere)

        def indentationSI():
            return (sphereFunc(0) - sphereFunc(self.time)) * self.L0

        def forceSI():
            return self.handle.indenter_force(sphere.contactId) * (self.p0 * self.L0**2)

        if record:
            self.recordedQuantities.append(indentationSI)
            self.recordedQuantities.append(forceSI)
        return sphere

    def setInteractionSphereIntegral(self, record=True, isSpherical=True):
        """Sphere contact integrated over the tetrahedra, as SimulationLegacy.py:206-273: the decay
        rate is the configuration's PotentialForceConst; the recorded force is -sum of the y
        forces times p0 L0^2 ReynoldScaling YoungsScaling."""
        radius = self.parameters["SphereRadiusSI"] / self.L0
        if isSpherical:
            start = self.parameters["CELL"]["RadiusSIM"] + radius + self.parameters["InitialDistance"]
        else:
            start = self.cell.mesh.points[3][1] + radius + self.parameters["InitialDistance"]
        v, tmove = self._move_params()
        sphereFunc = _linear_schedule(start, v, tmove)
        sphere = SphereIntegral(radius, sphereFunc, self.parameters["PotentialForceConst"])
        self.register(sphere)

        def indentationSI():
            return (sphereFunc(0) - sphereFunc(self.time)) * self.L0

        def forceSI():
            scale = (self.p0 * self.L0**2 * self.parameters.get("ReynoldScaling", 1.0)
                     * self.parameters["CELL"].get("YoungsScaling", 1.0))
            return self.handle.indenter_force(sphere.contactId) * scale

        if record:
            self.recordedQuantities.append(indentationSI)
            self.recordedQuantities.append(forceSI)
        return sphere

    def setInteractionTetra(self):
        youngsModulusSI = self.parameters["CELL"]["YoungsModulusSI"]
        poissonRatio = self.parameters["CELL"]["PoissonRatio"]
        mooneyRivlinRatio = self.parameters["CELL"].get("MooneyRivlinRatio", 1)
        youngsModulus = youngsModulusSI / self.p0
        model = Tetra.materialModel[self.parameters["CELL"]["model"]]
        self.register(Tetra(self.cell, youngsModulus, poissonRatio, mooneyRivlinRatio, model))

    def setInteractionFiniteStrainViscoplastic(self):
        """The viscoplastic material with the parameter mapping of the legacy driver
        (SimulationLegacy.py:842-882): mu1 = r G, mu2 = (1-r) G, K, flowRate = T0,
        yieldStress = timeConstantSI^(1/m) / YoungsScaling."""
        c = self.parameters["CELL"]
        youngsModulus = (c["YoungsModulusSI"] / self.parameters.get("ReynoldScaling", 1.0)
                         / c.get("YoungsScaling", 1.0) / self.p0)
        nu = c["PoissonRatio"]
        r = c.get("MooneyRivlinRatio", 1.0)
        G = youngsModulus / (2 * (1 + nu))
        K = youngsModulus / (3 * (1 - 2 * nu))
        m = c["ViscoplasticFlowExponent"]
        yieldStress = c["ViscoplasticTimeConstantSI"] ** (1.0 / m) / c.get("YoungsScaling", 1.0)
        self.register(FiniteStrainViscoplastic(r * G, (1 - r) * G, K, m, yieldStress, self.T0,
                                               c["HardeningThreshhold"], c["HardeningExponent"]))

    # Velocity Verlet last, as in the reference (Simulation.py:227)
    def setInteractionVelocityVerlet(self, fixTopBottom=False, damping=0.005):
        self.register(VelocityVerlet(self.numPoints, fixTopBottom, damping))

    # the lumped-mass form, SimulationLegacy.py:911-924 (density 1)
    def setInteractionVelocityVerlet2(self, damping=0.1):
        self.register(VelocityVerlet2(self.numPoints, damping))

    def _advance(self, n: int):
        for interaction in self.interactions:
            for t in range(self.time, self.time + n):
                interaction.beforeTimeStep(t)
            interaction.prepareSteps(self.time, n)
        self.handle.step(n)
        self.time += n

    def timeStep(self):
        self._advance(1)

    def run(self, writeStress=True, writePressure=True, writeVolumeChange=False, write=True):
        """The output loop of Simulation.py:239-290, with the same frames and simdata.dat rows.
        The device runs the next output interval while the host writes the current frame: each
        frame's positions come from an output snapshot (nfx_snapshot into page-locked buffers),
        and its recorded quantities and per-tetra fields are read at the frame's time before the
        next interval is enqueued. write=False does every readback of an output but writes no
        frame and no simdata.dat."""
        from .core import PinnedArray

        self._print(f"VTKInterval: {self.VTKInterval}")
        starttimes, endtimes = [], []
        numberCycles = self.parameters["VTKFramesTotal"]
        writeVTK(self, writeStress=writeStress, writePressure=writePressure, writeVolumeChange=writeVolumeChange,
                 write=write)
        dataPoints = np.array([quant() for quant in self.recordedQuantities])
        if write:
            np.savetxt(self.parameters["OutputDir"] + "simdata.dat", dataPoints)
        frames = [PinnedArray(3 * self.numPoints) for _ in range(2)]
        if numberCycles > 0:
            starttimes.append(time.time())
            self._advance(self.VTKInterval)
        for i in range(numberCycles):
            buf = frames[i % 2].array
            self.handle.snapshot(buf)  # positions at the end of this interval, copied asynchronously
            frame_time = self.time
            row = [quant() for quant in self.recordedQuantities]
            vm = self.handle.tet_field(0) if writeStress else None
            pr = self.handle.tet_field(1) if writePressure else None
            if i + 1 < numberCycles:  # the next interval runs while this frame is written
                starttimes.append(time.time())
                self._advance(self.VTKInterval)
            self.handle.snapshot_wait()
            anatime1 = time.time()
            writeVTK(self, writeStress=writeStress, writePressure=writePressure, writeVolumeChange=writeVolumeChange,
                     write=write, positions=buf, time=frame_time, vonMises=vm, pressure=pr)
            dataPoints = np.vstack((dataPoints, row))
            if write:
                np.savetxt(self.parameters["OutputDir"] + "simdata.dat", dataPoints)
            anatime2 = time.time()
            endtimes.append(time.time())
            cycleTime = np.average(np.array(endtimes) - np.array(starttimes[:len(endtimes)]))
            self._print(f"| Average # of simulation steps per second: {np.round(self.VTKInterval / cycleTime, 1)} "
                        f"| VTK cycle took {np.round(anatime2 - anatime1, 1)} seconds", end="\r")
        self.handle.sync()
        self._print("")
        return dataPoints

    def saveCheckpoint(self, path: str) -> None:
        """Write the whole device state (positions, velocities, previous forces, plastic state,
        time, recorded force rows) to `path`; loadCheckpoint resumes from it bit for bit. The
        reference's restart (SimulationLegacy.py:103-112) reloads positions only."""
        data = self.handle.checkpoint()
        with open(path, "wb") as f:
            f.write(data)

    def loadCheckpoint(self, path: str) -> None:
        """Restore a saveCheckpoint file into this simulation, set up with the same mesh and
        interactions (registered before the call)."""
        with open(path, "rb") as f:
            self.handle.restore(f.read())
        self.time = self.handle.time

    def close(self):
        self.handle.close()
