"""Output frames, nofluidx3d/util/IO.py:13-39.

writeVTK reads the node positions back from the device, checks them for NaN/Inf, updates the
cell mesh and writes a legacy-VTK frame with the optional per-tetra fields. The reference prints
a banner and exit()s on non-finite positions (IO.py:17-28); here FloatingPointError is raised.
"""

from __future__ import annotations

import numpy as np


def writeVTK(simulation, writeStress=True, writePressure=True, writeVolumeChange=False, write=True):
    positions = simulation.points.readFromGPU()
    positions = positions.reshape((3, simulation.numPoints)).transpose()
    if np.any(np.isnan(positions)):
        raise FloatingPointError("Encountered NaN when reading positions from the device")
    if np.any(np.isinf(positions)):
        raise FloatingPointError("Encountered INF when reading positions from the device")
    simulation.cell.mesh.points = positions.copy()
    if writeStress:
        simulation.cell.addTetraData("vonMises", simulation.vonMises.readFromGPU())
    if writePressure:
        simulation.cell.addTetraData("pressure", -simulation.pressure.readFromGPU())
    if writeVolumeChange:
        simulation.cell.calcVolumeChange()
    if write:
        simulation.cell.mesh.save(simulation.vtkfilespath + f"{simulation.time}.vtk")
