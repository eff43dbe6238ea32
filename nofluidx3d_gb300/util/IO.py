"""Output frames, nofluidx3d/util/IO.py:13-39.

writeVTK reads the node positions back from the device, checks them for NaN/Inf, updates the
cell mesh and writes a legacy-VTK frame with the optional per-tetra fields. The reference prints
a banner and exit()s on non-finite positions (IO.py:17-28); here FloatingPointError is raised.
"""

from __future__ import annotations

import numpy as np


def writeVTK(simulation, writeStress=True, writePressure=True, writeVolumeChange=False, write=True, positions=None,
             time=None, vonMises=None, pressure=None):
    """positions (SoA 3*np), time, vonMises and pressure may be given when the caller already read
    them (an output snapshot taken while later steps run); otherwise they are read back now."""
    if positions is None:
        positions = simulation.points.readFromGPU()
    else:
        simulation.points.arrayC[:] = positions
    positions = np.asarray(positions).reshape((3, simulation.numPoints)).transpose()
    if np.any(np.isnan(positions)):
        raise FloatingPointError("Encountered NaN when reading positions from the device")
    if np.any(np.isinf(positions)):
        raise FloatingPointError("Encountered INF when reading positions from the device")
    simulation.cell.mesh.points = positions.copy()
    if writeStress:
        simulation.cell.addTetraData("vonMises", simulation.vonMises.readFromGPU() if vonMises is None else vonMises)
    if writePressure:
        simulation.cell.addTetraData("pressure", -(simulation.pressure.readFromGPU() if pressure is None else pressure))
    if writeVolumeChange:
        simulation.cell.calcVolumeChange()
    if write:
        t = simulation.time if time is None else time
        simulation.cell.mesh.save(simulation.vtkfilespath + f"{t}.vtk")
