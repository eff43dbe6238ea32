"""TetraCell: the reference cell mesh and its per-tetra reference quantities.

Mirrors nofluidx3d/TetraCell.py:11-65. The mesh is read from a legacy VTK file (vtk.read_vtk
instead of pyvista), or taken from arrays (`TetraCell.from_arrays`, e.g. a generated Kuhn
sphere). With recenter=True point 0 is moved to the origin and the mesh is scaled so that the
x coordinate of point 1 equals `radius` (TetraCell.py:15-20).
"""

from __future__ import annotations

import numpy as np

from .mesh import CellMesh
from .vtk import VTK_TETRA, VtkMesh, read_vtk

__all__ = ["TetraCell"]


class TetraCell:
    def __init__(self, path, radius: float = 18.0, recenter: bool = True, mesh: VtkMesh | None = None):
        self.mesh = mesh if mesh is not None else read_vtk(str(path))
        if recenter:
            transvec = -self.mesh.points[0]  # the mesh's first point becomes the centre
            self.mesh.translate(transvec, inplace=True)
            radius_mesh = np.abs(self.mesh.points[1][0])  # the second point lies on the x axis at the radius
            self.mesh.scale(radius / radius_mesh, inplace=True)
        self.points = self.mesh.points
        self.radius = radius
        self.tetras = self.mesh.cells_dict[VTK_TETRA]
        R1, R2, R3 = self.calcEdgeVectors(self.points)
        self.edgeVectors = np.einsum("ijk -> jik", np.array([R1, R2, R3])).reshape(len(R1), 9)
        self.volumes = self.calcVolumes(R1, R2, R3)

    @classmethod
    def from_arrays(cls, points: np.ndarray, tets: np.ndarray, radius: float | None = None,
                    recenter: bool = False) -> "TetraCell":
        m = VtkMesh(points=np.array(points, dtype=np.float64), cells=[(VTK_TETRA, np.asarray(tets, np.int64))])
        r = float(radius) if radius is not None else float(np.abs(m.points[1][0]))
        return cls(None, radius=r, recenter=recenter, mesh=m)

    @classmethod
    def from_cell_mesh(cls, cm: CellMesh) -> "TetraCell":
        return cls.from_arrays(cm.points, cm.tets, radius=cm.radius, recenter=False)

    def calcEdgeVectors(self, points):
        """R_i = P_i - P_0 (TetraCell.py:33-38)."""
        p0 = points[self.tetras[:, 0]]
        return points[self.tetras[:, 1]] - p0, points[self.tetras[:, 2]] - p0, points[self.tetras[:, 3]] - p0

    def calcVolumes(self, R1, R2, R3):
        """Signed volume R1.(R2 x R3)/6 (TetraCell.py:40-41)."""
        return np.einsum("ij,ij->i", R1, np.cross(R2, R3)) / 6

    def scale(self, scaling):
        self.mesh.scale(scaling, inplace=True)
        self.points = self.mesh.points
        R1, R2, R3 = self.calcEdgeVectors(self.points)
        self.edgeVectors = np.einsum("ijk -> jik", np.array([R1, R2, R3])).reshape(len(R1), 9)
        self.volumes = self.calcVolumes(R1, R2, R3)

    def addTetraData(self, name, dataArray):
        """Attach per-tetra data, zero-padded in front to the mesh's cell count (TetraCell.py:53-56)."""
        dataArray = np.asarray(dataArray)
        padded = np.pad(dataArray, pad_width=(self.mesh.n_cells - dataArray.size, 0))
        self.mesh.cell_data.set_array(padded, name)

    def calcVolumeChange(self):
        """Current volume / reference volume - 1 per tetra (TetraCell.py:58-60)."""
        cur = self.calcVolumes(*self.calcEdgeVectors(self.mesh.points))
        self.addTetraData("volumeChange", cur / self.volumes - 1)
