"""Legacy-VTK unstructured-grid IO for tetrahedral cell meshes.

The reference reads its InitVTK mesh and writes every output frame through pyvista
(nofluidx3d/TetraCell.py:14, nofluidx3d/util/IO.py:39), which is not installed here. This module
reads and writes the legacy VTK format (``# vtk DataFile Version``, DATASET UNSTRUCTURED_GRID)
in ASCII or BINARY (big-endian) encoding: POINTS, CELLS, CELL_TYPES and CELL_DATA scalars.
`VtkMesh` offers the small part of pyvista's UnstructuredGrid the reference uses: ``points``,
``cells_dict[10]`` (VTK_TETRA), ``n_cells``, ``cell_data``, ``translate``, ``scale``, ``save``.
"""

from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

VTK_TETRA = 10

__all__ = ["VtkMesh", "read_vtk", "write_vtk", "VTK_TETRA"]


class _CellData(dict):
    def set_array(self, arr, name):
        self[name] = np.asarray(arr)


@dataclass
class VtkMesh:
    points: np.ndarray                       # (Np, 3) float64
    cells: list = field(default_factory=list)  # [(vtk type, (n, k) connectivity)]
    cell_data: _CellData = field(default_factory=_CellData)

    @property
    def cells_dict(self) -> dict:
        d: dict = {}
        for t, conn in self.cells:
            d[t] = conn if t not in d else np.concatenate([d[t], conn])
        return d

    @property
    def n_cells(self) -> int:
        return int(sum(c.shape[0] for _, c in self.cells))

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    def translate(self, v, inplace: bool = True):
        self.points = self.points + np.asarray(v, dtype=np.float64)
        return self

    def scale(self, s, inplace: bool = True):
        self.points = self.points * np.asarray(s, dtype=np.float64)
        return self

    def save(self, path: str, binary: bool = True) -> None:
        write_vtk(path, self.points, self.cells, dict(self.cell_data), binary=binary)


_NODES_PER_TYPE = {1: 1, 3: 2, 5: 3, 9: 4, 10: 4, 12: 8, 13: 6, 14: 5}


def write_vtk(path: str, points: np.ndarray, cells, cell_data: dict | None = None, binary: bool = True,
              title: str = "nofluidx3d_gb300 cell") -> None:
    """Write a legacy VTK unstructured grid. cells: list of (vtk type, (n, k) int array) or a
    single (Nt, 4) tetra array."""
    if isinstance(cells, np.ndarray):
        cells = [(VTK_TETRA, cells)]
    pts = np.asarray(points, dtype=np.float64)
    ncell = sum(c.shape[0] for _, c in cells)
    size = sum(c.shape[0] * (c.shape[1] + 1) for _, c in cells)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        enc = "BINARY" if binary else "ASCII"
        f.write(f"# vtk DataFile Version 3.0\n{title}\n{enc}\nDATASET UNSTRUCTURED_GRID\n".encode())
        f.write(f"POINTS {pts.shape[0]} double\n".encode())
        if binary:
            f.write(pts.astype(">f8").tobytes())
            f.write(b"\n")
        else:
            np.savetxt(f, pts, fmt="%.17g")
        f.write(f"CELLS {ncell} {size}\n".encode())
        for _, c in cells:
            arr = np.concatenate([np.full((c.shape[0], 1), c.shape[1], np.int64), c.astype(np.int64)], axis=1)
            if binary:
                f.write(arr.astype(">i4").tobytes())
            else:
                np.savetxt(f, arr, fmt="%d")
        if binary:
            f.write(b"\n")
        f.write(f"CELL_TYPES {ncell}\n".encode())
        types = np.concatenate([np.full(c.shape[0], t, np.int64) for t, c in cells])
        if binary:
            f.write(types.astype(">i4").tobytes())
            f.write(b"\n")
        else:
            np.savetxt(f, types, fmt="%d")
        if cell_data:
            f.write(f"CELL_DATA {ncell}\n".encode())
            for name, arr in cell_data.items():
                a = np.asarray(arr, dtype=np.float64).reshape(ncell, -1)
                ncomp = a.shape[1]
                f.write(f"SCALARS {name} double {ncomp}\nLOOKUP_TABLE default\n".encode())
                if binary:
                    f.write(a.astype(">f8").tobytes())
                    f.write(b"\n")
                else:
                    np.savetxt(f, a, fmt="%.17g")
    os.replace(tmp, path)


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0

    def line(self) -> str:
        while True:
            e = self.d.find(b"\n", self.p)
            if e < 0:
                e = len(self.d)
            s = self.d[self.p:e].decode("latin-1").strip()
            self.p = e + 1
            if s or self.p >= len(self.d):
                return s

    def ascii_values(self, n: int, dtype) -> np.ndarray:
        out = []
        while len(out) < n:
            out.extend(self.line().split())
        return np.array(out[:n], dtype=dtype)

    def binary_values(self, n: int, dtype: str) -> np.ndarray:
        nb = n * np.dtype(dtype).itemsize
        a = np.frombuffer(self.d, dtype=dtype, count=n, offset=self.p)
        self.p += nb
        if self.p < len(self.d) and self.d[self.p:self.p + 1] == b"\n":
            self.p += 1
        return a.astype(np.float64 if dtype[1] == "f" else np.int64)


_VTK_TYPES = {"float": ">f4", "double": ">f8", "int": ">i4", "vtktypeint32": ">i4", "long": ">i8",
              "vtktypeint64": ">i8", "unsigned_int": ">u4"}


def read_vtk(path: str) -> VtkMesh:
    """Read a legacy VTK unstructured grid (ASCII or BINARY)."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    if not r.line().startswith("# vtk DataFile"):
        raise ValueError(f"{path}: not a legacy VTK file")
    r.line()  # title
    enc = r.line().upper()
    binary = enc == "BINARY"
    if r.line().upper() != "DATASET UNSTRUCTURED_GRID":
        raise ValueError(f"{path}: only UNSTRUCTURED_GRID datasets are supported")
    points = None
    flat = None
    types = None
    cell_data = _CellData()
    ncell = 0
    while r.p < len(r.d):
        ln = r.line()
        if not ln:
            break
        tok = ln.split()
        key = tok[0].upper()
        if key == "POINTS":
            n, t = int(tok[1]), tok[2].lower()
            v = r.binary_values(3 * n, _VTK_TYPES[t]) if binary else r.ascii_values(3 * n, np.float64)
            points = v.reshape(n, 3).astype(np.float64)
        elif key == "CELLS":
            n, size = int(tok[1]), int(tok[2])
            flat = r.binary_values(size, ">i4") if binary else r.ascii_values(size, np.int64)
            ncell = n
        elif key == "CELL_TYPES":
            n = int(tok[1])
            types = r.binary_values(n, ">i4") if binary else r.ascii_values(n, np.int64)
        elif key == "CELL_DATA":
            ncell = int(tok[1])
        elif key == "SCALARS":
            name, t = tok[1], tok[2].lower()
            ncomp = int(tok[3]) if len(tok) > 3 else 1
            if r.line().upper().startswith("LOOKUP_TABLE"):
                pass
            cnt = ncell * ncomp
            v = r.binary_values(cnt, _VTK_TYPES[t]) if binary else r.ascii_values(cnt, np.float64)
            cell_data[name] = v.reshape(ncell, ncomp).squeeze()
        elif key in ("POINT_DATA", "FIELD", "METADATA"):
            break  # point data and field arrays are not needed
    if points is None or flat is None or types is None:
        raise ValueError(f"{path}: missing POINTS/CELLS/CELL_TYPES")
    cells = []
    i = 0
    conn_by_type: dict = {}
    for t in types:
        k = int(flat[i])
        conn_by_type.setdefault(int(t), []).append(flat[i + 1:i + 1 + k])
        i += k + 1
    for t, rows in conn_by_type.items():
        cells.append((t, np.array(rows, dtype=np.int64)))
    return VtkMesh(points=points, cells=cells, cell_data=cell_data)
