"""Synthetic cell meshes and the per-tetra reference quantities the step needs.

The reference reads a tetrahedral cell mesh from a VTK file through pyvista
(nofluidx3d/TetraCell.py:13-23). The benchmark cells here are generated instead:
a cubic grid of spacing 1, every cube whose centre lies strictly inside a sphere of
radius R kept, and each cube split into the 6 Kuhn tetrahedra around its (0,0,0)-(1,1,1)
diagonal. Kuhn splits of neighbouring cubes share faces, so the mesh is conforming.
Interior nodes (all 8 surrounding cubes kept) are jittered uniformly by +-jitter per
coordinate from a seeded generator.

Node order follows the reference's conventions for a cell mesh:
  node 0 is the centre (TetraCell recentres on it, TetraCell.py:16-17),
  node 1 is the outermost node on the +x axis (TetraCell scales by its x, :19-20),
  node 2 the outermost on +z, node 3 the top pole (max y) and node 4 the bottom pole
  (min y): the nodes VelocityVerlet pins with FIXED_TOP_BOTTOM
  (nofluidx3d/kernels/Interactions/VelocityVerlet.cl:17-22).
The remaining nodes follow in lexicographic (x, y, z) grid order; tetrahedra follow their
cube in lexicographic order, 6 per cube. All tetrahedra are positively oriented:
(P1-P0).((P2-P0)x(P3-P0)) > 0, which the reference's Neo-Hookean/Mooney-Rivlin force needs
(tetra.cl:132 divides by the signed reference volume).
"""

from __future__ import annotations

from dataclasses import dataclass
from itertools import permutations

import numpy as np

__all__ = ["CellMesh", "kuhn_sphere", "edge_vectors", "signed_volumes", "mesh_counts"]


@dataclass
class CellMesh:
    """A tetrahedral cell: points (Np, 3) float64 and tets (Nt, 4) int64."""

    points: np.ndarray
    tets: np.ndarray
    radius: float = 0.0

    @property
    def num_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def num_tetra(self) -> int:
        return int(self.tets.shape[0])


_CORNERS = np.array(
    [[i, j, k] for i in (0, 1) for j in (0, 1) for k in (0, 1)], dtype=np.int64
)  # corner c = 4*i + 2*j + k


def _kuhn_local() -> np.ndarray:
    """The 6 Kuhn tetrahedra of the unit cube as corner indices, positively oriented."""
    tets = []
    for a, b, _c in permutations(range(3)):
        v0 = np.zeros(3, np.int64)
        v1 = v0.copy()
        v1[a] = 1
        v2 = v1.copy()
        v2[b] = 1
        v3 = np.ones(3, np.int64)
        verts = [v0, v1, v2, v3]
        d = np.linalg.det(np.array([verts[1] - verts[0], verts[2] - verts[0], verts[3] - verts[0]], float))
        if d < 0:
            verts[2], verts[3] = verts[3], verts[2]
        tets.append([int(4 * v[0] + 2 * v[1] + v[2]) for v in verts])
    return np.array(tets, dtype=np.int64)


_KUHN = _kuhn_local()


def _kept_cubes(radius: float) -> np.ndarray:
    n = int(np.ceil(radius)) + 1
    ax = np.arange(-n, n, dtype=np.int64)
    g = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    c = g.astype(np.float64) + 0.5
    keep = (c * c).sum(1) < radius * radius
    return g[keep]


def mesh_counts(radius: float) -> tuple[int, int, int]:
    """(cubes, tets, nodes) of the Kuhn sphere of this radius, without building it."""
    cubes = _kept_cubes(radius)
    corners = (cubes[:, None, :] + _CORNERS[None]).reshape(-1, 3)
    nodes = np.unique(corners, axis=0).shape[0]
    return int(cubes.shape[0]), int(6 * cubes.shape[0]), int(nodes)


def kuhn_sphere(radius: float, jitter: float = 0.02, seed: int = 0) -> CellMesh:
    """Kuhn-split sphere of the given radius (lattice units, grid spacing 1)."""
    cubes = _kept_cubes(radius)
    if cubes.shape[0] == 0:
        raise ValueError(f"radius {radius} keeps no cube")
    n = int(np.ceil(radius)) + 2
    span = 2 * n + 1

    def key(p):
        return ((p[..., 0] + n) * span + (p[..., 1] + n)) * span + (p[..., 2] + n)

    corners = cubes[:, None, :] + _CORNERS[None]          # (nc, 8, 3)
    ckeys = key(corners)                                   # (nc, 8)
    ukeys, inv = np.unique(ckeys.reshape(-1), return_inverse=True)
    inv = inv.reshape(ckeys.shape)
    # grid coordinates of every unique node (lexicographic because keys are)
    gx = ukeys // (span * span) - n
    gy = (ukeys // span) % span - n
    gz = ukeys % span - n
    grid = np.stack([gx, gy, gz], 1)

    # interior nodes: all 8 surrounding cubes kept
    count = np.bincount(inv.reshape(-1), minlength=ukeys.size)
    interior = count == 8

    # special nodes first (reference conventions, see module docstring)
    def pick(mask_axis_val):
        return int(np.flatnonzero(mask_axis_val)[0])

    on_x = (gy == 0) & (gz == 0)
    on_y = (gx == 0) & (gz == 0)
    on_z = (gx == 0) & (gy == 0)
    centre = pick(on_x & (gx == 0))
    xmax = int(np.flatnonzero(on_x)[np.argmax(gx[on_x])])
    zmax = int(np.flatnonzero(on_z)[np.argmax(gz[on_z])])
    ytop = int(np.flatnonzero(on_y)[np.argmax(gy[on_y])])
    ybot = int(np.flatnonzero(on_y)[np.argmin(gy[on_y])])
    special = [centre, xmax, zmax, ytop, ybot]
    rest = np.setdiff1d(np.arange(ukeys.size), special, assume_unique=False)
    order = np.concatenate([np.array(special, np.int64), rest])
    newid = np.empty_like(order)
    newid[order] = np.arange(order.size)

    pts = grid[order].astype(np.float64)
    intr = interior[order].copy()
    intr[0] = False  # keep the centre exact so recentring is a no-op
    if jitter > 0:
        rng = np.random.default_rng(seed)
        idx = np.flatnonzero(intr)
        pts[idx] += rng.uniform(-jitter, jitter, size=(idx.size, 3))

    local = newid[inv]                                     # (nc, 8) node ids per cube corner
    tets = local[:, _KUHN].reshape(-1, 4)                  # 6 per cube, cube order
    # orientation check (jitter of +-2% cannot flip a Kuhn tet, but verify)
    vol = signed_volumes(pts, tets)
    if np.any(vol <= 0):
        raise RuntimeError("generated mesh has non-positive tetra volumes")
    return CellMesh(points=pts, tets=tets.astype(np.int64), radius=float(radius))


def edge_vectors(points: np.ndarray, tets: np.ndarray, base: int = 0) -> np.ndarray:
    """Reference edge vectors per tetra as (Nt, 9) rows [R1 R2 R3].

    base=0 gives R_i = P_i - P_0 for i = 1, 2, 3, as TetraCell.calcEdgeVectors
    (nofluidx3d/TetraCell.py:33-38) and the elastic kernel (tetra.cl:40-42) use.
    base=3 gives R_i = P_i - P_3 for i = 0, 1, 2, the convention of the viscoplastic kernel,
    whose base node is its fourth corner (InteractionFiniteStrainViscoplastic.cl:18-22).
    """
    p = [points[tets[:, k]] for k in range(4)]
    if base == 0:
        e = [p[1] - p[0], p[2] - p[0], p[3] - p[0]]
    elif base == 3:
        e = [p[0] - p[3], p[1] - p[3], p[2] - p[3]]
    else:
        raise ValueError("base must be 0 or 3")
    return np.concatenate(e, axis=1)


def signed_volumes(points: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """R1.(R2 x R3)/6 with node-0 edges (nofluidx3d/TetraCell.py:40-41)."""
    p0 = points[tets[:, 0]]
    r1 = points[tets[:, 1]] - p0
    r2 = points[tets[:, 2]] - p0
    r3 = points[tets[:, 3]] - p0
    return np.einsum("ij,ij->i", r1, np.cross(r2, r3)) / 6.0
