"""Synthetic Kuhn-sphere meshes and workload parameter mappings. CPU only."""

import numpy as np
import pytest

from nofluidx3d_gb300.mesh import edge_vectors, kuhn_sphere, mesh_counts, signed_volumes
from nofluidx3d_gb300.workloads import nh_to_reference, plain_large, plain_small


@pytest.mark.parametrize("R,expect", [(6, (912, 5472, 1285)), (8, (2176, 13056, 2849)),
                                      (16, (17256, 103536, 19789))])
def test_counts(R, expect):
    assert mesh_counts(R) == expect
    m = kuhn_sphere(R)
    assert (m.num_tetra, m.num_points) == expect[1:]


def test_conventions_and_orientation():
    m = kuhn_sphere(8, 0.02, 0)
    p = m.points
    np.testing.assert_array_equal(p[0], [0, 0, 0])
    np.testing.assert_array_equal(p[1], [8, 0, 0])
    np.testing.assert_array_equal(p[3], [0, 8, 0])
    np.testing.assert_array_equal(p[4], [0, -8, 0])
    v = signed_volumes(p, m.tets)
    assert v.min() > 0
    assert abs(v.sum() - 2176.0) < 1e-9  # jitter of interior nodes preserves the total volume
    # conforming: every interior face is shared by exactly two tets
    faces = np.sort(np.concatenate([m.tets[:, [0, 1, 2]], m.tets[:, [0, 1, 3]], m.tets[:, [0, 2, 3]],
                                    m.tets[:, [1, 2, 3]]]), axis=1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert set(np.unique(cnt)) <= {1, 2}


def test_jitter_is_seeded_and_bounded():
    a = kuhn_sphere(6, 0.02, 5)
    b = kuhn_sphere(6, 0.02, 5)
    c = kuhn_sphere(6, 0.02, 6)
    g = kuhn_sphere(6, 0.0)
    np.testing.assert_array_equal(a.points, b.points)
    assert not np.array_equal(a.points, c.points)
    d = np.abs(a.points - g.points)
    assert d.max() <= 0.02 and d.max() > 0.015


def test_edge_vector_bases():
    m = kuhn_sphere(4)
    e0 = edge_vectors(m.points, m.tets, 0)
    e3 = edge_vectors(m.points, m.tets, 3)
    np.testing.assert_allclose(e0[:, 0:3], m.points[m.tets[:, 1]] - m.points[m.tets[:, 0]])
    np.testing.assert_allclose(e3[:, 0:3], m.points[m.tets[:, 0]] - m.points[m.tets[:, 3]])


def test_nh_mapping_recovers_moduli():
    E, nu = nh_to_reference(1e-3, 1e-2)
    assert abs(E / (2 * (1 + nu)) - 1e-3) < 1e-15
    assert abs(E / (3 * (1 - 2 * nu)) - 1e-2) < 1e-15


def test_workload_definitions():
    s, l = plain_small(), plain_large()
    assert s.radius == 8 and s.steps == 20000 and s.record_every == 100
    assert l.radius == 64 and l.material == "mr_vp" and l.indenter == "sphere" and l.sphere_radius == 16
    par = l.vp_params()
    assert par[0] == 1e-3 and par[1] == 2e-4 and par[5] == pytest.approx(4e-3)


@pytest.mark.parametrize("R", [2.6, 3.6, 3.811, 6.5, 13.3, 17.0])
def test_batched_walls_start_tangent(R):
    """With d0 = None the substrate and the sphere start touching the bottom and top nodes and
    no node starts inside either wall, for integer and non-integer radii."""
    from nofluidx3d_gb300.workloads import batched_cells

    w = batched_cells(1, seed=3)[0].with_(radius=R, sphere_radius=R / 4.0)
    m = w.mesh()
    sub, sph = w.contacts(m)
    p = m.points
    assert sub["p0"] == pytest.approx(p[:, 1].min())
    assert sph["p0"] - sph["radius"] == pytest.approx(p[:, 1].max())
    assert np.all(p[:, 1] >= sub["p0"] - 1e-12)
    d = np.linalg.norm(p - np.array([0.0, sph["p0"], 0.0]), axis=1)
    assert d.min() >= sph["radius"] - 1e-12
    with pytest.raises(ValueError):
        w.contacts()  # d0 = None needs the mesh


def _plan_check(points: np.ndarray, tets: np.ndarray, tile: int) -> tuple[int, int]:
    import ctypes as C

    from nofluidx3d_gb300 import _lib

    L = _lib.load()
    P = np.ascontiguousarray(np.asarray(points, np.float64).T)   # SoA x..., y..., z...
    T = np.ascontiguousarray(np.asarray(tets, np.uint32).T)      # SoA corner 0..., 1..., 2..., 3...
    a, b = C.c_int64(), C.c_int64()
    _lib.check(L.nfx_plan_check(P.shape[1], T.shape[1], P.ctypes.data_as(C.c_void_p), T.ctypes.data_as(C.c_void_p),
                                tile, C.byref(a), C.byref(b)))
    return a.value, b.value


@pytest.mark.parametrize("tile", [64, 128, 256, 512])
def test_tile_plan_invariants(tile):
    """The host planner's tiles cover every tetra once, name the right nodes, and hold each node's
    corners in its incidence run (checked inside nfx_plan_check); region-grown tiles stay compact."""
    m = kuhn_sphere(12.0, 0.02, 0)
    ntiles, entries = _plan_check(m.points, m.tets, tile)
    # tiles close early only at the end of the curve or when the node cap binds (512-tetra tiles
    # have 256 node entries): at least 98 % of the slots hold a tetra
    assert -(-m.num_tetra // tile) <= ntiles and m.num_tetra / (ntiles * tile) > 0.98
    # each node entry of a tile costs a gather and three atomics; compact tiles share few nodes
    # (measured at R = 12: 0.605, 0.498, 0.421, 0.362 entries per tetra)
    assert entries / m.num_tetra < {64: 0.65, 128: 0.53, 256: 0.45, 512: 0.39}[tile]


def test_tile_plan_any_tetra_order():
    """Shuffled tetra order and a single tetra: the same invariants hold."""
    m = kuhn_sphere(6.0, 0.02, 1)
    rng = np.random.default_rng(5)
    _plan_check(m.points, np.asarray(m.tets)[rng.permutation(m.num_tetra)], 128)
    one = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    assert _plan_check(one, np.array([[0, 1, 2, 3]]), 128) == (1, 4)


def _star(n_ring: int) -> tuple[np.ndarray, np.ndarray]:
    """A node of very high valence: node 0 at the origin is a corner of every tetra, whose other
    corners are neighbouring triangles of a latitude-longitude sphere around it."""
    th = np.linspace(0.15, np.pi - 0.15, n_ring)
    ph = np.linspace(0.0, 2 * np.pi, 2 * n_ring, endpoint=False)
    pts = [[0.0, 0.0, 0.0]]
    for t in th:
        for p in ph:
            pts.append([np.sin(t) * np.cos(p), np.cos(t), np.sin(t) * np.sin(p)])
    pts = np.array(pts)
    idx = lambda i, j: 1 + i * len(ph) + (j % len(ph))  # noqa: E731
    tets = []
    for i in range(n_ring - 1):
        for j in range(len(ph)):
            for tri in ((idx(i, j), idx(i + 1, j), idx(i, j + 1)), (idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1))):
                a, b, c = (pts[k] for k in tri)
                tets.append((0, *tri) if np.dot(a, np.cross(b, c)) > 0 else (0, tri[0], tri[2], tri[1]))
    return pts, np.array(tets)


@pytest.mark.parametrize("tile", [64, 512])
def test_fixed_point_bound_covers_the_busiest_node(tile):
    """Every tile that lists a node adds one fixed-point tile sum to that node's 64-bit word; the
    planner shares the word's range out over the most tiles any node appears in, so that sums
    within the per-tile bound cannot wrap it. nfx_plan_check recounts the tiles per node and checks
    (tiles per node) x bound x 2^40 < 2^63. Here node 0 is a corner of all 2,574 tetrahedra and
    appears in dozens of tiles."""
    pts, tets = _star(40)
    assert len(tets) > 2000
    ntiles, _ = _plan_check(pts, tets, tile)
    assert ntiles >= len(tets) // tile
