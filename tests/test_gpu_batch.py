"""Batched cells (nfx_batch_*): every cell of a batch evolves exactly as the same cell run alone
through the plain path, and the autotuned batch agrees with the FP64 oracle."""

import numpy as np
import pytest

import oracle as O
from nofluidx3d_gb300.core import Batch, CellSim
from nofluidx3d_gb300.workloads import Workload, batched_cells
from tests.helpers import oracle_problem, rel_curve, rel_traj

pytestmark = pytest.mark.gpu


def small_population():
    cells = batched_cells(4, seed=7, r_range=(2.5, 4.0), steps=250)
    # faster indentation so short runs produce forces
    return [w.with_(speed=1e-3, record_every=50) for w in cells]


def test_batch_equals_cells_run_alone_bitwise(monkeypatch):
    """Same tile size as the plain path's default (128): same plans, and the same kernels (the
    plain path is a one-cell table), so every cell's state and curve match bit for bit."""
    monkeypatch.delenv("NFX_TILE_TETS", raising=False)
    cells = small_population()
    meshes = [w.mesh() for w in cells]
    b = Batch(0, tile_tets=128)
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 50, 10)
    b.finalize()
    b.step(250)  # five captured 50-step graphs
    b.record_now()
    assert b.status() == 0
    assert np.all(b.cell_status() == 0)
    for i, (w, m) in enumerate(zip(cells, meshes)):
        s = CellSim(0)
        w.configure(s, m, max_rows=10)
        s.step(250)
        s.record_now()
        assert s.status() == 0, i
        assert np.abs(s.curve()[:, 2]).max() > 0, i  # the cell touched the indenter
        assert np.array_equal(b.points(i), s.points()), i
        assert np.array_equal(b.curve(i), s.curve()), i
        s.close()
    b.close()


def test_batch_on_demand_readout_per_cell():
    """nfx_batch_indenter_force gives every cell's force, equal to the cell run alone."""
    cells = small_population()
    meshes = [w.mesh() for w in cells]
    b = Batch(0, tile_tets=128)
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 50, 10)
    b.finalize()
    b.step(120)
    got = b.indenter_force(1)
    assert got.shape == (4,)
    assert np.all(b.indenter_force(3) == 0.0)  # no cell has a fourth contact
    for i, (w, m) in enumerate(zip(cells, meshes)):
        s = CellSim(0)
        w.configure(s, m, max_rows=10)
        s.step(120)
        assert got[i] == s.indenter_force(1), i
        s.close()
    b.close()


def test_batch_autotuned_matches_oracle():
    cells = small_population()
    b = Batch(0, tile_tets=0)
    meshes = [w.mesh() for w in cells]
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 50, 10)
    b.finalize()
    info = b.info()
    assert info["tile_tets"] in (64, 128, 256)
    assert [t for t, _ in info["tuning"]] == [64, 128, 256]
    b.step(200)
    b.record_now()
    for i in (0, 3):
        st = O.State(oracle_problem(cells[i], meshes[i]), "f64")
        cref = st.run(200, 50)
        assert rel_traj(st.positions(), b.points(i)) < 1e-5
        assert rel_curve(cref, b.curve(i)) < 1e-4
    b.close()


def test_batch_rejects_mixed_models():
    b = Batch(0, tile_tets=128)
    w = Workload("x", radius=2.5, material="nh")
    m = w.mesh()
    c0 = b.add_cell(m.points, m.tets)
    c1 = b.add_cell(m.points, m.tets)
    b.set_tetra(c0, 0, 3e-3, 0.45, 1.0)
    with pytest.raises(Exception):
        b.set_viscoplastic(c1, (1e-3, 0, 1e-2, 1, 2e-4, 4e-3, 1, 0))
    b.close()


def test_batch_mixed_integrators_and_sphere_laws_bitwise():
    """Lumped-mass and unit-mass integrators, node-penalty and integrated spheres in one batch:
    each cell evolves exactly as it does alone."""
    base = Workload("mix", radius=3.0, material="mr", speed=1e-3, record_every=50, sphere_radius=2.0)
    cells = [base.with_(indenter="sphere", integrator="vv2", xi=0.05, seed=1),
             base.with_(indenter="sphere_integral", d0=0.3, seed=2),
             base.with_(indenter="sphere_integral", d0=0.3, integrator="vv2", xi=0.05, seed=3),
             base.with_(indenter="plane", seed=4)]
    meshes = [w.mesh() for w in cells]
    b = Batch(0, tile_tets=128)
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 50, 10)
    b.finalize()
    b.step(250)
    b.record_now()
    forces = b.indenter_force(1)
    assert b.status() == 0
    for i, (w, m) in enumerate(zip(cells, meshes)):
        s = CellSim(0)
        w.configure(s, m, max_rows=10)
        s.step(250)
        s.record_now()
        assert np.array_equal(b.points(i), s.points()), i
        assert np.array_equal(b.curve(i), s.curve()), i
        assert forces[i] == s.indenter_force(1), i
        s.close()
    b.close()


def test_cell_status_marks_only_the_failing_cell():
    """A cell that blows up physically (walls placed at +-R cut into a soft cell of non-integer
    radius; the FP64 oracle goes non-finite too) raises its own status; its neighbour stays 0."""
    pop = batched_cells(4, seed=7, r_range=(2.5, 4.0), steps=250)
    good = pop[0].with_(speed=1e-3)
    bad = pop[2].with_(speed=1e-3, d0=0.0)
    b = Batch(0, tile_tets=128)
    for w in (good, bad):
        w.add_to_batch(b, w.mesh())
    b.set_record(1, 50, 10)
    b.finalize()
    b.step(100)
    st = b.cell_status()
    assert st[0] == 0
    assert st[1] != 0
    assert b.status() == st[1]
    b.close()


def test_batch_material_corners_match_oracle():
    """The corners of the batched population's material box against the FP64 oracle, in one
    batch: the softest cell (shear modulus 2e-4, bulk/shear 5, yield 5e-5, viscosity 1e-2), whose
    nodal forces are the smallest the 2^-40 fixed-point accumulator has to resolve, the stiffest
    stable one and a middle one, each under its sphere for 2,000 steps."""
    base = batched_cells(1, seed=11, r_range=(5.0, 5.0), steps=2000)[0].with_(speed=2e-4, record_every=100)
    corners = [dict(C10=1e-4, K=1e-3, yield_stress=5e-5, viscosity=1e-2),      # mu = 2e-4, K/mu = 5
               dict(C10=2.5e-3, K=2.5e-2, yield_stress=1e-3, viscosity=1e-1),  # mu = 5e-3, K/mu = 5
               dict(C10=5e-4, K=2e-2, yield_stress=2e-4, viscosity=3e-2)]      # mu = 1e-3, K/mu = 20
    cells = [base.with_(seed=20 + i, **c) for i, c in enumerate(corners)]
    meshes = [w.mesh() for w in cells]
    b = Batch(0, tile_tets=128)
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 100, 30)
    b.finalize()
    b.step(2000)
    b.record_now()
    assert np.all(b.cell_status() == 0)
    for i, (w, m) in enumerate(zip(cells, meshes)):
        st = O.State(oracle_problem(w, m), "f64")
        cref = st.run(2000, 100)
        assert cref[-1, 2] > 0, i  # the sphere presses into the cell
        traj, curve = rel_traj(st.positions(), b.points(i)), rel_curve(cref, b.curve(i))
        print(f"corner {i}: trajectory {traj:.3e} curve {curve:.3e} peak force {cref[:, 2].max():.3e}")
        assert traj < 1e-5, i
        assert curve < 1e-4, i
    b.close()
