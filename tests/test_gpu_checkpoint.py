"""Checkpoint/resume of the full state and the inverted-element status, on the GPU.

The reference's only restart reloads node positions from a VTK frame
(nofluidx3d/SimulationLegacy.py:103-112) and loses velocities, forces and plastic state; its only
failure check is a host NaN/Inf test on positions at output time (nofluidx3d/util/IO.py:17-28).
Here a checkpoint holds the whole state, so a resumed run must equal the continuous run bit for
bit, and an element turned inside out on the host raises NFX_STATUS_INVERTED on the first step,
in a batch only on the cell it belongs to.
"""

import numpy as np
import pytest

from nofluidx3d_gb300.core import Batch, CellSim, NfxError
from nofluidx3d_gb300.workloads import Workload

pytestmark = pytest.mark.gpu

STATUS_INVERTED = 2


def vp_sphere(radius: float = 4.0) -> Workload:
    return Workload("checkpoint R4 MR+VP sphere", radius=radius, material="mr_vp", indenter="sphere",
                    sphere_radius=2.0, speed=1e-3, d0=None, record_every=50, steps=600)


def state(sim: CellSim) -> dict:
    return dict(points=sim.points_soa(), vel=sim.velocities(), fold=sim.force_old(), fp=sim.plastic_tensor_soa(),
                strain=sim.tet_field(2), curve=sim.curve(), time=sim.time, status=sim.status())


def assert_same(a: dict, b: dict):
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_resume_from_checkpoint_equals_continuous_run():
    w = vp_sphere()
    m = w.mesh()
    a = CellSim(0)
    w.configure(a, m, max_rows=20)
    a.step(150)  # a graph chunk and a partial one
    ck = a.checkpoint()
    a.step(250)
    cont = state(a)
    assert cont["curve"].shape[0] == 8 and cont["curve"][-1, 2] > 0  # rows at t = 0, 50, ..., 350; indenting

    b = CellSim(0)
    w.configure(b, m, max_rows=20)
    b.step(30)  # a different history, overwritten by the restore
    b.restore(ck)
    assert b.time == 150
    b.step(250)
    assert_same(cont, state(b))

    # rewinding the first handle to its own checkpoint reproduces the run as well
    a.restore(ck)
    a.step(250)
    assert_same(cont, state(a))
    a.close()
    b.close()


def test_checkpoint_refuses_another_mesh_or_model():
    w = vp_sphere()
    a = CellSim(0)
    w.configure(a, max_rows=20)
    a.step(10)
    ck = a.checkpoint()
    other = CellSim(0)
    w.with_(radius=3.0).configure(other, max_rows=20)
    with pytest.raises(NfxError):
        other.restore(ck)
    elastic = CellSim(0)
    w.with_(material="mr").configure(elastic, max_rows=20)
    with pytest.raises(NfxError):
        elastic.restore(ck)
    with pytest.raises(NfxError):
        a.restore(ck[:100])  # truncated
    for s in (a, other, elastic):
        s.close()


def test_plastic_tensor_round_trip():
    w = vp_sphere(3.0)
    sim = CellSim(0)
    w.configure(sim, max_rows=20)
    sim.step(300)
    fp = sim.plastic_tensor_soa()
    assert np.abs(fp - np.repeat(np.eye(3).reshape(9), sim.nt)).max() > 0  # plastic flow happened
    strain = sim.tet_field(2)
    sim.set_plastic_tensor_soa(fp)
    assert np.array_equal(sim.plastic_tensor_soa(), fp)
    assert np.array_equal(sim.tet_field(2), strain)
    ident = np.repeat(np.eye(3).reshape(9), sim.nt)
    sim.set_plastic_tensor_soa(ident)
    assert np.array_equal(sim.plastic_tensor_soa(), ident)
    sim.close()


def invert_one_tetra(points: np.ndarray, tets: np.ndarray, t: int = 0) -> np.ndarray:
    """Reflect corner 0 of tetra t through the plane of its other three corners."""
    p = np.array(points, np.float64)
    a, b, c, d = (p[k] for k in tets[t])
    n = np.cross(c - b, d - b)
    n /= np.linalg.norm(n)
    p[tets[t][0]] = a - 2.0 * np.dot(a - b, n) * n
    return p


def test_inverted_element_raises_status():
    w = Workload("inverted R3 NH plane", radius=3.0, material="nh", speed=1e-3)
    m = w.mesh()
    sim = CellSim(0)
    w.configure(sim, m, max_rows=4)
    sim.step(1)
    assert sim.status() == 0
    sim.set_points(invert_one_tetra(sim.points(), m.tets))
    sim.step(1)
    assert sim.status() & STATUS_INVERTED
    sim.close()


def test_inverted_element_quarantines_only_its_cell():
    w = Workload("inverted R3 MR+VP sphere", radius=3.0, material="mr_vp", indenter="sphere", sphere_radius=1.5,
                 speed=1e-3, d0=None)
    m = w.mesh()
    b = Batch(0, tile_tets=128)
    c0 = w.add_to_batch(b, m)
    c1 = w.add_to_batch(b, m, like=c0)
    b.set_record(1, 50, 8)
    b.finalize()
    b.step(1)
    assert b.status() == 0
    b.set_points(c0, invert_one_tetra(b.points(c0), m.tets))
    b.step(1)
    st = b.cell_status()
    assert st[c0] & STATUS_INVERTED
    assert st[c1] == 0
    b.close()
