"""Size-independent properties at the benchmark's full size (the R = 64 cell, 6,594,816 tetra),
where the FP64 oracle is too slow for a long comparison.

* Momentum: the element forces are internal (each tetrahedron's four corner forces sum to zero,
  f0 = -(f1 + f2 + f3), tetra.cl:159-168), so with no contact and unit masses the total velocity
  of a freely vibrating cell stays zero whatever the damping (VelocityVerlet.cl: v' = a v + hb
  (f + f_old) sums to a Σv + hb (Σf + Σf_old)); the fixed-point accumulation keeps each node's sum
  exact, so only per-node FP32 roundings remain.
* Rigid motion: a translated cell is unstrained, so the element pass leaves it at rest; a rotated
  one is unstrained too (objectivity), up to the FP32 rounding of its rotated edges.
"""

import numpy as np
import pytest

from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import plain_large

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big_mesh():
    return plain_large().mesh()


def free_cell(mesh, model_args=(0, 2.4e-3, 0.41, 0.833)) -> CellSim:
    """The R = 64 mesh, Mooney-Rivlin, no contact, damped unit-mass velocity Verlet."""
    s = CellSim(0)
    s.set_mesh(mesh.points, mesh.tets)
    s.set_tetra(*model_args)
    s.set_integrator(0.01)
    return s


def test_momentum_of_a_free_vibrating_cell_stays_zero(big_mesh):
    m = big_mesh
    s = free_cell(m)
    X = m.points
    # a smooth, non-rigid initial displacement of about 1e-2 lattice units
    u = 1e-2 * np.stack([np.sin(X[:, 1] / 9.0), np.sin(X[:, 2] / 11.0), np.sin(X[:, 0] / 7.0)], axis=1)
    s.set_points(X + u)
    s.step(300)
    assert s.status() == 0
    v = s.velocities()
    scale = np.abs(v).sum(axis=0)
    assert np.all(scale > 0)  # the cell vibrates
    drift = np.abs(v.sum(axis=0)) / scale
    print(f"R64 free vibration, 300 steps: |sum v| / sum |v| per axis {drift}")
    assert np.all(drift < 1e-5)
    s.close()


def test_translated_cell_stays_at_rest(big_mesh):
    m = big_mesh
    s = free_cell(m)
    s.set_points(m.points + np.array([0.25, -0.5, 0.125]))
    s.step(50)
    assert s.status() == 0
    v = s.velocities()
    print(f"R64 translated cell, 50 steps: max |v| {np.abs(v).max():.3e}")
    assert np.abs(v).max() < 1e-9
    s.close()


def test_rotated_cell_is_nearly_unstressed(big_mesh):
    """Objectivity of the finite-strain law: a cell turned rigidly by 0.3 rad is unstrained
    (F = R, E = F F^T - I = 0), so after 20 steps its nodes move by FP32 rounding only — three
    orders of magnitude less than those of the same cell given a 1e-2 strain instead."""
    m = big_mesh
    X = m.points
    c, sn = np.cos(0.3), np.sin(0.3)
    R = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]])
    a = free_cell(m)
    a.set_points(X @ R.T)
    a.step(20)
    b = free_cell(m)
    b.set_points(X * np.array([1.01, 1.0, 1.0]))  # 1 % stretch along x
    b.step(20)
    assert a.status() == 0 and b.status() == 0
    va, vb = np.abs(a.velocities()).max(), np.abs(b.velocities()).max()
    print(f"R64 rotated cell, 20 steps: max |v| {va:.3e}; stretched cell {vb:.3e}")
    assert vb > 0
    assert va < 1e-3 * vb
    a.close()
    b.close()
