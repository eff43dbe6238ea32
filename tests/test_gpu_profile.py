"""Timing helpers of the C ABI leave the simulation state as they found it."""

import numpy as np
import pytest

from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import Workload

pytestmark = pytest.mark.gpu


def test_profile_tet_pass_undoes_its_effects():
    """nfx_profile_tet_pass between steps: the viscoplastic cell then evolves bit for bit like a
    cell that was never profiled (forces, plastic state and the stress fields restored)."""
    w = Workload("vp_r4", 4.0, material="mr_vp", indenter="sphere", sphere_radius=3.0, speed=1e-3,
                 d0=None, record_every=50, steps=300)
    m = w.mesh()
    sims = []
    for profiled in (False, True):
        s = CellSim(0)
        w.configure(s, m, max_rows=10)
        s.step(149)  # the next step (end time 150) writes the stress fields
        if profiled:
            ms = s.profile_tet_pass(7)
            assert ms > 0.0
        s.step(151)
        s.record_now()
        assert s.status() == 0
        sims.append(s)
    a, b = sims
    assert np.abs(a.curve()[:, 2]).max() > 0
    assert np.array_equal(a.points(), b.points())
    assert np.array_equal(a.curve(), b.curve())
    assert np.array_equal(a.plastic_tensor_soa(), b.plastic_tensor_soa())
    for which in (0, 1, 2):
        assert np.array_equal(a.tet_field(which), b.tet_field(which))
    for s in sims:
        s.close()


def test_snapshot_matches_the_blocking_readback():
    """nfx_snapshot taken after 150 steps, with 150 more steps enqueued before waiting, holds the
    positions and force rows of step 150 bit for bit (a twin simulation stopped there reads them
    with the blocking getters); a second snapshot matches the blocking readback at step 300."""
    w = Workload("vp_r4", 4.0, material="mr_vp", indenter="sphere", sphere_radius=3.0, speed=1e-3,
                 d0=None, record_every=50, steps=300)
    m = w.mesh()
    a = CellSim(0)
    w.configure(a, m, max_rows=10)
    a.step(150)
    pts = np.empty(3 * a.np)
    rows = np.full((10, 3), np.nan)
    n = a.snapshot(pts, rows)
    a.step(150)  # runs while the snapshot is copied
    a.snapshot_wait()
    b = CellSim(0)
    w.configure(b, m, max_rows=10)
    b.step(150)
    assert n == b.curve().shape[0] == 3
    assert np.array_equal(pts, b.points_soa())
    assert np.array_equal(rows[:n], b.curve())
    pts2 = np.empty(3 * a.np)
    rows2 = np.full((10, 3), np.nan)
    n2 = a.snapshot(pts2, rows2)
    a.snapshot_wait()
    assert np.array_equal(pts2, a.points_soa())
    assert n2 == 6 and np.array_equal(rows2[:n2], a.curve())
    assert np.abs(rows2[:n2, 2]).max() > 0
    a.close()
    b.close()
