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
