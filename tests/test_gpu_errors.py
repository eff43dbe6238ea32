"""Invalid input through the C ABI on a live handle: every case is refused on the host with an
error code and a message, before any device work, and the handle stays usable afterwards (a
valid set-up on the same handle then steps with status 0). The reference has no such checks (an
out-of-range corner index or a non-finite position reaches its OpenCL kernels as is); these
pin the boundary's error behaviour."""

import numpy as np
import pytest

from nofluidx3d_gb300._lib import NfxError
from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import Workload

pytestmark = pytest.mark.gpu

W = Workload("errors R3 NH plane", radius=3.0, material="nh", speed=1e-3, record_every=50)


def usable(s: CellSim, m):
    """A valid set-up on the handle, stepped: the handle survived the refused calls."""
    W.configure(s, m, max_rows=4)
    s.step(20)
    assert s.status() == 0
    assert s.time == 20


def test_refused_mesh_inputs_leave_the_handle_usable():
    m = W.mesh()
    s = CellSim(0)
    with pytest.raises(NfxError, match="NFX_ERR_STATE"):
        s.step(1)  # no mesh yet
    bad = np.array(m.tets, copy=True)
    bad[5, 2] = m.num_points  # a corner index past the nodes
    with pytest.raises(NfxError, match="out of range"):
        s.set_mesh(m.points, bad)
    flat = np.array(m.tets, copy=True)
    flat[7, 3] = flat[7, 2]  # a repeated corner: zero reference volume
    with pytest.raises(NfxError, match="degenerate"):
        s.set_mesh(m.points, flat)
    pts = np.array(m.points, copy=True)
    pts[11, 1] = np.nan
    with pytest.raises(NfxError, match="non-finite"):
        s.set_mesh(pts, m.tets)
    usable(s, m)
    s.close()


def test_refused_parameters_leave_the_handle_usable():
    m = W.mesh()
    s = CellSim(0)
    s.set_mesh(m.points, m.tets)
    with pytest.raises(NfxError, match="unknown elastic model"):
        s.set_tetra(7, 1e-3, 0.3)
    with pytest.raises(NfxError, match="non-finite material"):
        s.set_tetra(0, float("inf"), 0.3)
    with pytest.raises(NfxError, match="non-finite viscoplastic"):
        s.set_viscoplastic([1e-3, 0.0, 1e-2, 1.0, float("nan"), 1e-3, 1.0, 0.0])
    with pytest.raises(NfxError, match="contact id out of range"):
        s.set_record(2, 50, 4)  # no contacts yet
    with pytest.raises(NfxError, match="NFX_ERR_STATE"):
        s.step(1)  # mesh but no material
    s.close()
    s = CellSim(0)
    usable(s, m)
    with pytest.raises(NfxError, match="contact id out of range"):
        s.set_contact_table(9, 0, np.zeros(4))
    with pytest.raises(NfxError, match="non-finite table position"):
        s.set_contact_table(0, s.time, np.array([0.0, np.inf]))
    s.step(10)  # the refused calls changed nothing the step reads
    assert s.status() == 0 and s.time == 30
    s.close()


def test_contact_limit():
    m = W.mesh()
    s = CellSim(0)
    s.set_mesh(m.points, m.tets)
    for _ in range(4):
        s.add_contact(0, 0.1, 0.0, -10.0, 0.0)
    with pytest.raises(NfxError, match="at most 4 contacts"):
        s.add_contact(0, 0.1, 0.0, -10.0, 0.0)
    s.close()
