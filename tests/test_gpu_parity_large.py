"""Viscoplastic 10^4-step parity on larger cells: the surrogate's R=16 cell (103,536 tetra) in the
GPU suite, and the 1M-tetra headline cell (R=34, 989,808 tetra) when NFX_LONG_TESTS=1 (about
three minutes of host time for the FP64 oracle). The oracle runs in parallel in chunks of one
record interval; the indenter-force row at each record time is the reference's sphere penalty
readout (Simulation.py:198-212) evaluated on the oracle's positions at that time, which is what
the device computes inside the step that starts at that time."""

import os

import numpy as np
import pytest

import oracle as O
from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import plain_large
from tests.helpers import oracle_problem, rel_curve, rel_traj

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-5
CURVE_TOL = 1e-4


def sphere_readout(x: np.ndarray, c: dict, t: int) -> float:
    """-sum of the sphere contact's y forces on the nodes at positions x (FP64)."""
    w = c["p0"] - c["v"] * min(float(t), c["tmove"])
    r = np.asarray(x, np.float64) - np.array([0.0, w, 0.0])
    ln = np.sqrt((r * r).sum(1))
    dis = np.maximum(c["radius"] - ln, 0.0)
    hit = dis > 0.0
    return float(-(c["k"] * dis[hit] * (r[hit, 1] / ln[hit])).sum())


def run_case(R: float, Rs: float, n: int):
    w = plain_large().with_(name=f"R{R:g} VP sphere", radius=R, sphere_radius=Rs, speed=1e-4, record_every=100)
    m = w.mesh()
    st = O.State(oracle_problem(w, m), "f64")
    c = w.contacts(m)[w.record_contact]
    rows = []
    for t in range(0, n + 1, w.record_every):
        if t > 0:
            st.run(w.record_every, parallel=True, threads=O.max_threads())
        rows.append((float(t), c["v"] * t, sphere_readout(st.positions(), c, t)))
    cref = np.array(rows)
    sim = CellSim(0)
    w.configure(sim, m, max_rows=n // w.record_every + 2)
    sim.step(n)
    sim.record_now()
    assert sim.status() == 0
    traj = rel_traj(st.positions(), sim.points())
    curve = rel_curve(cref, sim.curve())
    sim.close()
    assert cref[-1, 2] > 0  # the sphere pressed into the cell
    return traj, curve


def test_viscoplastic_sphere_r16_10k_steps_vs_fp64_oracle():
    """Measured on GB300: trajectory 1.4e-7, curve 9.9e-5 — close to the 1e-4 bar: a sphere of
    radius 4 presses few nodes hard, and its penalty force amplifies the FP32 error of the
    element forces in a quasi-static balance."""
    traj, curve = run_case(16.0, 4.0, 10000)
    print(f"R16: trajectory {traj:.3e} curve {curve:.3e}")
    assert traj < TRAJ_TOL
    assert curve < CURVE_TOL


@pytest.mark.skipif(os.environ.get("NFX_LONG_TESTS") != "1", reason="long: set NFX_LONG_TESTS=1")
def test_viscoplastic_sphere_r34_10k_steps_vs_fp64_oracle():
    """The 1M-tetra cell of the headline configuration (sphere of radius 16). Measured on GB300:
    trajectory 3.1e-8, curve 7.6e-5."""
    traj, curve = run_case(34.0, 16.0, 10000)
    print(f"R34: trajectory {traj:.3e} curve {curve:.3e}")
    assert traj < TRAJ_TOL
    assert curve < CURVE_TOL
