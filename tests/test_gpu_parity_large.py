"""Viscoplastic parity on the large cells the benchmark runs, against the FP64 oracle.

Cases (Mooney-Rivlin + finite-strain viscoplastic law, sphere indenter at 1e-4 per step, the
plain-large construction of the benchmark at three radii):
  * R = 16 (103,536 tetra, sphere of radius 4), 10^4 steps — the surrogate's cell;
  * R = 34 (989,808 tetra, sphere of radius 16), 10^4 steps — the 1M-tetra headline cell;
  * R = 64 (6,594,816 tetra, sphere of radius 16), 2,000 steps — the benchmark's own cell.
The oracle runs in parallel in chunks of one record interval; the indenter-force row at each
record time is the reference's sphere penalty readout (Simulation.py:198-212) evaluated on the
oracle's positions at that time, which is what the device computes inside the step that starts at
that time. Reported per case: the trajectory error relative to the positions, the same error
relative to the displacement field (x - X, much smaller than x), and the relative L2 error of the
force curve. Bars: trajectory 1e-5, curve 1e-4 (the benchmark spec's); the displacement error is
held to 1e-3."""

import numpy as np
import pytest

import oracle as O
from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import plain_large
from tests.helpers import oracle_problem, rel_curve, rel_disp, rel_traj

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-5
DISP_TOL = 1e-3
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
    x = sim.points()
    traj = rel_traj(st.positions(), x)
    disp = rel_disp(st.positions(), x, m.points)
    cgpu = sim.curve()
    curve = rel_curve(cref, cgpu)
    sim.close()
    assert cref[-1, 2] > 0  # the sphere pressed into the cell
    err = np.abs(cgpu[:, 2] - cref[:, 2])
    k = int(np.argmax(err))
    print(f"R{R:g}: {n} steps, trajectory {traj:.3e}, displacement {disp:.3e}, curve {curve:.3e}; "
          f"largest row error {err[k]:.3e} at t = {cref[k, 0]:.0f} (force {cref[k, 2]:.4e}, peak {cref[:, 2].max():.4e})")
    return traj, disp, curve


def test_viscoplastic_sphere_r16_10k_steps_vs_fp64_oracle():
    traj, disp, curve = run_case(16.0, 4.0, 10000)
    assert traj < TRAJ_TOL
    assert disp < DISP_TOL
    assert curve < CURVE_TOL


def test_viscoplastic_sphere_r34_10k_steps_vs_fp64_oracle():
    """The 1M-tetra cell of the headline configuration (about two minutes of oracle time on 16
    host cores)."""
    traj, disp, curve = run_case(34.0, 16.0, 10000)
    assert traj < TRAJ_TOL
    assert disp < DISP_TOL
    assert curve < CURVE_TOL


def test_viscoplastic_sphere_r64_2k_steps_vs_fp64_oracle():
    """The benchmark's cell (6.6 M tetra) for 2,000 steps (about two and a half minutes of
    oracle time on 16 host cores): the sphere presses 0.2 lattice units into the cell."""
    traj, disp, curve = run_case(64.0, 16.0, 2000)
    assert traj < TRAJ_TOL
    assert disp < DISP_TOL
    assert curve < CURVE_TOL
