"""Parity of the CUDA step (through the C ABI) with the reference: golden vectors from the
reference's own kernels and the FP64 oracle run live. Tolerances are the spec bars:
node trajectories within 1e-5 relative, force-depth curves within 1e-4 relative (L2 over the
recorded rows); the FP32 kernels carry the displacement as hi+lo floats."""

import os

import numpy as np
import pytest

import oracle as O
from nofluidx3d_gb300.core import CellSim
from nofluidx3d_gb300.workloads import Workload, plain_small
from tests.golden.cases import CASES
from tests.helpers import oracle_problem, rel_curve, rel_disp, rel_traj

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

TRAJ_TOL = 1e-5
CURVE_TOL = 1e-4


def gpu_case(case, steps=None):
    w = case.workload
    sim = CellSim(0)
    m = w.configure(sim)
    if case.model is not None:
        model, E, nu, mr = w.tetra_params()
        sim.set_tetra(case.model, E, nu, mr)
    if case.fix_top_bottom:
        sim.set_integrator(w.xi, True)
    n = case.steps if steps is None else steps
    sim.step(n)
    sim.record_now()
    return sim, m


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(name):
    case = CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    sim, m = gpu_case(case)
    x = sim.points()
    c = sim.curve()
    assert sim.status() == 0
    assert rel_traj(g["points"], x) < TRAJ_TOL
    assert rel_disp(g["points"], x, m.points) < 1e-3
    assert rel_curve(g["curve"], c) < CURVE_TOL, (g["curve"], c)
    if "Fp" in g:
        Fp = sim.plastic_tensor_soa()
        np.testing.assert_allclose(Fp, g["Fp"], atol=1e-5)
    if case.fix_top_bottom:
        ids = [3, 4]
        assert np.all(x[ids, 0] == 0.0) and np.all(x[ids, 2] == 0.0)
    sim.close()


def test_gpu_plain_small_10k_steps_vs_fp64_oracle():
    """The plain small workload (R=8 NH, 13,056 tetra) for 10^4 steps against the FP64 oracle."""
    w = plain_small()
    n = 10000
    mesh = w.mesh()
    st = O.State(oracle_problem(w, mesh), "f64")
    cref = st.run(n, w.record_every)
    sim = CellSim(0)
    w.configure(sim, mesh)
    sim.step(n)
    sim.record_now()
    x = sim.points()
    c = sim.curve()
    assert sim.status() == 0
    e_traj = rel_traj(st.positions(), x)
    e_curve = rel_curve(cref, c)
    print(f"plain-small 1e4 steps: trajectory rel {e_traj:.3e}, curve rel {e_curve:.3e}")
    assert e_traj < TRAJ_TOL
    assert e_curve < CURVE_TOL
    sim.close()


def test_gpu_single_tetra_force():
    """One step from a deformed single tetra: the stored previous force equals the oracle's
    element force (tetra.cl) for NH, MR, SVK and SVKK."""
    X = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    T = np.array([[0, 1, 2, 3]])
    rng = np.random.default_rng(3)
    x = X + rng.uniform(-0.05, 0.05, X.shape)
    for model, mr in [(O.MODEL_MR, 1.0), (O.MODEL_MR, 0.7), (O.MODEL_SVK, 1.0), (O.MODEL_SVKK, 1.0)]:
        P = O.Problem(X, T, model=model, E=3e-3, nu=0.45, mr=mr, xi=0.0)
        st = O.State(P, "f64")
        st.points[:] = x.T.reshape(-1)
        st.run(1)
        sim = CellSim(0)
        sim.set_mesh(X, T)
        sim.set_tetra(model, 3e-3, 0.45, mr)
        sim.set_integrator(0.0)
        sim.set_points(x)
        sim.step(1)
        f_gpu = sim.force_old()
        f_ref = st.fold.reshape(3, -1).T
        np.testing.assert_allclose(f_gpu, f_ref, rtol=2e-4, atol=1e-9 * np.abs(f_ref).max())
        np.testing.assert_allclose(sim.points(), st.positions(), rtol=0, atol=1e-7)
        sim.close()


def test_gpu_graph_chunks_match_single_steps():
    w = CASES["nh_plane_R3"].workload
    a, b = CellSim(0), CellSim(0)
    w.configure(a)
    w.configure(b)
    a.step(250)  # two captured 100-step graphs + 50 single steps
    for _ in range(250):
        b.step(1)
    np.testing.assert_allclose(a.points(), b.points(), rtol=0, atol=1e-6)
    a.record_now()
    b.record_now()
    np.testing.assert_allclose(a.curve(), b.curve(), rtol=1e-4, atol=1e-12)
    a.close()
    b.close()


@pytest.mark.parametrize("name", ["nh_plane_R3", "vp_sphere_R3"])
def test_gpu_bitwise_reproducible(name):
    """Nodal forces accumulate as fixed-point integers and every reduction has a fixed order,
    so two runs of the same case agree to the bit."""
    w = CASES[name].workload
    runs = []
    for _ in range(2):
        sim = CellSim(0)
        w.configure(sim)
        sim.step(257)
        sim.record_now()
        runs.append((sim.points(), sim.velocities(), sim.curve(), sim.plastic_tensor_soa()))
        sim.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_gpu_indenter_force_equals_recorded_row():
    w = CASES["nh_plane_R3"].workload
    sim = CellSim(0)
    w.configure(sim)
    sim.step(100)
    f = sim.indenter_force(1)
    sim.record_now()
    c = sim.curve()
    assert c.shape[0] == 3 and c[-1, 0] == 100
    assert f == c[-1, 2]
    sim.close()


def test_gpu_contact_table_equals_schedule():
    """Per-step positions from a host table (arbitrary wallFunc) give the same run as the
    on-device linear schedule."""
    w = CASES["nh_plane_R3"].workload
    a, b = CellSim(0), CellSim(0)
    w.configure(a)
    w.configure(b)
    c = w.contacts()[1]
    t = np.arange(0, 300, dtype=np.float64)
    b.set_contact_table(1, 0, c["p0"] - c["v"] * t)
    a.step(300)
    b.step(300)
    np.testing.assert_allclose(a.points(), b.points(), rtol=0, atol=1e-6)
    a.close()
    b.close()


def test_gpu_nonfinite_input_raises_status():
    w = CASES["nh_plane_R3"].workload
    sim = CellSim(0)
    m = w.configure(sim)
    x = m.points.copy()
    x[10, 1] = np.nan
    sim.set_points(x)
    sim.step(2)
    assert sim.status() & 1
    sim.close()


def test_sphere_integral_readout_in_step_equals_on_demand():
    """The integrated sphere's force row at t = 100 recorded inside step 100 (tile partials from
    the step's sphere pass) equals the row recorded between steps (its readout pass) and the
    on-demand readout, bit for bit."""
    w = CASES["mr_sphereint_R3"].workload
    a, b = CellSim(0), CellSim(0)
    w.configure(a, max_rows=10)
    w.configure(b, max_rows=10)
    a.step(101)
    b.step(100)
    b.record_now()
    ra, rb = a.curve()[2], b.curve()[2]
    assert ra[0] == 100 and rb[0] == 100
    assert np.array_equal(ra, rb)
    assert b.indenter_force(1) == rb[2]
    assert rb[2] > 0
    a.close()
    b.close()


def test_gpu_viscoplastic_sphere_10k_steps_vs_fp64_oracle():
    """R=8 Mooney-Rivlin + viscoplastic cell under a sphere of radius 2, 10^4 steps, against the
    FP64 oracle, at the bars of 1e-5 (trajectories) and 1e-4 (force curve); a direct FP32 port of
    the reference reaches 1.8e-5 and 1.4e-2 here."""
    from nofluidx3d_gb300.workloads import plain_large

    w = plain_large().with_(name="R8 VP sphere", radius=8.0, sphere_radius=2.0, speed=1e-4, record_every=100)
    m = w.mesh()
    n = 10000
    st = O.State(oracle_problem(w, m), "f64")
    cref = st.run(n, w.record_every)  # serial FP64 (about 20 s)
    sim = CellSim(0)
    w.configure(sim, m, max_rows=n // w.record_every + 2)
    sim.step(n)
    sim.record_now()
    assert sim.status() == 0
    traj, curve = rel_traj(st.positions(), sim.points()), rel_curve(cref, sim.curve())
    print(f"R8 VP sphere 1e4 steps: trajectory {traj:.3e} curve {curve:.3e}")
    assert traj < TRAJ_TOL
    assert curve < CURVE_TOL
    sim.close()


@pytest.mark.parametrize("model,label", [(O.MODEL_SVK, "SVK"), (O.MODEL_SVKK, "SVKK"), (O.MODEL_MR, "MR")])
def test_gpu_elastic_laws_sphere_10k_steps_vs_fp64_oracle(model, label):
    """The other elastic laws of tetra.cl over the parity bars' horizon: Saint-Venant-Kirchhoff
    (:94-114), its Kellnberger variant (:76-93, ten Newton steps of the polar factor) and
    Mooney-Rivlin (:115-168, mr ratio 0.8) on the R=8 cell under a sphere of radius 2, 10^4 steps
    against the FP64 oracle; the golden cases run these laws for a few hundred steps only."""
    w = Workload(f"R8 {label} sphere", radius=8.0, material="mr", C10=4e-4, C01=1e-4, K=1e-2, indenter="sphere",
                 sphere_radius=2.0, speed=1e-4, d0=None, record_every=100)
    m = w.mesh()
    n = 10000
    _, E, nu, mr = w.tetra_params()
    prob = oracle_problem(w, m)
    prob.model = model
    st = O.State(prob, "f64")
    cref = st.run(n, w.record_every)
    sim = CellSim(0)
    w.configure(sim, m, max_rows=n // w.record_every + 2)
    sim.set_tetra(model, E, nu, mr)
    sim.step(n)
    sim.record_now()
    assert sim.status() == 0
    assert cref[-1, 2] > 0  # the sphere pressed into the cell
    traj, curve = rel_traj(st.positions(), sim.points()), rel_curve(cref, sim.curve())
    print(f"R8 {label} sphere 1e4 steps: trajectory {traj:.3e} curve {curve:.3e}")
    assert traj < TRAJ_TOL
    assert curve < CURVE_TOL
    sim.close()


@pytest.mark.parametrize("label", ["VV2 sphere", "integrated sphere"])
def test_gpu_integrator_and_contact_variants_10k_steps_vs_fp64_oracle(label):
    """The lumped-mass integrator (velocityVerlet2.cl, damping 0.05) and the integrated sphere
    contact (InteractionSphereIntegral.cl) on the R=8 Mooney-Rivlin cell over 10^4 steps against the
    FP64 oracle; the golden cases run them for a few hundred steps only."""
    base = Workload(f"R8 {label}", radius=8.0, material="mr", C10=4e-4, C01=1e-4, K=1e-2, speed=1e-4,
                    sphere_radius=2.0, record_every=100)
    w = (base.with_(indenter="sphere", d0=None, integrator="vv2", xi=0.05) if label == "VV2 sphere"
         else base.with_(indenter="sphere_integral", d0=0.3))
    m = w.mesh()
    n = 10000
    st = O.State(oracle_problem(w, m), "f64")
    cref = st.run(n, w.record_every)
    sim = CellSim(0)
    w.configure(sim, m, max_rows=n // w.record_every + 2)
    sim.step(n)
    sim.record_now()
    assert sim.status() == 0
    assert np.abs(cref[:, 2]).max() > 0
    traj, curve = rel_traj(st.positions(), sim.points()), rel_curve(cref, sim.curve())
    print(f"R8 {label} 1e4 steps: trajectory {traj:.3e} curve {curve:.3e}")
    assert traj < TRAJ_TOL
    assert curve < CURVE_TOL
    sim.close()
