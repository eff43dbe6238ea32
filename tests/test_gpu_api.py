"""The reference-mirroring Python API (Simulation / TetraCell / interactions / writeVTK) on the
GPU, against the FP64 oracle. The config uses SI values that make the unit conversion the
identity (L0 = p0 = V0 = T0 = 1), so lattice parameters can be compared directly."""

import os

import numpy as np
import pytest

import oracle as O
from nofluidx3d_gb300.mesh import kuhn_sphere
from nofluidx3d_gb300.vtk import read_vtk, write_vtk
from nofluidx3d_gb300.workloads import nh_to_reference
from tests.helpers import rel_traj

pytestmark = pytest.mark.gpu


def make_config(tmp_path, R=3.0, frames=3, steps=150, model="NH"):
    mesh = kuhn_sphere(R, 0.02, 0)
    vtk = os.path.join(tmp_path, "cell.vtk")
    write_vtk(vtk, mesh.points, mesh.tets)
    E, nu = nh_to_reference(1e-3, 1e-2)
    cfg = {
        "gpu": 0, "RhoSI": 1.0, "SimulationTimeSI": float(steps), "VTKFramesTotal": frames,
        "OutputDir": os.path.join(tmp_path, "out") + "/", "InitialDistance": 0.0, "MoveTimeSI": 1e9,
        "VelocitySI": 1e-3, "SphereRadiusSI": 2.0,
        "CELL": {"RadiusSI": R, "RadiusSIM": R, "YoungsModulusSI": 1e-2, "PoissonRatio": nu, "model": model,
                 "InitVTK": vtk, "MooneyRivlinRatio": 1.0},
    }
    return cfg, mesh, E, nu


def test_simulation_run_matches_oracle(tmp_path):
    from nofluidx3d_gb300.Simulation import Simulation

    cfg, mesh, E, nu = make_config(str(tmp_path))
    sim = Simulation(cfg, verbose=False)
    assert sim.T0 == 1.0 and sim.L0 == 1.0 and sim.p0 == 1.0
    sim.setInteractionSubstrate()
    sim.setInteractionPlane()
    sim.setInteractionTetra()
    sim.setInteractionVelocityVerlet()
    data = sim.run()
    # oracle with the same interactions (reference damping 0.005)
    P = O.Problem(mesh.points, mesh.tets, model=O.MODEL_MR, E=1e-2 * (E / 1e-2), nu=nu, mr=1.0,
                  contacts=[O.Contact(O.SUBSTRATE, 0.1, p0=-3.0), O.Contact(O.PLANE, 0.1, p0=3.0, v=1e-3)],
                  xi=0.005, record_contact=1)
    P.E = cfg["CELL"]["YoungsModulusSI"] / sim.p0
    st = O.State(P, "f64")
    curve = st.run(150, 50)
    x = sim.points.readFromGPU().reshape(3, -1).T
    assert rel_traj(st.positions(), x) < 1e-5
    assert data.shape == (4, 3)
    np.testing.assert_allclose(data[:, 0], curve[:, 0])
    np.testing.assert_allclose(data[:, 1], curve[:, 1], rtol=1e-12)
    assert np.linalg.norm(data[:, 2] - curve[:, 2]) / np.linalg.norm(curve[:, 2]) < 1e-4
    # frames and simdata written
    frames = sorted(os.listdir(os.path.join(cfg["OutputDir"], "vtkfiles")))
    assert frames == ["frame0.vtk", "frame100.vtk", "frame150.vtk", "frame50.vtk"]
    f = read_vtk(os.path.join(cfg["OutputDir"], "vtkfiles", "frame150.vtk"))
    np.testing.assert_allclose(f.points, x)
    assert "vonMises" in f.cell_data
    assert os.path.exists(os.path.join(cfg["OutputDir"], "simdata.dat"))
    sim.close()


def test_callable_positions_match_device_schedule(tmp_path):
    """A plain Python wallFunc (evaluated on the host per step) gives the run of the built-in
    schedule that runs on the device."""
    from nofluidx3d_gb300.interactions import Plane
    from nofluidx3d_gb300.Simulation import Simulation

    cfg, mesh, E, nu = make_config(str(tmp_path))
    a = Simulation(cfg, verbose=False)
    b = Simulation(cfg, verbose=False)
    for s in (a, b):
        s.setInteractionSubstrate()
    a.setInteractionPlane(record=False)
    b.register(Plane(lambda t: 3.0 - 1e-3 * t, 0.1))
    for s in (a, b):
        s.setInteractionTetra()
        s.setInteractionVelocityVerlet()
    for _ in range(3):
        a.timeStep()
        b.timeStep()
    a._advance(120)
    b._advance(120)
    xa = a.points.readFromGPU().copy()
    xb = b.points.readFromGPU().copy()
    np.testing.assert_allclose(xa, xb, rtol=0, atol=1e-6)
    assert a.handle.indenter_force(1) == pytest.approx(b.handle.indenter_force(1), rel=1e-5)
    a.close()
    b.close()


def test_sphere_and_viscoplastic_plugins(tmp_path):
    from nofluidx3d_gb300.interactions import FiniteStrainViscoplastic
    from nofluidx3d_gb300.Simulation import Simulation

    cfg, mesh, E, nu = make_config(str(tmp_path), steps=100, frames=2)
    sim = Simulation(cfg, verbose=False)
    sim.setInteractionSubstrate()
    sphere = sim.setInteractionSphere()
    par = (1e-3, 2e-4, 1e-2, 1.0, 2e-4, 4e-3, 1.0, 0.0)
    sim.register(FiniteStrainViscoplastic(*par))
    sim.setInteractionVelocityVerlet(damping=1e-2)
    data = sim.run(writeStress=True, writePressure=True)
    P = O.Problem(mesh.points, mesh.tets, model=O.MODEL_VP, vp_par=par,
                  contacts=[O.Contact(O.SUBSTRATE, 0.1, p0=-3.0), O.Contact(O.SPHERE, 0.1, p0=5.0, v=1e-3, radius=2.0)],
                  xi=1e-2, record_contact=1)
    st = O.State(P, "f64")
    curve = st.run(100, 50)
    x = sim.points.readFromGPU().reshape(3, -1).T
    assert rel_traj(st.positions(), x) < 1e-5
    assert np.linalg.norm(data[:, 2] - curve[:, 2]) / np.linalg.norm(curve[:, 2]) < 1e-4
    # von Mises of the last step (written on the output interval) against the oracle's
    vm = sim.vonMises.readFromGPU()
    assert np.linalg.norm(vm - st.vonMises) / np.linalg.norm(st.vonMises) < 1e-3
    sim.close()
