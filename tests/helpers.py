"""Test helpers: map a workload onto the CPU oracle, compare trajectories and curves."""

from __future__ import annotations

import numpy as np

import oracle as O
from nofluidx3d_gb300.workloads import Workload


def oracle_problem(w: Workload, mesh=None) -> O.Problem:
    m = mesh if mesh is not None else w.mesh()
    contacts = [O.Contact(c["kind"], c["k"], p0=c["p0"], v=c["v"], tmove=min(c["tmove"], 1e300), radius=c["radius"])
                for c in w.contacts(m)]
    integ = dict(integrator=O.INTEGRATOR_VV2 if w.integrator == "vv2" else O.INTEGRATOR_VV, density=w.density)
    if w.material == "mr_vp":
        return O.Problem(m.points, m.tets, model=O.MODEL_VP, vp_par=w.vp_params(), contacts=contacts, xi=w.xi,
                         record_contact=w.record_contact, **integ)
    model, E, nu, mr = w.tetra_params()
    return O.Problem(m.points, m.tets, model=model, E=E, nu=nu, mr=mr, contacts=contacts, xi=w.xi,
                     record_contact=w.record_contact, **integ)


def rel_traj(x_ref: np.ndarray, x: np.ndarray) -> float:
    """||x - x_ref|| / ||x_ref|| over all node coordinates."""
    return float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref))


def rel_disp(x_ref: np.ndarray, x: np.ndarray, X: np.ndarray) -> float:
    """Relative error of the displacement field x - X."""
    return float(np.linalg.norm(x - x_ref) / max(np.linalg.norm(x_ref - X), 1e-300))


def rel_curve(c_ref: np.ndarray, c: np.ndarray) -> float:
    """Relative L2 error of the force column of two force-depth curves with the same rows."""
    assert c_ref.shape == c.shape, (c_ref.shape, c.shape)
    assert np.array_equal(c_ref[:, 0], c[:, 0])
    return float(np.linalg.norm(c[:, 2] - c_ref[:, 2]) / max(np.linalg.norm(c_ref[:, 2]), 1e-300))
