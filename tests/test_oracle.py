"""The CPU oracle against the reference's own kernels (golden vectors and, where the reference
tree is present, the live shim build). CPU only."""

import os

import numpy as np
import pytest

import oracle as O
from tests.golden.cases import CASES

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_f64_matches_golden(name):
    case = CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    st = O.State(case.problem(), "f64")
    curve = st.run(case.steps, case.workload.record_every)
    # same arithmetic in the same order as the reference kernels: equal to rounding of libm pow
    np.testing.assert_allclose(st.positions(), g["points"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(st.velocities(), g["velocities"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(curve, g["curve"], rtol=1e-10, atol=1e-16)
    if "Fp" in g:
        np.testing.assert_allclose(st.Fp, g["Fp"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(st.acc, g["acc"], rtol=1e-10, atol=1e-16)
        np.testing.assert_allclose(st.vonMises, g["vonMises"], rtol=1e-9, atol=1e-18)


@pytest.mark.skipif(not O.ref_available(), reason="reference kernels not built here (python oracle/build_ref.py)")
@pytest.mark.parametrize("name", ["nh_plane_R3", "vp_sphere_R3", "svkk_plane_R3", "nh_fixtb_R3"])
def test_oracle_bitwise_equals_reference_kernels(name):
    case = CASES[name]
    a = O.State(case.problem(), "f64")
    b = O.State(case.problem(), "f64")
    ca = a.run(120, 40)
    cb = O.ref_run(b, 120, 40)
    assert np.array_equal(a.points, b.points)
    assert np.array_equal(a.vel, b.vel)
    assert np.array_equal(ca, cb)
    if case.problem().model == O.MODEL_VP:
        assert np.array_equal(a.Fp, b.Fp)


def test_oracle_f32_close_to_f64():
    case = CASES["nh_plane_R3"]
    a = O.State(case.problem(), "f64")
    b = O.State(case.problem(), "f32")
    a.run(100)
    b.run(100)
    assert np.linalg.norm(a.positions() - b.positions()) / np.linalg.norm(a.positions()) < 1e-5


def test_planted_error_is_caught():
    """A wrong damping in the oracle run changes the result beyond the golden tolerance."""
    case = CASES["nh_plane_R3"]
    g = np.load(os.path.join(GOLDEN, "nh_plane_R3.npz"))
    p = case.problem()
    p.xi = p.xi * 1.01
    st = O.State(p, "f64")
    st.run(case.steps)
    assert np.abs(st.positions() - g["points"]).max() > 1e-9


def test_parallel_oracle_matches_serial():
    case = CASES["vp_sphere_R3"]
    a = O.State(case.problem(), "f64")
    b = O.State(case.problem(), "f64")
    a.run(50)
    b.run(50, parallel=True, threads=2)
    np.testing.assert_allclose(b.positions(), a.positions(), rtol=0, atol=1e-12)
