"""The learned part end to end on the small protocol (radius-8 cell, 2,400 steps per curve): the
batched simulator generates curves, the MLP kernels train on them, and the surrogate-assisted
inverse fit reaches the plain simulator-only fit's error with several times fewer full
simulations. Every error is measured by the simulator, not by the network."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def experiment():
    from nofluidx3d_gb300 import surrogate as S

    return S.run_experiment(S.SMALL, n_curves=4096, n_hold=512, n_targets=32, n_plain=32, train_steps=20000,
                            batch=256, seed=0, log=lambda *a: None)


def test_simulated_curves_match_the_plain_path():
    """simulate_curves (batched, shared mesh) equals CellSim runs of the same inputs (inputs from
    the softer half of the box, well inside the scheme's stability limit; no roughness filter)."""
    import dataclasses

    from nofluidx3d_gb300 import surrogate as S
    from nofluidx3d_gb300.core import CellSim

    proto = dataclasses.replace(S.SMALL, max_roughness=float("inf"))
    rng = np.random.default_rng(11)
    P = S.from_unit(rng.uniform(-0.8, 0.2, (3, 6)), proto)
    F = S.simulate_curves(P, proto)
    mesh = proto.mesh()
    rows = proto.steps // proto.record_every + 1
    for i in range(3):
        s = CellSim(0)
        S.workload(P[i], proto).configure(s, mesh, max_rows=rows)
        s.step(proto.steps)
        s.record_now()
        c = s.curve()
        np.testing.assert_array_equal(np.interp(proto.depths(), c[:, 1], c[:, 2]), F[i])
        s.close()
    assert np.all(np.isfinite(F)) and np.all(F[:, -1] > 0)


def test_surrogate_learns_the_curves(experiment):
    # inputs past the explicit scheme's stability limit (stiff corner of the box) and, on this
    # small cell with few nodes in contact, jagged curves are discarded
    assert experiment["dataset"]["non_finite"] <= 0.35 * experiment["dataset"]["curves"]
    assert experiment["held_out_curve_error"]["median"] < 0.08


def test_surrogate_fit_needs_fewer_simulations(experiment):
    fit = experiment["inverse_fit"]
    # a final error (measured by the simulator) no worse than the simulator-only fit's ...
    assert fit["surrogate"]["error"]["median"] <= fit["plain"]["error"]["median"] * 1.1 + 1e-3
    # ... with at least ten times fewer full simulations
    assert fit["sims_ratio_plain_over_surrogate"] >= 10.0
