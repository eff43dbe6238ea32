"""Host logic of the surrogate module on the CPU: input scaling, the protocol, and the batched
Levenberg-Marquardt fit against an analytic stand-in for the simulator (so the fit logic and
its simulation accounting are checked without a GPU)."""

import numpy as np
import pytest

from nofluidx3d_gb300 import surrogate as S


def test_unit_box_round_trip():
    for proto in (S.FULL, S.SMALL):
        P = S.sample_params(200, proto, seed=3)
        lo, hi = proto.bounds()
        assert np.all(P >= lo * (1 - 1e-12)) and np.all(P <= hi * (1 + 1e-12))
        u = S.to_unit(P, proto)
        assert np.all(np.abs(u) <= 1 + 1e-12)
        np.testing.assert_allclose(S.from_unit(u, proto), P, rtol=1e-12)
    assert S.FULL.steps == 48000 and S.FULL.max_depth == pytest.approx(4.8)  # 4.8 at 1e-4 per step
    assert S.SMALL.steps == 2400
    assert S.FULL.bounds()[0][5] == 4.0 and S.FULL.bounds()[1][5] == 24.0  # indenter radius 4..24 at R = 16


def fake_sim(P, proto, stats=None):
    """A smooth stand-in for the indentation curve with the same six inputs."""
    P = np.asarray(P, np.float64).reshape(-1, 6)
    d = proto.depths()[None, :] / proto.max_depth
    mu, r, kr, Y, eta, Rs = (P[:, j:j + 1] for j in range(6))
    F = mu * np.sqrt(Rs) * (d ** 1.5 * (1 + 0.3 * r) + 0.05 * np.log(kr) * d) / (1 + (mu / Y) * d * eta)
    if stats is not None:
        stats.sims += P.shape[0]
    return F


def test_lm_fit_recovers_inputs_and_counts_simulations():
    proto = S.SMALL
    P_true = S.sample_params(12, proto, seed=5)
    T = fake_sim(P_true, proto)
    start = S.from_unit(np.zeros((12, 6)), proto)
    start[:, 5] = P_true[:, 5]
    st = S.SimStats()
    res = S.lm_fit(T, start, proto, max_iter=40, rtol=1e-6, stats=st, simulate=fake_sim)
    assert np.median(res.error) < 1e-3
    assert np.all(res.params[:, 5] == P_true[:, 5])  # the indenter radius is not fitted
    # 1 evaluation at the start, then 5 Jacobian columns + 1 trial per iteration
    np.testing.assert_array_equal(res.sims, 1 + 6 * res.iterations)
    assert st.sims == res.sims.sum()


def test_lm_fit_from_a_good_start_is_cheap():
    proto = S.SMALL
    P_true = S.sample_params(8, proto, seed=6)
    T = fake_sim(P_true, proto)
    near = S.from_unit(S.to_unit(P_true, proto) + 0.01 * np.r_[1, 1, 1, 1, 1, 0], proto)
    far = S.from_unit(np.zeros((8, 6)), proto)
    far[:, 5] = P_true[:, 5]
    a = S.lm_fit(T, near, proto, max_iter=40, simulate=fake_sim)
    b = S.lm_fit(T, far, proto, max_iter=40, simulate=fake_sim)
    assert a.sims.mean() < b.sims.mean()
    assert np.median(a.error) <= np.median(b.error) + 1e-3


def test_roughness_separates_smooth_and_jagged_curves():
    d = np.linspace(0, 1, 64)
    smooth = d ** 1.5
    jag = smooth + 0.05 * (np.arange(64) % 2)
    assert S.roughness(smooth) < 0.01
    assert S.roughness(jag) > S.FULL.max_roughness
