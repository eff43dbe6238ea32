"""Surrogate MLP kernels (nfx_mlp_*, BF16 operands, FP32 accumulation) against the CPU oracle
(oracle/mlp.py, same rounding points): forward, parameter and input gradients, AdamW, and that
on-device training and input fitting converge."""

import numpy as np
import pytest

from oracle import mlp as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def net():
    from nofluidx3d_gb300.mlp import MLP

    shape = M.MLPShape(n_in=6, width=256, depth=3, n_out=64)
    m = MLP(6, 256, 3, 64, max_batch=512)
    p = shape.init(7)
    m.set_params(p)
    yield shape, m, p
    m.close()


@pytest.mark.parametrize("B", [1, 37, 256])
def test_forward_matches_oracle(net, B):
    shape, m, p = net
    m.set_params(p)
    x = np.random.default_rng(B).uniform(-1, 1, (B, 6)).astype(np.float32)
    y = m.forward(x)
    y_ref, _ = M.forward(shape, p, x)
    # same bf16 rounding points; only the fp32 summation order differs (an activation may land
    # one bf16 ulp apart)
    assert rel(y, y_ref) < 5e-3


@pytest.mark.parametrize("B", [37, 256])
def test_gradients_match_oracle(net, B):
    shape, m, p = net
    m.set_params(p)
    rng = np.random.default_rng(100 + B)
    x = rng.uniform(-1, 1, (B, 6)).astype(np.float32)
    t = rng.normal(0, 1, (B, 64)).astype(np.float32)
    w = rng.uniform(0.5, 2, B).astype(np.float32)
    loss, dx = m.backward(x, t, w, scale=1.0 / B, want_dx=True)
    g = m.grads()
    rows, g_ref, dx_ref = M.loss_and_grads(shape, p, x, t, w, scale=1.0 / B)
    assert rel(loss, rows) < 5e-3
    off = 0
    for (o, i) in shape.layers():
        gw, gb = g[off:off + o * i], g[off + o * i:off + o * i + o]
        rw, rb = g_ref[off:off + o * i], g_ref[off + o * i:off + o * i + o]
        assert rel(gw, rw) < 2e-2, (o, i)
        assert rel(gb, rb) < 2e-2, (o, i)
        off += o * i + o
    assert rel(dx, dx_ref) < 2e-2
    # the exact (float64, unrounded) gradient is close too
    _, g64, _ = M.loss_and_grads(shape, p, x, t, w, scale=1.0 / B, exact=True)
    assert rel(g, g64) < 3e-2


def test_adamw_matches_oracle(net):
    shape, m, p = net
    m.set_params(p)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (64, 6)).astype(np.float32)
    t = rng.normal(0, 1, (64, 64)).astype(np.float32)
    m.backward(x, t, scale=1.0 / 64)
    g = m.grads()
    m.adamw(1e-3, 0.9, 0.999, 1e-8, 0.01)
    z = np.zeros_like(p)
    p1, _, _ = M.adamw(p, g, z, z, 1, 1e-3, 0.9, 0.999, 1e-8, 0.01, shape)
    np.testing.assert_allclose(m.params(), p1, rtol=1e-5, atol=1e-7)


def test_training_fits_smooth_map():
    from nofluidx3d_gb300.mlp import MLP

    shape = M.MLPShape(n_in=6, width=256, depth=3, n_out=64)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (4096, 6)).astype(np.float32)
    s = np.linspace(0, 1, 64, dtype=np.float32)
    t = (x[:, :1] * s + 0.5 * x[:, 1:2] * s ** 2 + 0.3 * np.sin(2 * x[:, 2:3] + 3 * s) * x[:, 3:4]).astype(np.float32)
    with MLP(6, 256, 3, 64, max_batch=256) as m:
        m.set_params(shape.init(1))
        losses = m.train(x, t, steps=1500, batch=256, lr=2e-3, lr_min=1e-5, seed=3)
        assert np.isfinite(losses).all()
        assert losses[-50:].mean() < 0.02 * losses[:10].mean()
        y = m.forward(x[:512])
        assert rel(y, t[:512]) < 0.05


def test_fit_inputs_recovers_hidden_inputs(net):
    shape, m, p = net
    m.set_params(p)
    rng = np.random.default_rng(9)
    x_true = rng.uniform(-0.8, 0.8, (32, 6)).astype(np.float32)
    target = m.forward(x_true)
    x0 = np.zeros_like(x_true)
    x0[:, 5] = x_true[:, 5]  # one input known (fixed), the rest fitted
    mask = np.array([1, 1, 1, 1, 1, 0], bool)
    lo, hi = -np.ones(6, np.float32), np.ones(6, np.float32)
    loss0 = m.backward(x0, target)
    x, loss = m.fit_inputs(x0, target, mask, lo, hi, steps=600, lr=2e-2)
    assert np.all(x[:, 5] == x_true[:, 5])
    assert np.all(x <= 1) and np.all(x >= -1)
    assert np.median(loss) < 1e-3 * np.median(loss0)


def test_output_gain_matches_oracle(net):
    shape, m, p = net
    m.set_params(p)
    m.set_output_gain(0, 1.6)
    try:
        rng = np.random.default_rng(21)
        x = rng.uniform(-1, 1, (45, 6)).astype(np.float32)
        t = rng.normal(0, 1, (45, 64)).astype(np.float32)
        y = m.forward(x)
        y_ref, _ = M.forward(shape, p, x, gain=(0, 1.6))
        assert rel(y, y_ref) < 5e-3
        loss, dx = m.backward(x, t, scale=1.0 / 45, want_dx=True)
        rows, g_ref, dx_ref = M.loss_and_grads(shape, p, x, t, scale=1.0 / 45, gain=(0, 1.6))
        assert rel(loss, rows) < 5e-3
        assert rel(m.grads(), g_ref) < 2e-2
        assert rel(dx, dx_ref) < 2e-2
    finally:
        m.set_output_gain(-1, 0.0)
