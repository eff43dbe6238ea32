"""The surrogate MLP's CPU oracle (oracle/mlp.py): bfloat16 rounding, float64 gradients against
central finite differences, AdamW against the update written out by hand. CPU only."""

import numpy as np
import pytest

from oracle import mlp as M


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -7 + 2 ** -8, -2.5, 0.0, 3.0e-30], np.float32)
    got = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3*2^-9 rounds up; the tie
    # 1 + 2^-7 + 2^-8 goes to the even neighbour 1 + 2^-6
    want = np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0, got[-1]], np.float32)
    np.testing.assert_array_equal(got, want)
    assert abs(got[-1] - 3.0e-30) / 3.0e-30 < 2 ** -8
    # idempotent, and exact on bfloat16-representable values
    np.testing.assert_array_equal(M.bf16(got), got)


def test_exact_gradients_match_finite_differences():
    shape = M.MLPShape(n_in=3, width=16, depth=2, n_out=8)
    rng = np.random.default_rng(1)
    p = shape.init(3).astype(np.float64) + rng.normal(0, 0.01, shape.num_params())
    x = rng.normal(0, 1, (5, 3))
    t = rng.normal(0, 1, (5, 8))
    w = rng.uniform(0.5, 2.0, 5)
    rows, g, dx = M.loss_and_grads(shape, p, x, t, w, scale=0.3, exact=True)

    def L(pp, xx):
        return 0.3 * M.loss_and_grads(shape, pp, xx, t, w, scale=0.3, exact=True)[0].sum()

    h = 1e-6
    for k in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[k] = h
        fd = (L(p + e, x) - L(p - e, x)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), k
    for b in range(5):
        for k in range(3):
            e = np.zeros_like(x)
            e[b, k] = h
            fd = (L(p, x + e) - L(p, x - e)) / (2 * h)
            assert abs(fd - dx[b, k]) <= 1e-6 * max(1.0, abs(fd))


def test_rounded_gradients_close_to_exact():
    shape = M.MLPShape(n_in=6, width=64, depth=3, n_out=16)
    rng = np.random.default_rng(2)
    p = shape.init(5)
    x = rng.uniform(-1, 1, (64, 6)).astype(np.float32)
    t = rng.normal(0, 1, (64, 16)).astype(np.float32)
    _, g64, _ = M.loss_and_grads(shape, p, x, t, exact=True)
    _, g16, _ = M.loss_and_grads(shape, p, x, t, exact=False)
    assert np.linalg.norm(g16 - g64) / np.linalg.norm(g64) < 2e-2


def test_adamw_step_by_hand():
    shape = M.MLPShape(n_in=2, width=16, depth=1, n_out=8)
    n = shape.num_params()
    rng = np.random.default_rng(4)
    p = rng.normal(0, 1, n).astype(np.float32)
    g = rng.normal(0, 1, n).astype(np.float32)
    m0 = np.zeros(n, np.float32)
    v0 = np.zeros(n, np.float32)
    p1, m1, v1 = M.adamw(p, g, m0, v0, 1, lr=1e-2, b1=0.9, b2=0.99, eps=1e-8, wd=0.1, shape=shape)
    # first step: m/c1 = g, v/c2 = g^2, so the move is lr * g/(|g| + eps) plus decay on weights
    nW = 16 * 2
    np.testing.assert_allclose(p1[:nW], p[:nW] * (1 - 1e-3) - 1e-2 * g[:nW] / (np.abs(g[:nW]) + 1e-8), rtol=1e-5)
    np.testing.assert_allclose(p1[nW:nW + 16], p[nW:nW + 16] - 1e-2 * g[nW:nW + 16] / (np.abs(g[nW:nW + 16]) + 1e-8),
                               rtol=1e-5)
    np.testing.assert_allclose(m1, 0.1 * g, rtol=1e-6)
    np.testing.assert_allclose(v1, 0.01 * g * g, rtol=1e-5)


def test_exact_gradients_with_output_gain():
    shape = M.MLPShape(n_in=3, width=16, depth=2, n_out=8)
    rng = np.random.default_rng(7)
    p = shape.init(2).astype(np.float64)
    x = rng.uniform(-1, 1, (4, 3))
    t = rng.normal(0, 1, (4, 8))
    gain = (0, 1.7)
    _, g, dx = M.loss_and_grads(shape, p, x, t, exact=True, gain=gain)

    def L(pp, xx):
        return M.loss_and_grads(shape, pp, xx, t, exact=True, gain=gain)[0].sum()

    h = 1e-6
    for k in rng.choice(p.size, 20, replace=False):
        e = np.zeros_like(p)
        e[k] = h
        fd = (L(p + e, x) - L(p - e, x)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd))
    for b in range(4):
        for k in range(3):
            e = np.zeros_like(x)
            e[b, k] = h
            fd = (L(p, x + e) - L(p, x - e)) / (2 * h)
            assert abs(fd - dx[b, k]) <= 1e-6 * max(1.0, abs(fd))
