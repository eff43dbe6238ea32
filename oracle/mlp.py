"""CPU oracle of the surrogate MLP (test infrastructure only; nothing in the product imports it).

Restates, in numpy, what the nfx_mlp_* kernels compute (nofluidx3d_gb300/csrc/nfx_mlp.cu):
layers n_in -> width (x depth, SiLU) -> n_out, weights and activations rounded to bfloat16 at
the same points as the kernels, products accumulated in float32, FP32 master weights, AdamW.
The reference (noFluidX3D) has no learned part, so there is nothing of it to pin here; this
oracle is pinned instead by its float64 mode, whose gradients are checked against central finite
differences in tests/test_mlp_oracle.py.

Parameter layout (shared with the C ABI): for each layer l in order, W_l [out_l, in_l]
row-major, then b_l [out_l].
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest, ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


@dataclass
class MLPShape:
    n_in: int
    width: int
    depth: int
    n_out: int

    def layers(self) -> list[tuple[int, int]]:
        """(out, in) of every layer."""
        dims = [self.n_in] + [self.width] * self.depth + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def num_params(self) -> int:
        return sum(o * i + o for o, i in self.layers())

    def split(self, p: np.ndarray) -> list[tuple[np.ndarray, np.ndarray]]:
        out, off = [], 0
        for o, i in self.layers():
            W = p[off:off + o * i].reshape(o, i)
            off += o * i
            b = p[off:off + o]
            off += o
            out.append((W, b))
        return out

    def init(self, seed: int = 0) -> np.ndarray:
        """He-uniform weights, zero biases (float32)."""
        rng = np.random.default_rng(seed)
        parts = []
        for o, i in self.layers():
            lim = np.sqrt(6.0 / i)
            parts.append(rng.uniform(-lim, lim, o * i))
            parts.append(np.zeros(o))
        return np.concatenate(parts).astype(np.float32)


def forward(shape: MLPShape, p: np.ndarray, x: np.ndarray, exact: bool = False, gain=None):
    """Returns (y, cache). exact=True: float64 without bf16 rounding (the finite-difference
    reference); exact=False: the kernels' rounding points, float32 accumulation. gain = (k, alpha):
    y = exp(alpha * x[:, k]) * last layer output, x in full precision (nfx_mlp_set_output_gain)."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    layers = shape.split(p.astype(dt))
    xf = np.asarray(x, dt)
    X = rnd(xf)
    cache = {"X": [X], "Z": [], "W": [], "g": None}
    for li, (W, b) in enumerate(layers):
        Wr = rnd(W)
        cache["W"].append(Wr)
        Z = (X.astype(dt) @ Wr.T.astype(dt)).astype(dt) + b.astype(dt)
        if li == len(layers) - 1:
            if gain is not None:
                g = np.exp(dt(gain[1]) * xf[:, gain[0]]).astype(dt)
                cache["g"] = g
                Z = (Z * g[:, None]).astype(dt)
            return Z, cache
        cache["Z"].append(Z)
        X = rnd(silu(Z).astype(dt))
        cache["X"].append(X)
    raise AssertionError("unreachable")


def loss_and_grads(shape: MLPShape, p: np.ndarray, x: np.ndarray, t: np.ndarray, w: np.ndarray | None = None,
                   scale: float = 1.0, exact: bool = False, gain=None):
    """L = scale * sum_b w_b ||y_b - t_b||^2; returns (per-row losses w_b ||.||^2, dL/dp flat,
    dL/dx)."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    y, c = forward(shape, p, x, exact, gain)
    B = y.shape[0]
    wv = np.ones(B, dt) if w is None else np.asarray(w, dt)
    d = y - np.asarray(t, dt)
    rows = wv * (d * d).sum(1)
    dl = (scale * 2.0 * wv[:, None] * d).astype(dt)
    g = c["g"] if c["g"] is not None else np.ones(B, dt)
    G = rnd((dl * g[:, None]).astype(dt))
    grads = []
    nl = len(c["W"])
    dx = None
    for li in range(nl - 1, -1, -1):
        X = c["X"][li]
        gW = (G.T.astype(dt) @ X.astype(dt)).astype(dt)
        gb = G.astype(dt).sum(0)
        grads.append((gW, gb))
        dX = (G.astype(dt) @ c["W"][li].astype(dt)).astype(dt)
        if li > 0:
            G = rnd((dX * silu_grad(c["Z"][li - 1])).astype(dt))
        else:
            dx = dX.copy()
            if gain is not None:
                dx[:, gain[0]] += dt(gain[1]) * (y * dl).sum(1)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return rows, flat, dx


def adamw(p, g, m, v, step, lr, b1, b2, eps, wd, shape: MLPShape):
    """One AdamW step in float32 (decoupled weight decay on weights only, bias-corrected)."""
    p = p.astype(np.float32).copy()
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    decay = np.zeros_like(p)
    off = 0
    for o, i in shape.layers():
        decay[off:off + o * i] = wd
        off += o * i + o
    p = p * (1 - lr * decay)
    p = p - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p.astype(np.float32), m.astype(np.float32), v.astype(np.float32)
