"""Python handle of the surrogate MLP kernels (nfx_mlp_* in include/nfx.h).

Layers n_in -> width (x depth hidden layers, SiLU) -> n_out; BF16 weights and activations,
FP32 accumulation on the tensor cores, FP32 master weights and AdamW, all on the GPU. Arrays
cross the boundary as host float32, row-major. There is no CPU fallback: without the native
library or a GPU every call raises NfxError.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class MLP:
    def __init__(self, n_in: int, width: int, depth: int, n_out: int, max_batch: int, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.nfx_mlp_create(int(device), int(n_in), int(width), int(depth), int(n_out), int(max_batch),
                                     C.byref(h)))
        self._h = h
        self.n_in, self.width, self.depth, self.n_out, self.max_batch = n_in, width, depth, n_out, max_batch

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.nfx_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_output_gain(self, input_index: int, alpha: float) -> None:
        """y = exp(alpha * x[input_index]) * network output; input_index -1 removes the gain."""
        check(self._L.nfx_mlp_set_output_gain(self._h, int(input_index), C.c_float(alpha)))
        self.gain = (int(input_index), float(alpha))

    @property
    def num_params(self) -> int:
        n = C.c_int64()
        check(self._L.nfx_mlp_num_params(self._h, C.byref(n)))
        return n.value

    def set_params(self, p) -> None:
        p = _f32(p)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        check(self._L.nfx_mlp_set_params(self._h, _ptr(p)))

    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        check(self._L.nfx_mlp_get_params(self._h, _ptr(out)))
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        check(self._L.nfx_mlp_get_grads(self._h, _ptr(out)))
        return out

    def forward(self, x) -> np.ndarray:
        """f(x) for any number of rows (in chunks of max_batch)."""
        x = _f32(x).reshape(-1, self.n_in)
        y = np.empty((x.shape[0], self.n_out), np.float32)
        for a in range(0, x.shape[0], self.max_batch):
            xa = np.ascontiguousarray(x[a:a + self.max_batch])
            ya = np.empty((xa.shape[0], self.n_out), np.float32)
            check(self._L.nfx_mlp_forward(self._h, _ptr(xa), xa.shape[0], _ptr(ya)))
            y[a:a + xa.shape[0]] = ya
        return y

    def backward(self, x, target, weight=None, scale: float = 1.0, want_dx: bool = False):
        """Per-row losses (and dL/dx when want_dx); parameter gradients stay on the device."""
        x = _f32(x).reshape(-1, self.n_in)
        t = _f32(target).reshape(x.shape[0], self.n_out)
        w = None if weight is None else _f32(weight).reshape(x.shape[0])
        loss = np.empty(x.shape[0], np.float32)
        dx = np.empty_like(x) if want_dx else None
        check(self._L.nfx_mlp_backward(self._h, _ptr(x), _ptr(t), None if w is None else _ptr(w), x.shape[0],
                                       C.c_float(scale), _ptr(loss), None if dx is None else _ptr(dx)))
        return (loss, dx) if want_dx else loss

    def adamw(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
              weight_decay: float = 0.0) -> None:
        check(self._L.nfx_mlp_adamw(self._h, C.c_float(lr), C.c_float(beta1), C.c_float(beta2), C.c_float(eps),
                                    C.c_float(weight_decay)))

    def train(self, x, target, steps: int, batch: int, lr: float = 1e-3, lr_min: float = 1e-5, beta1: float = 0.9,
              beta2: float = 0.999, eps: float = 1e-8, weight_decay: float = 0.0, weight=None,
              seed: int = 0) -> np.ndarray:
        """Minibatch AdamW training on the GPU; returns the mean loss of every step."""
        x = _f32(x).reshape(-1, self.n_in)
        t = _f32(target).reshape(x.shape[0], self.n_out)
        w = None if weight is None else _f32(weight).reshape(x.shape[0])
        hp = _f32([lr, beta1, beta2, eps, weight_decay, lr_min])
        losses = np.empty(max(int(steps), 1), np.float32)
        check(self._L.nfx_mlp_train(self._h, _ptr(x), _ptr(t), None if w is None else _ptr(w), x.shape[0],
                                    int(batch), int(steps), _ptr(hp), C.c_uint64(seed), _ptr(losses)))
        return losses[:steps]

    def fit_inputs(self, x0, target, free_mask, lo, hi, steps: int, lr: float = 1e-2, beta1: float = 0.9,
                   beta2: float = 0.999, eps: float = 1e-8, weight=None):
        """Adam on the inputs (free entries only, clamped to [lo, hi]) towards the targets.
        Returns (x, per-row loss)."""
        x = _f32(x0).reshape(-1, self.n_in).copy()
        t = _f32(target).reshape(x.shape[0], self.n_out)
        w = None if weight is None else _f32(weight).reshape(x.shape[0])
        mask = np.ascontiguousarray(np.asarray(free_mask, bool).astype(np.uint8).reshape(self.n_in))
        lo_, hi_ = _f32(lo).reshape(self.n_in), _f32(hi).reshape(self.n_in)
        hp = _f32([lr, beta1, beta2, eps])
        loss = np.empty(x.shape[0], np.float32)
        check(self._L.nfx_mlp_fit_inputs(self._h, _ptr(x), _ptr(t), None if w is None else _ptr(w), x.shape[0],
                                         _ptr(mask), _ptr(lo_), _ptr(hi_), int(steps), _ptr(hp), _ptr(loss)))
        return x, loss


def main(argv=None) -> int:
    """Training throughput of the surrogate's network (6 -> 256 x 3 -> 64, batch 512) on a synthetic
    smooth map: wall time per nfx_mlp_train step over --steps steps, after a warm-up call."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(description="time nfx_mlp_train on the surrogate's network")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--rows", type=int, default=6144)
    ap.add_argument("--width", type=int, default=256)
    ap.add_argument("--depth", type=int, default=3)
    a = ap.parse_args(argv)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.0, 1.0, (a.rows, 6)).astype(np.float32)
    d = np.linspace(0.0, 1.0, 64, dtype=np.float32)
    t = (np.exp(0.3 * x[:, :1]) * d ** (1.5 + 0.3 * x[:, 1:2]) * (1.0 + 0.2 * np.sin(3.0 * x[:, 2:3] * d))).astype(np.float32)
    m = MLP(6, a.width, a.depth, 64, a.batch)
    fan = [6] + [a.width] * a.depth
    outs = [a.width] * a.depth + [64]
    p = np.concatenate([np.concatenate([rng.standard_normal(o * i) * np.sqrt(2.0 / i), np.zeros(o)])
                        for i, o in zip(fan, outs)]).astype(np.float32)
    m.set_params(p)
    m.train(x, t, steps=32, batch=a.batch)  # warm-up
    t0 = time.perf_counter()
    losses = m.train(x, t, steps=a.steps, batch=a.batch)
    dt = time.perf_counter() - t0
    m.close()
    print(json.dumps({"steps": a.steps, "batch": a.batch, "ms_per_step": 1e3 * dt / a.steps,
                      "first_loss": float(losses[0]), "last_loss": float(losses[-1])}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
