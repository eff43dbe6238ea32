"""The element laws' device divide (an approximate reciprocal refined by Markstein's method)
agrees with correctly rounded float32 division to within one unit in the last place."""

import ctypes as C

import numpy as np
import pytest

from nofluidx3d_gb300 import _lib

pytestmark = pytest.mark.gpu


def ulp_distance(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between float32 arrays of equal signs."""
    xi = x.view(np.int32).astype(np.int64)
    yi = y.view(np.int32).astype(np.int64)
    return np.abs(xi - yi)


def test_device_divide_within_one_ulp():
    rng = np.random.default_rng(3)
    n = 1 << 20
    # magnitudes over the range the element laws see (determinants, stresses, rates) and beyond
    a = (rng.uniform(0.5, 1.0, n) * 10.0 ** rng.uniform(-15, 15, n)).astype(np.float32)
    b = (rng.uniform(0.5, 1.0, n) * 10.0 ** rng.uniform(-15, 15, n)).astype(np.float32)
    a *= np.where(rng.random(n) < 0.5, -1, 1).astype(np.float32)
    b *= np.where(rng.random(n) < 0.5, -1, 1).astype(np.float32)
    # near-1 denominators, as in 1 / det(I + P) and 1 / det F
    b[: n // 4] = (1.0 + rng.uniform(-0.3, 0.3, n // 4)).astype(np.float32)
    a[: n // 8] = 1.0
    q = np.empty(n, np.float32)
    L = _lib.load()
    ptr = lambda x: x.ctypes.data_as(C.c_void_p)
    _lib.check(L.nfx_divide_check(0, n, ptr(a), ptr(b), ptr(q)))
    ref = (a / b).astype(np.float32)
    assert np.all(np.isfinite(q))
    assert np.all(np.sign(q) == np.sign(ref))
    d = ulp_distance(q, ref)
    assert d.max() <= 1, (d.max(), a[d.argmax()], b[d.argmax()])
    # almost every quotient is the correctly rounded one
    assert (d == 0).mean() > 0.99
