"""The tcgen05 BF16 -> FP32 tile product (puck_tc_selftest) against a host
product of the same BF16 values.

BF16 x BF16 products are exact in FP32, so the only difference is the FP32
accumulation order over k; the tolerance is 1e-5 relative to the sum of
absolute terms.
"""
import ctypes

import numpy as np
import pytest

from puck_gb300 import _lib

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """Round-to-nearest-even FP32 -> BF16 bit patterns."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("k,n", [(16, 16), (64, 32), (112, 16), (240, 48), (256, 256)])
def test_tc_tile_product_matches_host(k, n):
    L = _lib.load()
    rng = np.random.default_rng(k * 1000 + n)
    a = to_bf16_bits(rng.standard_normal((128, k)).astype(np.float32))
    b = to_bf16_bits((rng.random((n, k)) * np.exp(-3 * rng.random((n, k)))).astype(np.float32))
    d = np.zeros((128, n), np.float32)
    st = L.puck_tc_selftest(0, k, n, a.ctypes.data, b.ctypes.data, d.ctypes.data)
    assert st == 0, _lib.last_error()
    A, B = from_bf16_bits(a).astype(np.float64), from_bf16_bits(b).astype(np.float64)
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    err = np.abs(d - ref) / np.maximum(scale, 1e-30)
    assert err.max() < 1e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))


def test_tc_selftest_rejects_bad_shapes():
    L = _lib.load()
    z = np.zeros(128 * 32, np.uint16)
    d = np.zeros(128 * 32, np.float32)
    assert L.puck_tc_selftest(0, 24, 16, z.ctypes.data, z.ctypes.data, d.ctypes.data) == 6
    assert L.puck_tc_selftest(0, 16, 8, z.ctypes.data, z.ctypes.data, d.ctypes.data) == 6
