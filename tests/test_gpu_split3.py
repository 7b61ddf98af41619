"""The operand packings on the device, bit for bit against their integer
models: the BF16 three-piece split (oracle/split3.py) and the exact-slice
digit slices with their row exponents (oracle/ozaki.py), each through both
pack kernels (row walk and transposing tiles)."""
import ctypes

import numpy as np
import pytest

from oracle import ozaki as oz
from oracle import split3 as sp

pytestmark = pytest.mark.gpu


def _device_split(x, row_fastest, scale):
    from fermicc import _lib
    lib = _lib.load()
    R, K = x.shape
    src = np.ascontiguousarray(x.T if row_fastest else x)          # row_fastest: column-major R x K
    out = np.empty((R, 3 * K), dtype=np.uint16)
    rc = lib.fcc_test_split3(src.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), R, K, int(row_fastest), scale,
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
    assert rc == 0
    return out.reshape(R, 3, K).transpose(0, 2, 1)                  # [r, k, piece]


@pytest.mark.parametrize("row_fastest", [0, 1])
@pytest.mark.parametrize("scale", [1.0, -1.0, 0.5])
@pytest.mark.parametrize("K", [45, 64])
def test_device_split_is_the_integer_model(row_fastest, scale, K):
    # K = 45: ragged against the 32 x 32 tiles, element-wise stores; K = 64:
    # the 8-byte (row walk) and 4-byte (tiles) stores
    rng = np.random.default_rng(7 + row_fastest + K)
    R = 70
    x = rng.standard_normal((R, K)) * 10.0 ** rng.uniform(-40, 40, (R, K))
    x[0, :5] = [0.0, -0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 257.0]
    x[1, :3] = [5e-324, 2.0 ** -130, -(2.0 ** 100)]
    got = _device_split(x, row_fastest, scale)
    want = sp.split3_array(x * scale)
    assert np.array_equal(got, want)


def _bf16_bits(d):
    """bf16 bit patterns of small integers (exact in bf16)."""
    f = np.asarray(d, dtype=np.float32)
    return (f.view(np.uint32) >> 16).astype(np.uint16)


@pytest.mark.parametrize("row_fastest", [0, 1])
@pytest.mark.parametrize("S", [1, 5, 6, 7, 8])
def test_device_digit_slices_are_the_integer_model(row_fastest, S):
    from fermicc import _lib
    lib = _lib.load()
    rng = np.random.default_rng(11 + S + 10 * row_fastest)
    R, K = 70, 100                                                 # ragged against the tiles and Kpad = 128
    x = rng.standard_normal((R, K)) * 10.0 ** rng.uniform(-3, 3, (R, 1))
    x[2, :] *= 10.0 ** rng.uniform(-12, 0, K)                      # a row of widely spread magnitudes
    x[3, :] = 0.0                                                  # an all-zero row
    x[4, :6] = [1.0, -1.0, 0.5, -0.75, 63.0 / 64.0, 5e-324]
    x[5, :] = 2.0 ** 40 * np.sign(rng.standard_normal(K))
    Kpad = (K + 63) // 64 * 64
    src = np.ascontiguousarray(x.T if row_fastest else x)
    out = np.empty((R, S * Kpad), dtype=np.uint16)
    ex = np.empty(R, dtype=np.int32)
    rc = lib.fcc_test_pack_oz(src.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), R, K, int(row_fastest), S,
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                              ex.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    assert rc == 0
    D, _ = oz.slice_matrix(x, S)                                   # D[s, r, k]
    mx = np.abs(x).max(axis=1)
    want_ex = np.where(mx > 0, np.frexp(mx)[1] + 1022, 0)          # biased exponent of the row maximum
    assert np.array_equal(ex, want_ex)
    got = out.reshape(R, S, Kpad)
    assert not got[:, :, K:].any()                                 # zero padding
    want = _bf16_bits(D.transpose(1, 0, 2))
    assert np.array_equal(got[:, :, :K], want)
