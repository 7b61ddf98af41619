"""The operand packing's BF16 three-piece split on the device, bit for bit
against the integer model (oracle/split3.py), through both pack kernels."""
import ctypes

import numpy as np
import pytest

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
def test_device_split_is_the_integer_model(row_fastest, scale):
    rng = np.random.default_rng(7 + row_fastest)
    R, K = 70, 45                                                   # ragged against the 32 x 32 tiles
    x = rng.standard_normal((R, K)) * 10.0 ** rng.uniform(-40, 40, (R, K))
    x[0, :5] = [0.0, -0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 257.0]
    x[1, :3] = [5e-324, 2.0 ** -130, -(2.0 ** 100)]
    got = _device_split(x, row_fastest, scale)
    want = sp.split3_array(x * scale)
    assert np.array_equal(got, want)
