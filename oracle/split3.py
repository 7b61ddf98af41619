"""Test-infrastructure model: the three-piece BF16 split of the tensor-core
operand packing (csrc/gemm_tc.cu ``split3``), in plain Python integers.

x = (-1)^s M 2^e0 with the 53-bit integer M.  hi is M rounded to 8
significant bits (nearest, ties to even), mid the same of the exact remainder,
lo of the next remainder, so |x - hi - mid - lo| <= 2^-24 |x|; each piece
becomes a bf16 bit pattern (zero below 2^-126, infinity above the bf16 range).
FP64 zeros and subnormals give three zero pieces.  Only the tests use this
module.
"""
from __future__ import annotations

import struct

import numpy as np


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _round8(a: int):
    n = a.bit_length()
    if n <= 8:
        return a, 0
    sh = n - 8
    q, rem, half = a >> sh, a & ((1 << sh) - 1), 1 << (sh - 1)
    if rem > half or (rem == half and (q & 1)):
        q += 1
    return q, sh


def _bf16(sgn: int, m: int, e: int) -> int:
    if m == 0:
        return 0
    while m < 128:
        m <<= 1
        e -= 1
    if m == 256:
        m >>= 1
        e += 1
    b = e + 7 + 127
    if b <= 0:
        return 0
    if b >= 255:
        return (sgn << 15) | 0x7F80
    return (sgn << 15) | (b << 7) | (m & 0x7F)


def split3_bits(x: float) -> tuple:
    u = _bits(x)
    ex = (u >> 52) & 0x7FF
    if ex == 0:
        return 0, 0, 0
    if ex == 0x7FF:
        raise ValueError("non-finite input")
    M = (u & ((1 << 52) - 1)) | (1 << 52)
    e0 = ex - 1075
    sg = u >> 63
    out = []
    r = M
    for _ in range(3):
        if r == 0:
            out.append(0)
            continue
        if r < 0:
            sg ^= 1
            r = -r
        q, sh = _round8(r)
        out.append(_bf16(sg, q, e0 + sh))
        r -= q << sh
    return tuple(out)


def bf16_value(bits) -> np.ndarray:
    """float64 values of bf16 bit patterns."""
    b = np.asarray(bits, dtype=np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def split3_array(x: np.ndarray) -> np.ndarray:
    """[..., 3] uint16 pieces of every element."""
    flat = np.asarray(x, dtype=np.float64).ravel()
    out = np.array([split3_bits(float(v)) for v in flat], dtype=np.uint16)
    return out.reshape(np.shape(x) + (3,))
