"""Test-infrastructure model of the exact-slice (Ozaki-scheme) product.

A numpy restatement of the scheme the exact-slice tensor-core kernel
implements (Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59, 95 (2012);
on tensor cores: Mukunoki et al., ISC 2020), used by the tests to check the
digit decomposition and the error bound on the CPU:

* each row r of an operand gets the exponent e_r with max_k |x_rk| < 2^e_r;
* y = x 2^-e_r is rounded to Z = round(|y| 64^S) and cut into S balanced
  base-64 digits d_1..d_S (d_1 in [0, 64], d_s in [-32, 32) for s >= 2,
  carrying into the next digit), all signed like x;
* A.B^T = 2^(e_r + e_c) sum over slice pairs (s, t) with s + t <= G of
  64^-(s+t) D^A_s (D^B_t)^T, the digit products summed exactly.
Only the tests use this module.
"""
import struct

import numpy as np

BITS = 6


def row_exponent(x: np.ndarray) -> int:
    m = float(np.max(np.abs(x))) if x.size else 0.0
    return int(np.frexp(m)[1]) if m > 0 else 0


def digits(x: float, e: int, S: int) -> list:
    """The S digits of one element, by the same integer arithmetic on the FP64
    bits as the device kernel."""
    bits = struct.unpack("<Q", struct.pack("<d", x))[0]
    be = (bits >> 52) & 0x7FF
    Z = 0
    if be:
        m = (bits & ((1 << 52) - 1)) | (1 << 52)        # |x| = m 2^(be - 1075)
        sh = 1075 + e - BITS * S - be                    # Z = m 2^-sh
        if sh <= 0:
            Z = m << (-sh)
        elif sh < 64:
            Z = (m >> sh) + ((m >> (sh - 1)) & 1)
    neg = bits >> 63
    d = [0] * S
    for s in range(S - 1, 0, -1):
        r = Z & 63
        Z >>= 6
        if r >= 32:
            r -= 64
            Z += 1
        d[s] = -r if neg else r
    d[0] = -Z if neg else Z
    return d


def slice_matrix(X: np.ndarray, S: int):
    """Digit slices D[s] (rows x K, integers) and row exponents of X."""
    R, K = X.shape
    e = np.array([row_exponent(X[r]) for r in range(R)])
    D = np.zeros((S, R, K), dtype=np.int64)
    for r in range(R):
        for k in range(K):
            D[:, r, k] = digits(float(X[r, k]), int(e[r]), S)
    return D, e


def product(A: np.ndarray, B: np.ndarray, G: int) -> np.ndarray:
    """A @ B.T by the exact-slice scheme with G weight groups (exact integer
    sums, then one rounding to FP64 per element)."""
    S = G - 1
    DA, eA = slice_matrix(A, S)
    DB, eB = slice_matrix(B, S)
    acc = np.zeros((A.shape[0], B.shape[0]), dtype=object)
    for g in range(2, G + 1):
        part = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
        for s in range(1, g):
            t = g - s
            if s > S or t > S:
                continue
            part += DA[s - 1] @ DB[t - 1].T
        acc = acc + part.astype(object) * (1 << (BITS * (G - g)))
    out = np.array([[float(v) for v in row] for row in acc])
    return out * np.ldexp(1.0, (eA[:, None] + eB[None, :] - BITS * G).astype(np.int64))
