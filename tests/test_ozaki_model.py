"""CPU checks of the exact-slice (Ozaki-scheme) numerics the tensor-core
kernel implements: digit bounds, reconstruction, exactness and the error
decrease with the number of weight groups."""
import numpy as np
import pytest

from oracle import ozaki


def test_digits_bounds_and_reconstruction():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(2000) * np.logspace(0, -6, 2000)
    e = ozaki.row_exponent(x)
    for S in (3, 5, 7):
        err = 0.0
        for v in x:
            d = ozaki.digits(float(v), e, S)
            assert abs(d[0]) <= 64 and all(-32 <= t <= 32 for t in d[1:])
            rec = sum(di * 64.0 ** -(i + 1) for i, di in enumerate(d)) * 2.0 ** e
            err = max(err, abs(rec - v))
        assert err <= 0.5 * 64.0 ** -S * 2.0 ** e * (1 + 1e-12)


def test_digits_are_exact_for_short_mantissas():
    # k/64 with |k| <= 64 needs at most two digits: the slices hold it exactly
    for k in range(-64, 65):
        x = k / 64.0
        d = ozaki.digits(x, 1, 7)
        assert sum(di * 64.0 ** -(i + 1) for i, di in enumerate(d)) * 2.0 == x


@pytest.mark.parametrize("G,tol", [(5, 5e-7), (6, 2e-8), (7, 3e-10), (8, 5e-12)])
def test_product_error_falls_by_64_per_group(G, tol):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((12, 150))
    B = rng.standard_normal((9, 150))
    ref = A @ B.T
    err = np.abs(ozaki.product(A, B, G) - ref).max() / np.abs(ref).max()
    assert err < tol, (G, err)


def test_product_is_exact_on_representable_inputs():
    rng = np.random.default_rng(2)
    Ai = rng.integers(-64, 65, size=(5, 300))
    Bi = rng.integers(-64, 65, size=(4, 300))
    out = ozaki.product(Ai / 64.0, Bi / 64.0, 8)
    assert np.array_equal(out, (Ai @ Bi.T) / 4096.0)


def test_chunk_sums_stay_exact_in_fp32():
    # 2048 digit products of magnitude <= 64 * 64 sum to at most 2^23 in
    # magnitude: every partial sum of such a chunk is exactly representable
    # in FP32 (24-bit significand)
    assert 2048 * 64 * 64 <= 2 ** 23
    rng = np.random.default_rng(3)
    d = rng.integers(-64, 65, size=(2, 2048)).astype(np.float32)
    s = np.float32(0.0)
    for p in d[0] * d[1]:
        s = np.float32(s + p)
    assert int(s) == int(np.sum(d[0].astype(np.int64) * d[1].astype(np.int64)))


def test_biased_plain_digits_are_the_sequential_cut():
    # the device cuts Z into balanced digits as the plain base-64 digits of
    # Z + 32 (64^(S-2) + ... + 1), less 32 (top digit: the rest), with every
    # shift a constant; the same digits as the sequential cut with carries
    rng = np.random.default_rng(3)
    for S in range(1, 9):
        C = 32 * ((64 ** (S - 1) - 1) // 63)
        for Z in list(rng.integers(0, 64 ** S + 1, 3000, dtype=np.int64)) + [0, 31, 32, 63, 64, 64 ** S]:
            Z = int(Z)
            seq, t = [0] * S, Z
            for s in range(S - 1, 0, -1):
                r = t & 63
                t >>= 6
                if r >= 32:
                    r -= 64
                    t += 1
                seq[s] = r
            seq[0] = t
            Zc = Z + C
            plain = [Zc >> (6 * (S - 1))] + [((Zc >> (6 * (S - 1 - s))) & 63) - 32 for s in range(1, S)]
            assert plain == seq, (S, Z)
