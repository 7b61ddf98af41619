"""The BF16 three-piece split model (oracle/split3.py) on the CPU: exact
remainders, the 2^-24 bound, ties to even, signs and zeros."""
import numpy as np

from oracle import split3 as sp


def _sum(pieces):
    v = sp.bf16_value(np.asarray(pieces))
    return v[..., 0] + v[..., 1] + v[..., 2]


def test_three_pieces_reproduce_x_to_2_pow_minus_24():
    # each remainder is at most 2^-8 of the previous one: |x - hi - mid - lo|
    # <= 2^-24 |x| (while lo stays in the bf16 range), typically ~2^-27
    rng = np.random.default_rng(0)
    x = rng.standard_normal(4000) * 10.0 ** rng.uniform(-30, 30, 4000)
    p = sp.split3_array(x)
    err = np.abs(_sum(p) - x)
    big = np.abs(x) > 1e-30
    assert np.all(err[big] <= 2.0 ** -24 * np.abs(x[big]))
    assert np.median(err[big] / np.abs(x[big])) < 2.0 ** -26
    # hi is within half a bf16 ulp of x
    hi = sp.bf16_value(p[:, 0])
    ulp = 2.0 ** (np.floor(np.log2(np.abs(hi))) - 7)
    assert np.all(np.abs(x - hi) <= 0.5 * ulp * (1 + 1e-15))


def test_ties_round_to_even_and_signs():
    one = 0x3F80
    assert sp.split3_bits(1.0 + 2.0 ** -8) == (one, 0x3B80, 0)         # tie -> even 1.0, mid 2^-8
    h, m, l = sp.split3_bits(1.0 + 3 * 2.0 ** -8)                       # tie -> even 1 + 2^-6
    assert sp.bf16_value(h) == 1.0 + 2.0 ** -6 and sp.bf16_value(m) == -(2.0 ** -8) and l == 0
    assert sp.split3_bits(0.0) == (0, 0, 0) and sp.split3_bits(-0.0) == (0, 0, 0)
    assert sp.split3_bits(5e-324) == (0, 0, 0)                          # FP64 subnormal
    rng = np.random.default_rng(1)
    for v in rng.standard_normal(200):
        a, b = sp.split3_bits(float(v)), sp.split3_bits(float(-v))
        assert all((x ^ y) in (0, 0x8000) for x, y in zip(a, b)) and a[0] ^ b[0] == 0x8000


def test_exact_small_values_need_one_piece():
    for v in (1.0, -3.0, 0.5, 255.0, 2.0 ** 100, -(2.0 ** -100)):
        h, m, l = sp.split3_bits(v)
        assert sp.bf16_value(h) == v and m == 0 and l == 0
    h, m, l = sp.split3_bits(257.0)          # 9 significant bits: two pieces
    assert sp.bf16_value(h) + sp.bf16_value(m) == 257.0 and l == 0
