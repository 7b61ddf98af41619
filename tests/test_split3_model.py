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


# --- the device's single-precision path (csrc/gemm_tc.cu split3), restated
# with exact integer emulation of each float operation: the 24-bit cut with
# rounding to odd, then the float-to-bf16 rounding (nearest, ties to even)

def _bf16_rne_of_float(b32):
    """bf16 bits of the float with bits b32 (finite), nearest-even."""
    return ((b32 + 0x7FFF + ((b32 >> 16) & 1)) >> 16) & 0xFFFF


def _float_bits(m, e):
    """bits of the normal float m * 2^e with 2^23 <= m < 2^24."""
    return ((e + 23 + 127) << 23) | (m & 0x7FFFFF)


def _rne8_units(a, e0):
    """bf16 bits of round8(a * 2^e0) through the round-to-odd float (a > 0)."""
    n = a.bit_length()
    if n <= 24:
        m, sh = a << (24 - n), -(24 - n)
    else:
        sh = n - 24
        m = a >> sh
        if (m << sh) != a:      # bits lost below the cut: set the last one
            m |= 1
    return _bf16_rne_of_float(_float_bits(m, sh + e0))


def _units(pb, e0):
    m8, sh = 0x80 | (pb & 0x7F), ((pb >> 7) & 0xFF) - 134 - e0
    return m8 << sh if sh >= 0 else m8 >> -sh


def _split3_device_model(x):
    import struct
    u = struct.unpack("<Q", struct.pack("<d", x))[0]
    ex = (u >> 52) & 0x7FF
    if ex < 949 or ex > 1149:                       # the all-integer path
        return sp.split3_bits(x)
    sg, e0 = u >> 63, ex - 1075
    M = (u & ((1 << 52) - 1)) | (1 << 52)
    hb = _rne8_units(M, e0)
    r1 = M - _units(hb, e0)
    m = l = 0
    if r1:
        sg1 = sg ^ (r1 < 0)
        mb = _rne8_units(abs(r1), e0)
        m = (sg1 << 15) | mb
        r2 = abs(r1) - _units(mb, e0)
        if r2:
            l = ((sg1 ^ (r2 < 0)) << 15) | _rne8_units(abs(r2), e0)
    return ((sg << 15) | hb, m, l)


def test_round_to_odd_path_is_the_integer_model():
    # cutting the remainder at 24 bits with the last bit set when bits were
    # lost, then rounding that float to bf16, equals rounding the remainder
    # itself (Boldo & Melquiond): the device's fast path gives the pieces of
    # split3_bits bit for bit, ties included
    rng = np.random.default_rng(11)
    xs = list(rng.standard_normal(4000) * 10.0 ** rng.uniform(-30, 30, 4000))
    xs += [1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 257.0, 1.0 + 2.0 ** -9 + 2.0 ** -17, 1.0 + 2.0 ** -16 + 2.0 ** -25,
           2.0 ** -74, 1.7 * 2.0 ** -73, 1.9 * 2.0 ** 126, -1.5 * 2.0 ** 127, 1.0 / 3.0, -255.0]
    for _ in range(2000):                                               # exact ties below hi and mid
        base = int(rng.integers(128, 256))
        k = int(rng.integers(0, 27))
        M = (base << 45) + (int(rng.integers(128, 256)) << (36 - k)) + (1 << (35 - k))
        xs.append(float(np.ldexp(float(M), int(rng.integers(-100, 60)) - 52)))
    for x in xs:
        assert _split3_device_model(float(x)) == sp.split3_bits(float(x)), x
