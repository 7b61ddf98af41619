"""Single-contraction checks of the device kernels against numpy.

FP64 (DMMA) must agree to round-off; the split-BF16 tensor-core kernel
(three products, FP32 accumulation) to about 1e-5 of the largest |C|; the
exact-slice kernel (Ozaki scheme) to its slice truncation (with 8
weight groups: ~1e-12 of max|C|) and bit-exactly on operands its slices
represent exactly.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("mk,nk->mn", (128, 64), (128, 64), (128, 128)),
    ("mk,nk->mn", (200, 70), (130, 70), (200, 130)),
    ("ik,kj->ij", (333, 250), (250, 97), (333, 97)),
    ("ijcd,acbd->ijab", (6, 5, 9, 11), (7, 9, 8, 11), (6, 5, 7, 8)),
    ("kjbc,kiac->ijab", (5, 6, 7, 8), (5, 4, 9, 8), (4, 6, 9, 7)),
    ("lb,lca->abc", (9, 40), (9, 33, 37), (37, 40, 33)),
    ("Qai,Qbj->ijab", (50, 20, 6), (50, 21, 7), (6, 7, 20, 21)),
    ("abd,cd->abc", (17, 19, 150), (300, 150), (17, 19, 300)),
    ("ikac,kc->ia", (40, 5, 36, 7), (5, 7), (40, 36)),              # N = 1 (matrix-vector)
    ("jlcd,klcd->kj", (20, 9, 30, 11), (24, 9, 30, 11), (24, 20)),  # few tiles, long K (split-K)
]


def _run(prec, spec, A, B, C, alpha=1.0, beta=0.0):
    from fermicc import _lib
    lib = _lib.load()
    i64 = lambda shape: (ctypes.c_int64 * len(shape))(*shape)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    A = np.ascontiguousarray(A); B = np.ascontiguousarray(B)
    out = np.ascontiguousarray(C.copy())
    rc = lib.fcc_test_contract(prec, spec.encode(), dp(A), i64(A.shape), A.ndim, dp(B), i64(B.shape), B.ndim,
                               dp(out), i64(out.shape), out.ndim, alpha, beta)
    return rc, out


@pytest.mark.parametrize("spec,sa,sb,sc", CASES)
def test_fp64_contraction(spec, sa, sb, sc):
    rng = np.random.default_rng(0)
    A, B, C = rng.standard_normal(sa), rng.standard_normal(sb), rng.standard_normal(sc)
    rc, out = _run(0, spec, A, B, C, 0.7, -1.3)
    assert rc == 0
    ref = 0.7 * np.einsum(spec, A, B) - 1.3 * C
    assert np.abs(out - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("spec,sa,sb,sc", CASES)
def test_split_bf16_tensor_core_contraction(spec, sa, sb, sc):
    rng = np.random.default_rng(1)
    A, B, C = rng.standard_normal(sa), rng.standard_normal(sb), rng.standard_normal(sc)
    rc, out = _run(1, spec, A, B, C, 1.0, 0.0)
    assert rc == 0
    ref = np.einsum(spec, A, B)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 3e-5, err
    rc, out2 = _run(1, spec, A, B, C, -0.5, 2.0)
    assert rc == 0
    ref2 = -0.5 * ref + 2.0 * C
    assert np.abs(out2 - ref2).max() / np.abs(ref2).max() < 3e-5


@pytest.mark.parametrize("spec,sa,sb,sc", CASES)
def test_six_product_split_contraction(spec, sa, sb, sc):
    # hi/mid/lo pieces, six products: error ~2^-24 (FP32 accumulation)
    rng = np.random.default_rng(2)
    A, B, C = rng.standard_normal(sa), rng.standard_normal(sb), rng.standard_normal(sc)
    rc, out = _run(2, spec, A, B, C, 1.0, 0.0)
    assert rc == 0
    ref = np.einsum(spec, A, B)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 6e-6, err


@pytest.mark.parametrize("spec,sa,sb,sc", CASES)
def test_exact_slice_contraction(spec, sa, sb, sc):
    # 8 weight groups (28 slice-pair products): truncation ~2^-42 of
    # max|A_r| max|B_c| per term, ~1e-12 of max|C| for Gaussian operands
    rng = np.random.default_rng(3)
    A, B, C = rng.standard_normal(sa), rng.standard_normal(sb), rng.standard_normal(sc)
    rc, out = _run(3, spec, A, B, C, 0.7, -1.3)
    assert rc == 0
    ref = 0.7 * np.einsum(spec, A, B) - 1.3 * C
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 1e-11, err


@pytest.mark.parametrize("G,tol", [(5, 2e-6), (7, 5e-10)])
def test_exact_slice_groups_set_the_accuracy(G, tol):
    spec, sa, sb, sc = "mk,nk->mn", (200, 700), (130, 700), (200, 130)
    rng = np.random.default_rng(4)
    A, B = rng.standard_normal(sa), rng.standard_normal(sb)
    rc, out = _run(10 + G, spec, A, B, np.zeros(sc))
    assert rc == 0
    ref = A @ B.T
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < tol, (G, err)


def test_exact_slice_accumulation_is_exact():
    # entries k/64 (|k| <= 64): one or two 6-bit slices hold them exactly, so
    # the product must equal the exact integer result bit for bit, over a K
    # long enough for several exact FP32 chunks (2048 products each) and a
    # split of the k loop over CTAs
    rng = np.random.default_rng(5)
    M, N, K = 150, 140, 5000
    Ai = rng.integers(-64, 65, size=(M, K))
    Bi = rng.integers(-64, 65, size=(N, K))
    Ai[3, :] = 64                      # a row at exactly 1.0: its scale is 2, two slices
    Bi[7, :] = -64
    A, B = Ai / 64.0, Bi / 64.0
    rc, out = _run(3, "mk,nk->mn", A, B, np.zeros((M, N)))
    assert rc == 0
    ref = (Ai @ Bi.T).astype(np.float64) / 4096.0      # exact: |sum| < 2^53
    assert np.array_equal(out, ref), np.abs(out - ref).max()


def test_exact_slice_largest_chunk_sums_stay_exact():
    # rows of 63/64 (one digit 63 each): every digit product is 3969, the
    # largest a chunk of 2048 products can hold is ~2^23 -- still exact in FP32
    M, N, K = 128, 128, 4100
    A = np.full((M, K), 63.0 / 64.0)
    B = np.full((N, K), -63.0 / 64.0)
    rc, out = _run(3, "mk,nk->mn", A, B, np.zeros((M, N)))
    assert rc == 0
    assert np.array_equal(out, np.full((M, N), -K * 3969.0 / 4096.0))
