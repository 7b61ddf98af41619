"""The allocation-free FP64 GEMM entry point (fcc_gemm_f64_noalloc).

Callers that cannot allocate device memory -- code recording a CUDA graph, a
host framework that hands out every device buffer from its own pool, a path
that must not absorb cudaMalloc's implicit synchronisation -- pass their own
device arrays; the entry point keeps its split-K partial sums in a fixed
device array instead of allocating.  Its results must match the regular
contraction entry point.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular(A, B, C, alpha, beta):
    """Same product through fcc_test_contract (host arrays, allocates)."""
    from fermicc import _lib
    lib = _lib.load()
    i64 = lambda shape: (ctypes.c_int64 * len(shape))(*shape)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    out = np.ascontiguousarray(C.copy())
    rc = lib.fcc_test_contract(0, b"mk,kn->mn", dp(A), i64(A.shape), 2, dp(B), i64(B.shape), 2, dp(out),
                               i64(out.shape), 2, alpha, beta)
    assert rc == 0
    return out


def test_noalloc_gemm_matches_regular_entry_point_twice():
    import torch
    from fermicc import _lib
    lib = _lib.load()
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream()
    # two calls in a row on different data: the shared scratch keeps nothing
    # that the second call could pick up
    for call, (M, N, K, alpha, beta) in enumerate([(40, 24, 20000, 1.0, 0.0), (96, 70, 9000, -0.7, 0.5)]):
        A = rng.standard_normal((M, K))
        B = rng.standard_normal((K, N))
        C = rng.standard_normal((M, N))
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        dC = torch.from_numpy(C).cuda()
        torch.cuda.synchronize()
        rc = lib.fcc_gemm_f64_noalloc(M, N, K, alpha, ctypes.c_void_p(dA.data_ptr()), K,
                                      ctypes.c_void_p(dB.data_ptr()), N, beta, ctypes.c_void_p(dC.data_ptr()), N,
                                      ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        got = dC.cpu().numpy()
        ref = _regular(A, B, C, alpha, beta)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), call


def test_noalloc_gemm_rejects_sizes_beyond_its_scratch():
    from fermicc import _lib
    lib = _lib.load()
    null = ctypes.c_void_p(0)
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    assert lib.fcc_gemm_f64_noalloc(2048, 1024, 64, 1.0, dummy, 64, dummy, 1024, 0.0, dummy, 1024, null) == \
        _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_gemm_f64_noalloc(0, 4, 4, 1.0, dummy, 4, dummy, 4, 0.0, dummy, 4, null) == _lib.FCC_ERR_BAD_ARG
