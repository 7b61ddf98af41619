"""The allocation-free FP64 GEMM entry point (fcc_gemm_f64_noalloc).

Some callers cannot allocate device memory: a host framework that hands out
every device buffer from its own pool and forbids other allocations, or a
latency-critical path that must not absorb cudaMalloc's implicit device
synchronisation.  They pass their own device arrays; the entry point keeps
its split-K partial sums in a fixed device array instead of allocating.
Its results must equal alpha * A @ B + beta * C computed on the host, on
consecutive calls that share that array.  This file is collected last on
purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# DMMA products against numpy's BLAS: both are FP64 with different summation
# orders, so they agree to a small multiple of K * 2^-53 relative
TOL = 1e-12


def _call(lib, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc, stream):
    return lib.fcc_gemm_f64_noalloc(M, N, K, alpha, ctypes.c_void_p(dA.data_ptr()), lda,
                                    ctypes.c_void_p(dB.data_ptr()), ldb, beta, ctypes.c_void_p(dC.data_ptr()), ldc,
                                    ctypes.c_void_p(stream))


def test_noalloc_gemm_matches_host_product_on_consecutive_calls():
    import torch
    from fermicc import _lib
    lib = _lib.load()
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    # consecutive calls on different data and shapes: the shared scratch keeps
    # nothing that a later call could pick up; the second and third use padded
    # leading dimensions (lda > K, ldb > N, ldc > N)
    cases = [(40, 24, 20000, 1.0, 0.0, 0, 0, 0), (96, 70, 9000, -0.7, 0.5, 5, 3, 7), (33, 129, 4100, 2.0, -1.0, 1, 9, 2)]
    for call, (M, N, K, alpha, beta, pa, pb, pc) in enumerate(cases):
        A = rng.standard_normal((M, K + pa))
        B = rng.standard_normal((K, N + pb))
        C = rng.standard_normal((M, N + pc))
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        dC = torch.from_numpy(C).cuda()
        torch.cuda.synchronize()
        rc = _call(lib, M, N, K, alpha, dA, K + pa, dB, N + pb, beta, dC, N + pc, stream)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        got = dC.cpu().numpy()
        ref = alpha * (A[:, :K] @ B[:, :N]) + beta * C[:, :N]
        assert np.abs(got[:, :N] - ref).max() <= TOL * max(1.0, np.abs(ref).max()), call
        # the padding columns of C are not written
        assert np.array_equal(got[:, N:], C[:, N:]), call


def test_noalloc_gemm_rejects_sizes_beyond_its_scratch():
    from fermicc import _lib
    lib = _lib.load()
    null = ctypes.c_void_p(0)
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size checks come first
    f = lib.fcc_gemm_f64_noalloc
    assert f(2048, 1024, 64, 1.0, dummy, 64, dummy, 1024, 0.0, dummy, 1024, null) == _lib.FCC_ERR_BAD_ARG
    assert f(0, 4, 4, 1.0, dummy, 4, dummy, 4, 0.0, dummy, 4, null) == _lib.FCC_ERR_BAD_ARG
    # M * N would wrap around in 64 bits: rejected before the product is formed
    big = 1 << 43
    assert f(big, 1 << 21, 4, 1.0, dummy, 4, dummy, 1 << 21, 0.0, dummy, 1 << 21, null) == _lib.FCC_ERR_BAD_ARG
    assert f(4, big, 4, 1.0, dummy, 4, dummy, big, 0.0, dummy, big, null) == _lib.FCC_ERR_BAD_ARG
    # leading dimensions shorter than the rows
    assert f(4, 4, 8, 1.0, dummy, 7, dummy, 4, 0.0, dummy, 4, null) == _lib.FCC_ERR_BAD_ARG
