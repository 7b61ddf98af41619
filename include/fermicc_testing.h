/*
 * fermicc_testing.h -- test hooks of libfermicc.so.
 *
 * These entry points have no counterpart in Fermi.jl.  They expose single
 * device contractions so the test suite can check each kernel against a
 * host reference in isolation.
 */
#ifndef FERMICC_TESTING_H
#define FERMICC_TESTING_H

#include <stdint.h>

#include "fermicc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C = alpha * einsum(spec, A, B) + beta * C on device 0 for row-major host
 * tensors (rank <= 4 each).  precision FCC_PREC_FP64 runs the DMMA kernel;
 * FCC_PREC_MIXED forces the three-product split-BF16 tensor-core kernel,
 * 2 the six-product one, 3 the exact-slice (Ozaki) kernel with 8 weight
 * groups and 10 + G the exact-slice kernel with G groups (2 <= G <= 9)
 * (error if the contraction cannot be expressed for it).  Returns an fcc
 * status code. */
int fcc_test_contract(int32_t precision, const char* spec, const double* A, const int64_t* adims, int32_t arank,
                      const double* B, const int64_t* bdims, int32_t brank, double* C, const int64_t* cdims,
                      int32_t crank, double alpha, double beta);

/* The three-piece BF16 split of the tensor-core operand packing on device 0:
 * x is R x K (row-major, or column-major when row_fastest != 0), multiplied
 * by scale; out receives R rows of 3K bf16 bit patterns, [hi(K) | mid(K) |
 * lo(K)] per row. */
int fcc_test_split3(const double* x, int64_t R, int64_t K, int32_t row_fastest, double scale, uint16_t* out);

/* The exact-slice operand packing on device 0: x is R x K (row-major, or
 * column-major when row_fastest != 0), cut into S (1..8) signed 6-bit digit
 * slices; out receives R rows of S * Kpad bf16 bit patterns (Kpad = K
 * rounded up to 64; slice s at columns [s * Kpad, s * Kpad + K), zeros to
 * (s + 1) * Kpad) and ex the R biased FP64 exponents of the row maxima. */
int fcc_test_pack_oz(const double* x, int64_t R, int64_t K, int32_t row_fastest, int32_t S, uint16_t* out,
                     int32_t* ex);

/* Number of kernels this library has launched in the process so far. */
int64_t fcc_stat_launches(void);

/* The CUDA stream (cudaStream_t) every call on ctx runs on, so a caller can
 * bracket library work with its own events. */
void* fcc_stream(const fcc_ctx* ctx);

/* Force the B tile width (128, 160, 192, 256; 0 = chosen from v) of the mixed
 * (T) GEMM, e.g. to run several column tiles on a small system. */
int fcc_test_set_t3_bn(fcc_ctx* ctx, int32_t bn);

/* Number of k values per mixed (T) launch (1..64; 0 = the default run
 * length), e.g. to compare run lengths or to cover several runs on a small
 * system. */
int fcc_test_set_t3_kc(fcc_ctx* ctx, int32_t kc);

/* One-shot failure injection on ctx for the error-path tests; nothing here
 * faults the GPU.  FCC_TEST_FAULT_NO_LOADS: the first split-BF16 tensor-core
 * GEMM of the next mixed-form fcc_ccsd_run issues no TMA loads, so its MMA
 * thread's bounded mbarrier wait (2 s) gives up with nothing in flight, the
 * kernel frees its TMEM and returns, and the run reports FCC_ERR_TIMEOUT.
 * FCC_TEST_FAULT_NAN: a NaN is written into the doubles residual of the next
 * iteration before the device update, which then reports FCC_ERR_NAN. */
#define FCC_TEST_FAULT_NO_LOADS 1
#define FCC_TEST_FAULT_NAN 2
int fcc_test_inject(fcc_ctx* ctx, int32_t kind);

/* FP64 (T) energy contributions of n single triplets ijk[3q..3q+2] = (i, j, k)
 * with i >= j >= k (0-based active occupied indices), each including its
 * weight 2 - d_ij - d_jk, from the current amplitudes (after fcc_ccsd_run);
 * the sum over all triplets is the FP64 E(T) that fcc_triples returns. */
int fcc_test_triples_subset(fcc_ctx* ctx, const int32_t* ijk, int32_t n, double* e_each);

/* Opt-in per-class kernel timing with CUDA events on the launching stream:
 * classes 0 FP64 contractions (work = 2MNK flop), 1 tensor-core GEMMs (work =
 * executed BF16 flop), 2 operand packing (work = bytes), 3 updates, 4 (T)
 * energy, 5 exact-slice GEMMs (work = executed BF16 flop).  fcc_prof_read fills out[4*c + {0,1,2,3}] = launches, total ms,
 * work, longest launch ms for c < ncls and clears the log. */
int fcc_prof_enable(int32_t on);
int fcc_prof_read(double* out, int32_t ncls);

#ifdef __cplusplus
}
#endif
#endif /* FERMICC_TESTING_H */
