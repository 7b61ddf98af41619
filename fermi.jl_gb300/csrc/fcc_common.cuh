// Shared definitions for the GB300 coupled-cluster library (libfermicc).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/fermicc.h"

namespace fcc {

// Internal exception carrying an fcc status code; converted to a return code
// at the C ABI so nothing ever aborts the caller's process.
struct Error {
  int code;
  std::string what;
};

[[noreturn]] inline void fail(int code, const std::string& what) { throw Error{code, what}; }

#define FCC_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e__ = (call);                                                                   \
    if (e__ != cudaSuccess)                                                                     \
      ::fcc::fail(e__ == cudaErrorMemoryAllocation ? FCC_ERR_OOM : FCC_ERR_CUDA,                \
                  std::string(#call) + ": " + cudaGetErrorString(e__));                         \
  } while (0)

// Every kernel launch site is followed by this check, which also counts the
// launch (the count is exposed for measurement through fcc_stat_launches).
void note_launch();
#define FCC_CHECK_LAUNCH()          \
  do {                              \
    ::fcc::note_launch();           \
    FCC_CUDA(cudaGetLastError());   \
  } while (0)

// Opt-in kernel timing (csrc/prof.cu): classes of work.
enum { PROF_F64 = 0, PROF_TC = 1, PROF_PACK = 2, PROF_UPDATE = 3, PROF_TRIPLES = 4, PROF_OZ = 5, PROF_NCLS = 6 };
int prof_begin(cudaStream_t s);
void prof_end(cudaStream_t s, int idx, int cls, double work);

// Device buffer owned by a context.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    FCC_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void zero(cudaStream_t s) { if (p) FCC_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s)); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Split-K partial sums of the FP64 contraction go to a buffer owned by the
// context (or DF-RHF handle) whose call runs on this host thread, so two
// contexts never share one: contexts may sit on different devices or
// streams.  Entry points install their buffer with WorkspaceScope; without
// one, contract_f64_launch allocates a buffer for the call and frees it
// before returning (cudaFree waits for the device).
DBuf<double>*& f64_workspace();
struct WorkspaceScope {
  DBuf<double>* prev;
  explicit WorkspaceScope(DBuf<double>* w) : prev(f64_workspace()) { f64_workspace() = w; }
  ~WorkspaceScope() { f64_workspace() = prev; }
  WorkspaceScope(const WorkspaceScope&) = delete;
  WorkspaceScope& operator=(const WorkspaceScope&) = delete;
};

// A strided view of a device tensor with up to 4 named indices.
struct TView {
  double* p = nullptr;
  int rank = 0;
  int64_t dim[4] = {1, 1, 1, 1};
  int64_t str[4] = {0, 0, 0, 0};
};

// Row-major view (last index fastest) over a contiguous buffer.
inline TView rm(double* p, std::initializer_list<int64_t> dims) {
  TView t;
  t.p = p;
  t.rank = (int)dims.size();
  int k = 0;
  for (auto d : dims) t.dim[k++] = d;
  int64_t s = 1;
  for (int i = t.rank - 1; i >= 0; --i) { t.str[i] = s; s *= t.dim[i]; }
  return t;
}
// Column-major view (first index fastest), the layout of Julia arrays.
inline TView cm(double* p, std::initializer_list<int64_t> dims) {
  TView t;
  t.p = p;
  t.rank = (int)dims.size();
  int k = 0;
  for (auto d : dims) t.dim[k++] = d;
  int64_t s = 1;
  for (int i = 0; i < t.rank; ++i) { t.str[i] = s; s *= t.dim[i]; }
  return t;
}
// Sub-range of one index (offsets the pointer, shrinks the extent).
inline TView slice(TView t, int idx, int64_t begin, int64_t count) {
  t.p += begin * t.str[idx];
  t.dim[idx] = count;
  return t;
}

// ---------------------------------------------------------------- kernels
// Contraction descriptor consumed by the FP64 kernel: M = M1*M2*M3,
// N = N1*N2*N3, K = K1*K2 with independent strides for every sub-index
// (m = (m1*M2 + m2)*M3 + m3, likewise n and k), plus a batch index with
// uniform strides.  M3 = N3 = 1 with zero strides gives two-level groups.
struct CtrDesc {
  int64_t M, N, K, M2, N2, K2, batch;
  int64_t a_m1, a_m2, a_k1, a_k2, a_b;
  int64_t b_k1, b_k2, b_n1, b_n2, b_b;
  int64_t c_m1, c_m2, c_n1, c_n2, c_b;
  double alpha, beta;
  int64_t M3 = 1, N3 = 1;
  int64_t a_m3 = 0, c_m3 = 0, b_n3 = 0, c_n3 = 0;
};

void contract_f64_launch(const double* A, const double* B, double* C, const CtrDesc& d, cudaStream_t s);

// out[perm] = alpha * in + beta * out over a 4-index box (general strides).
void tensor_axpby_launch(const TView& in, const TView& out, double alpha, double beta, cudaStream_t s);

// Einsum front end: C = alpha * contract(A, B) + beta * C.  Subscripts use
// single letters; every index of C must appear in A or B.  Indices are
// grouped into batch (A,B,C), M (A,C), N (B,C) and K (A,B); M and N may hold
// up to three indices, K two and batch one (after fusing indices that are
// contiguous in every operand).
void einsum(double alpha, const char* spec, const TView& A, const TView& B, double beta, const TView& C,
            cudaStream_t s);
// Single-operand form "abcd->dcba": C = alpha * permute(A) + beta * C.
void einsum1(double alpha, const char* spec, const TView& A, double beta, const TView& C, cudaStream_t s);

}  // namespace fcc
