// Split-BF16 tensor-core contraction: operand packing and the tcgen05 GEMM.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "fcc_common.cuh"

namespace fcc {

// Split schemes.  x = hi + mid + lo with hi = bf16(x), mid = bf16(x - hi),
// lo = bf16(x - hi - mid).  A product A.B is evaluated as a sum of P piece
// products, stored as P column blocks of the packed operands:
//   3 products: A' = [hi hi mid],          B' = [hi mid hi]          (~2^-16)
//   6 products: A' = [hi hi mid hi mid lo], B' = [hi mid hi lo mid hi] (~2^-24)
// Piece p of an operand holds level (code >> 2p) & 3 (0 hi, 1 mid, 2 lo).
struct SplitScheme {
  int P;
  uint32_t code_a, code_b;
};
constexpr SplitScheme SPLIT3{3, 0u | (0u << 2) | (1u << 4), 0u | (1u << 2) | (0u << 4)};
constexpr SplitScheme SPLIT6{6, 0u | (0u << 2) | (1u << 4) | (0u << 6) | (1u << 8) | (2u << 10),
                             0u | (1u << 2) | (0u << 4) | (2u << 6) | (1u << 8) | (0u << 10)};

// Gather spec of a packed operand: row r = (r1*rd2 + r2)*rd3 + r3 and column
// k = (k1*kd2 + k2)*kd3 + k3 of a strided FP64 source; the destination is
// R rows x Kp bf16 with split piece p at columns [p*K, (p+1)*K), zero from
// P*K to Kp.
struct PackSpec {
  int64_t R, K, Kp;
  int64_t rd2, rd3, rs1, rs2, rs3;
  int64_t kd2, kd3, ks1, ks2, ks3;
  int P = 3;
  uint32_t code = 0;
  double scale = 1.0;   // the source is multiplied by this (exact for +-1 and powers of two)
};

// Source offsets of packed row r and packed column k (32-bit index
// arithmetic: pack_split / pack_oz reject R or K of 2^31 or more).
__device__ __forceinline__ int64_t pack_row_off(const PackSpec& ps, int64_t r) {
  const uint32_t rr = (uint32_t)r, d3 = (uint32_t)ps.rd3, d2 = (uint32_t)ps.rd2;
  const uint32_t r3 = rr % d3, q = rr / d3;
  return (int64_t)(q / d2) * ps.rs1 + (int64_t)(q % d2) * ps.rs2 + (int64_t)r3 * ps.rs3;
}
__device__ __forceinline__ int64_t pack_col_off(const PackSpec& ps, int64_t k) {
  const uint32_t kk = (uint32_t)k, d3 = (uint32_t)ps.kd3, d2 = (uint32_t)ps.kd2;
  const uint32_t k3 = kk % d3, q = kk / d3;
  return (int64_t)(q / d2) * ps.ks1 + (int64_t)(q % d2) * ps.ks2 + (int64_t)k3 * ps.ks3;
}
// Walks consecutive packed columns k, k+1, ... without divisions.
struct PackColIter {
  uint32_t k2, k3;
  int64_t off;
  __device__ __forceinline__ PackColIter(const PackSpec& ps, int64_t k) {
    const uint32_t kk = (uint32_t)k, d3 = (uint32_t)ps.kd3, d2 = (uint32_t)ps.kd2;
    k3 = kk % d3;
    const uint32_t q = kk / d3;
    k2 = q % d2;
    off = (int64_t)(q / d2) * ps.ks1 + (int64_t)k2 * ps.ks2 + (int64_t)k3 * ps.ks3;
  }
  __device__ __forceinline__ void next(const PackSpec& ps) {
    if (++k3 < (uint32_t)ps.kd3) { off += ps.ks3; return; }
    k3 = 0;
    off += ps.ks2 - (ps.kd3 - 1) * ps.ks3;
    if (++k2 < (uint32_t)ps.kd2) return;
    k2 = 0;
    off += ps.ks1 - ps.kd2 * ps.ks2;   // from (k1, kd2, 0) to (k1 + 1, 0, 0)
  }
};

// k is one source index (k3 = k): column offset k * ks3, no divisions
__host__ __device__ inline bool pack_k_single(const PackSpec& ps) { return ps.kd2 == 1 && ps.kd3 >= ps.K; }

// Source values of packed columns k0 .. k0 + cnt - 1 (cnt <= 4) of the row at
// source offset ro; zeros past cnt.
__device__ __forceinline__ void pack_load4(const double* __restrict__ src, const PackSpec& ps, bool k1, int64_t ro,
                                           int64_t k0, int cnt, double (&x)[4]) {
  if (k1) {
    const double* sp = src + ro + k0 * ps.ks3;
#pragma unroll
    for (int q = 0; q < 4; ++q) x[q] = q < cnt ? sp[q * ps.ks3] : 0.0;
  } else {
    PackColIter ci(ps, k0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      x[q] = q < cnt ? src[ro + ci.off] : 0.0;
      if (q + 1 < cnt) ci.next(ps);
    }
  }
}

// Row walk of the row-major pack kernels: a unit is a segment of gseg
// 4-column groups of one packed row (nseg segments per row), walked by 2^lg
// threads (32 ... 256); 256 >> lg units per block of 256 threads.  Rows are
// cut into segments when there are too few of them to fill the GPU.
struct PackWalk {
  int lg;
  int64_t gseg, nseg;
};
inline PackWalk pack_walk(int64_t R, int64_t groups) {
  PackWalk w;
  w.lg = 5;
  while (w.lg < 8 && (int64_t(1) << w.lg) < groups) ++w.lg;
  const int64_t tpr = int64_t(1) << w.lg;
  // about 152 SMs x 2048 threads, up to 8 groups each
  const int64_t per_thread = std::max<int64_t>(1, std::min<int64_t>(8, R * groups / (152 * 2048)));
  w.gseg = std::min(groups, tpr * per_thread);
  w.nseg = (groups + w.gseg - 1) / w.gseg;
  return w;
}
inline unsigned pack_walk_grid(const PackWalk& w, int64_t R) {
  const int64_t upb = 256 >> w.lg;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((R * w.nseg + upb - 1) / upb, 152 * 32));
}

// Output scatter of the GEMM: element (m, n) goes to
// C[m1*ms1 + m2*ms2 + m3*ms3 + n1*ns1 + n2*ns2 + n3*ns3] as
//   EPI_F64 / EPI_F32: alpha * acc + beta * C (atomic add when split over K);
//   EPI_SPLIT: the split pieces of alpha * acc written at offsets p * piece
//              (levels per `code`, P pieces), i.e. straight into the packed
//              operand of a following GEMM.
enum { EPI_F64 = 0, EPI_F32 = 1, EPI_SPLIT = 2 };
struct EpiMap {
  int64_t M = 0, N = 0;
  int64_t md2 = 1, md3 = 1, ms1 = 0, ms2 = 0, ms3 = 0;
  int64_t nd2 = 1, nd3 = 1, ns1 = 0, ns2 = 0, ns3 = 0;
  double alpha = 1.0, beta = 0.0;
  void* C = nullptr;
  int mode = EPI_F64;
  int atomic = 0;
  int64_t piece = 0;
  int P = 3;
  uint32_t code = 0;
  double work = 0.0;   // algorithmic BF16 flops for the timing log (0: use the padded count)
  int no_loads = 0;    // test hook: the producer issues no TMA loads, so the bounded waits give up
};

int64_t packed_kp(int64_t K, int P = 3);
void pack_split(const double* src, const PackSpec& ps, __nv_bfloat16* dst, cudaStream_t s);
// D = A' B'^T over Kp packed columns; rows a_row0.. of A' (a_rows total) and
// b_row0.. of B' (b_rows total); err set to 1 if a bounded wait gave up.
void gemm_bf16x3(const __nv_bfloat16* A, int64_t a_rows, int64_t a_row0, const __nv_bfloat16* B, int64_t b_rows,
                 int64_t b_row0, int64_t Kp, const EpiMap& ep, int* err, cudaStream_t s);

// 2-D TMA map over a row-major [rows][cols] BF16 array, boxes of 64 columns
// (one 128-byte swizzle atom) x box_rows rows; cols must be a multiple of 64.
CUtensorMap tma_map_bf16(const __nv_bfloat16* base, int64_t rows, int64_t cols, int box_rows);
// C = beta * C over an epilogue map (before a GEMM adds into C atomically)
void scale_output(const EpiMap& ep, double beta, cudaStream_t s);

// Exact-slice products (the Ozaki scheme: Ozaki, Ogita, Oishi & Rump, Numer.
// Algorithms 59, 95 (2012); on tensor cores: Mukunoki et al., ISC 2020).
// Each row r of an operand is scaled by 2^e_r (|x| < 2^e_r over the row) and
// cut into S = G-1 signed 6-bit digit slices, x = 2^e_r sum_s d_s 2^(-6(s+1)),
// |d| <= 64, stored exactly in BF16.  A.B^T is the sum over slice pairs
// (s, t) with s + t + 2 <= G of the digit products; pairs of one weight
// 2^(-6(s+t+2)) are summed on the tensor cores in FP32 over chunks of 2048
// products (|sum| <= 2^23, so every partial sum is an exact integer) and the
// chunks are added in double-FP32 (~2^-48 relative) in TMEM.  The result
// carries the slice truncation error, ~2^(-6(G-1)) of max|A_r| max|B_c| per
// term (G = 8: ~1e-12 of max|C| for Gaussian operands).
constexpr int OZ_G_DEFAULT = 8;
// packed layout: row r holds slice s at columns [s*Kpad, s*Kpad + K), zero up
// to (s+1)*Kpad; ex[r] = biased FP64 exponent of max_k |x_rk| (0: all zero)
int64_t oz_kpad(int64_t K);
void pack_oz(const double* src, const PackSpec& ps, int S, __nv_bfloat16* dst, int* ex, cudaStream_t s);
// FP64 epilogue (EPI_F64) of the exact-slice product over packed operands
void gemm_oz(const __nv_bfloat16* A, int64_t a_rows, const int* exA, const __nv_bfloat16* B, int64_t b_rows,
             const int* exB, int64_t Kpad, int G, const EpiMap& ep, int* err, cudaStream_t s);

// Engine state for einsum calls that run on the tensor cores: scratch for
// the packed operands, the device error flag, the routing threshold and
// counters of what ran.
struct TcEngine {
  bool enabled = false;
  SplitScheme scheme = SPLIT3;
  bool exact = false;      // exact-slice products instead of the split scheme
  int oz_groups = OZ_G_DEFAULT;
  DBuf<int> exA, exB;
  double min_flops = 1e6;
  int64_t min_dim = 16;   // smallest M and N routed to the tensor cores
  DBuf<__nv_bfloat16> bufA, bufB;
  int* err = nullptr;
  int no_loads_once = 0;   // test hook: the next split-BF16 GEMM runs with EpiMap::no_loads
  // Packed A operands kept across calls: an A operand whose source is one of
  // keep_src (set by a KeepPackedA scope, whose caller guarantees that those
  // sources do not change meanwhile) is packed into its own entry and packed
  // again only when its layout or slice count changes, so an operand used by
  // every block of a loop is packed once.
  struct KeptPack {
    PackSpec ps{};
    int S = 0;
    bool valid = false;
    DBuf<__nv_bfloat16> buf;
    DBuf<int> ex;
  };
  const double* keep_src[2] = {nullptr, nullptr};
  KeptPack kept[2];
  int64_t tc_calls = 0, f64_calls = 0;
  double tc_flops = 0, f64_flops = 0;
};

// Keep the packed forms of the A operands with sources a0 and a1 over the
// following contractions; they are dropped when the scope ends.
struct KeepPackedA {
  TcEngine* tc;
  KeepPackedA(TcEngine* e, const double* a0, const double* a1) : tc(e) {
    if (!tc) return;
    tc->keep_src[0] = a0;
    tc->keep_src[1] = a1;
    for (auto& k : tc->kept) k.valid = false;
  }
  ~KeepPackedA() {
    if (!tc) return;
    tc->keep_src[0] = tc->keep_src[1] = nullptr;
    for (auto& k : tc->kept) k.valid = false;
  }
};

// Current engine of this host thread (nullptr: every contraction is FP64).
TcEngine*& tc_engine();

struct TcScope {
  TcEngine* prev;
  explicit TcScope(TcEngine* e) : prev(tc_engine()) { tc_engine() = e; }
  ~TcScope() { tc_engine() = prev; }
};

}  // namespace fcc
