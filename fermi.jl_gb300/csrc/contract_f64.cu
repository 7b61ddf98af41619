// FP64 tensor contraction on the DMMA pipe (mma.sync m8n8k4 .f64) and the
// einsum-style front end used by the CCSD driver.
//
// Every contraction of the amplitude equations is C = alpha * A.B + beta * C
// where the M, N and K matrix indices are each a pair of tensor indices with
// arbitrary strides, so index permutations are folded into the loads and
// stores instead of separate transpose passes.  On GB300 the FP64 pipe
// (about 1 TFLOP/s per GPU) is the bound of this kernel; a 64x64 tile with
// 16-deep K steps staged through shared memory keeps it saturated.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>

#include "fcc_common.cuh"
#include "fcc_tc.cuh"

namespace fcc {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 128;
constexpr int LDS = BM + 8;  // 72 doubles: rows 64 B apart modulo 128 B

__device__ __forceinline__ void dmma884(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(NT) contract_f64_kernel(const double* __restrict__ A,
                                                          const double* __restrict__ B,
                                                          double* __restrict__ C, CtrDesc d,
                                                          int a_mfast, int b_nfast, int64_t k_chunk,
                                                          double* __restrict__ partial) {
  __shared__ double As[BK][LDS];
  __shared__ double Bs[BK][LDS];
  __shared__ int64_t rowA[BM], colB[BN];
  __shared__ int8_t rowOK[BM], colOK[BN];

  const int tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  // blockIdx.z: batch index, or the K slice when split over K (partial != 0)
  const int64_t bz = partial ? 0 : blockIdx.z;
  const int64_t kbeg = partial ? (int64_t)blockIdx.z * k_chunk : 0;
  const int64_t kend = partial ? min(d.K, kbeg + k_chunk) : d.K;
  A += bz * d.a_b;
  B += bz * d.b_b;
  C += bz * d.c_b;

  if (tid < BM) {
    int64_t m = m0 + tid;
    bool ok = m < d.M;
    int64_t m1 = ok ? m / d.M2 : 0, m2 = ok ? m - m1 * d.M2 : 0;
    rowA[tid] = m1 * d.a_m1 + m2 * d.a_m2;
    rowOK[tid] = ok;
  } else {
    int t = tid - BM;
    int64_t n = n0 + t;
    bool ok = n < d.N;
    int64_t n1 = ok ? n / d.N2 : 0, n2 = ok ? n - n1 * d.N2 : 0;
    colB[t] = n1 * d.b_n1 + n2 * d.b_n2;
    colOK[t] = ok;
  }
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
    // ---- stage A (BM x BK) and B (BK x BN) into shared memory
    if (a_mfast) {
      int m = tid & 63, kb = tid >> 6;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int kk = kb + 2 * r;
        int64_t k = k0 + kk;
        double v = 0.0;
        if (rowOK[m] && k < kend) {
          int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
          v = A[rowA[m] + k1 * d.a_k1 + k2 * d.a_k2];
        }
        As[kk][m] = v;
      }
    } else {
      int kk = tid & 15, mb = tid >> 4;
      int64_t k = k0 + kk;
      bool kok = k < kend;
      int64_t koff = 0;
      if (kok) {
        int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
        koff = k1 * d.a_k1 + k2 * d.a_k2;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int m = mb + 8 * r;
        As[kk][m] = (kok && rowOK[m]) ? A[rowA[m] + koff] : 0.0;
      }
    }
    if (b_nfast) {
      int n = tid & 63, kb = tid >> 6;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int kk = kb + 2 * r;
        int64_t k = k0 + kk;
        double v = 0.0;
        if (colOK[n] && k < kend) {
          int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
          v = B[colB[n] + k1 * d.b_k1 + k2 * d.b_k2];
        }
        Bs[kk][n] = v;
      }
    } else {
      int kk = tid & 15, nb = tid >> 4;
      int64_t k = k0 + kk;
      bool kok = k < kend;
      int64_t koff = 0;
      if (kok) {
        int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
        koff = k1 * d.b_k1 + k2 * d.b_k2;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int n = nb + 8 * r;
        Bs[kk][n] = (kok && colOK[n]) ? B[colB[n] + koff] : 0.0;
      }
    }
    __syncthreads();
    // ---- 4 k-steps of m8n8k4 per 16-deep tile
#pragma unroll
    for (int ks = 0; ks < BK; ks += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[ks + (lane & 3)][wm + 8 * i + (lane >> 2)];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[ks + (lane & 3)][wn + 8 * j + (lane >> 2)];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma884(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    __syncthreads();
  }

  // ---- epilogue: C = alpha * acc + beta * C with general output strides
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int ml = wm + 8 * i + (lane >> 2);
    int64_t m = m0 + ml;
    if (m >= d.M) continue;
    int64_t m1 = m / d.M2, m2 = m - m1 * d.M2;
    int64_t crow = m1 * d.c_m1 + m2 * d.c_m2;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int64_t n = n0 + wn + 8 * j + 2 * (lane & 3) + h;
        if (n >= d.N) continue;
        if (partial) {   // split-K: raw partial sums, reduced in a fixed order later
          partial[((int64_t)blockIdx.z * d.M + m) * d.N + n] = acc[i][j][h];
          continue;
        }
        int64_t n1 = n / d.N2, n2 = n - n1 * d.N2;
        double* dst = C + crow + n1 * d.c_n1 + n2 * d.c_n2;
        double v = d.alpha * acc[i][j][h];
        if (d.beta != 0.0) v += d.beta * *dst;
        *dst = v;
      }
    }
  }
}

// C = alpha * sum_z partial[z] + beta * C, summed in slice order.
__global__ void splitk_reduce_kernel(const double* __restrict__ partial, int splits, double* __restrict__ C,
                                     CtrDesc d) {
  const int64_t MN = d.M * d.N;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < MN; t += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; ++z) s += partial[(int64_t)z * MN + t];
    const int64_t m = t / d.N, n = t - m * d.N;
    const int64_t m1 = m / d.M2, m2 = m - m1 * d.M2, n1 = n / d.N2, n2 = n - n1 * d.N2;
    double* dst = C + m1 * d.c_m1 + m2 * d.c_m2 + n1 * d.c_n1 + n2 * d.c_n2;
    double v = d.alpha * s;
    if (d.beta != 0.0) v += d.beta * *dst;
    *dst = v;
  }
}

// N == 1 (matrix-vector): one warp per output row, lanes stride over K.
__global__ void gemv_f64_kernel(const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C,
                                CtrDesc d) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t bz = blockIdx.y;
  A += bz * d.a_b;
  B += bz * d.b_b;
  C += bz * d.c_b;
  for (int64_t m = warp; m < d.M; m += nwarps) {
    const int64_t m1 = m / d.M2, m2 = m - m1 * d.M2;
    const double* a = A + m1 * d.a_m1 + m2 * d.a_m2;
    double s = 0.0;
    for (int64_t k = lane; k < d.K; k += 32) {
      const int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
      s += a[k1 * d.a_k1 + k2 * d.a_k2] * B[k1 * d.b_k1 + k2 * d.b_k2];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      double* dst = C + m1 * d.c_m1 + m2 * d.c_m2;
      double v = d.alpha * s;
      if (d.beta != 0.0) v += d.beta * *dst;
      *dst = v;
    }
  }
}

__global__ void axpby4_kernel(const double* __restrict__ in, double* __restrict__ out, int64_t d0,
                              int64_t d1, int64_t d2, int64_t d3, int64_t si0, int64_t si1, int64_t si2,
                              int64_t si3, int64_t so0, int64_t so1, int64_t so2, int64_t so3,
                              double alpha, double beta, int64_t total) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    int64_t i3 = r % d3; r /= d3;
    int64_t i2 = r % d2; r /= d2;
    int64_t i1 = r % d1; r /= d1;
    int64_t i0 = r;
    double v = alpha * in[i0 * si0 + i1 * si1 + i2 * si2 + i3 * si3];
    double* o = out + i0 * so0 + i1 * so1 + i2 * so2 + i3 * so3;
    if (beta != 0.0) v += beta * *o;
    *o = v;
  }
}

}  // namespace

void contract_f64_launch(const double* A, const double* B, double* C, const CtrDesc& d, cudaStream_t s) {
  if (d.M <= 0 || d.N <= 0 || d.batch <= 0) return;
  int64_t gm = (d.M + BM - 1) / BM, gn = (d.N + BN - 1) / BN;
  if (gn > 65535 || d.batch > 65535) fail(FCC_ERR_BAD_ARG, "contraction grid too large");
  if (d.K <= 0) fail(FCC_ERR_BAD_ARG, "empty contraction index");
  const int pidx = prof_begin(s);
  const double pflops = 2.0 * (double)d.M * (double)d.N * (double)d.K * (double)d.batch;
  if (d.N == 1) {
    const int64_t blocks = std::min<int64_t>((d.M + 7) / 8, 152 * 16);
    gemv_f64_kernel<<<dim3((unsigned)blocks, (unsigned)d.batch), 256, 0, s>>>(A, B, C, d);
    FCC_CHECK_LAUNCH();
    prof_end(s, pidx, PROF_F64, pflops);
    return;
  }
  // fewer output tiles than one wave of resident CTAs (96 registers x 128
  // threads: 5 per SM) and a long K: split K so that about 8 CTAs per SM
  // share the work (partials reduced in a fixed order, so results stay
  // deterministic).  Under one wave the FP64 pipe idles on DMMA latency:
  // 387 CTAs ran at 0.8 TFLOP/s where 1216 reach 1.08.
  constexpr int64_t WAVE_CTAS = 5 * 152, SPLIT_CTAS = 8 * 152;
  if (d.batch == 1 && gm * gn < WAVE_CTAS && d.K >= 32 * BK) {
    int64_t splits = std::min<int64_t>((SPLIT_CTAS + gm * gn - 1) / (gm * gn), d.K / (8 * BK));
    splits = std::max<int64_t>(2, std::min<int64_t>(splits, 1024));
    const int64_t chunk = ((d.K + splits - 1) / splits + BK - 1) / BK * BK;
    splits = (d.K + chunk - 1) / chunk;
    static thread_local DBuf<double> scratch;
    const int64_t need = splits * d.M * d.N;
    if ((int64_t)scratch.n < need) scratch.alloc(need);
    dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)splits);
    contract_f64_kernel<<<grid, NT, 0, s>>>(A, B, C, d, d.a_m2 == 1 ? 1 : 0, d.b_n2 == 1 ? 1 : 0, chunk, scratch.p);
    FCC_CHECK_LAUNCH();
    const int64_t MN = d.M * d.N;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>((MN + 255) / 256, 152 * 8), 256, 0, s>>>(scratch.p, (int)splits,
                                                                                                 C, d);
    FCC_CHECK_LAUNCH();
    prof_end(s, pidx, PROF_F64, pflops);
    return;
  }
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)d.batch);
  contract_f64_kernel<<<grid, NT, 0, s>>>(A, B, C, d, d.a_m2 == 1 ? 1 : 0, d.b_n2 == 1 ? 1 : 0, d.K, nullptr);
  FCC_CHECK_LAUNCH();
  prof_end(s, pidx, PROF_F64, pflops);
}

void tensor_axpby_launch(const TView& in, const TView& out, double alpha, double beta, cudaStream_t s) {
  int64_t total = out.dim[0] * out.dim[1] * out.dim[2] * out.dim[3];
  if (total <= 0) return;
  int threads = 256;
  int64_t blocks = std::min<int64_t>((total + threads - 1) / threads, 152 * 32);
  axpby4_kernel<<<(unsigned)blocks, threads, 0, s>>>(in.p, out.p, out.dim[0], out.dim[1], out.dim[2],
                                                      out.dim[3], in.str[0], in.str[1], in.str[2],
                                                      in.str[3], out.str[0], out.str[1], out.str[2],
                                                      out.str[3], alpha, beta, total);
  FCC_CHECK_LAUNCH();
}

// ------------------------------------------------------------ einsum front end
namespace {

struct Operand {
  std::string idx;
  const TView* t;
  int pos(char c) const { auto p = idx.find(c); return p == std::string::npos ? -1 : (int)p; }
  int64_t stride(char c) const { int p = pos(c); return p < 0 ? 0 : t->str[p]; }
  int64_t dim(char c) const { int p = pos(c); return p < 0 ? 1 : t->dim[p]; }
};

// A merged index: extent plus the stride it has in each operand.
struct Ix {
  int64_t dim;
  int64_t s[3];
};

void parse(const char* spec, std::vector<std::string>& ins, std::string& out) {
  std::string s(spec);
  auto arrow = s.find("->");
  if (arrow == std::string::npos) fail(FCC_ERR_BAD_ARG, std::string("einsum spec without ->: ") + spec);
  out = s.substr(arrow + 2);
  std::string lhs = s.substr(0, arrow);
  size_t start = 0;
  while (true) {
    auto c = lhs.find(',', start);
    ins.push_back(lhs.substr(start, c == std::string::npos ? std::string::npos : c - start));
    if (c == std::string::npos) break;
    start = c + 1;
  }
}

// Fuse indices of a group until it has at most `cap` members; two indices x
// (slower) and y (faster) fuse when str[x] == dim[y] * str[y] in every operand.
bool try_fuse(std::vector<Ix>& g, int cap) {
  while ((int)g.size() > cap) {
    bool done = false;
    for (size_t x = 0; x < g.size() && !done; ++x)
      for (size_t y = 0; y < g.size() && !done; ++y) {
        if (x == y) continue;
        bool ok = true;
        for (int o = 0; o < 3; ++o) {
          bool zx = g[x].s[o] == 0, zy = g[y].s[o] == 0;
          if (zx != zy) { ok = false; break; }
          if (!zx && g[x].s[o] != g[y].dim * g[y].s[o]) { ok = false; break; }
        }
        if (ok) {
          g[y].dim *= g[x].dim;
          g.erase(g.begin() + x);
          done = true;
        }
      }
    if (!done) return false;
  }
  return true;
}

void fuse(std::vector<Ix>& g, int cap, const char* spec) {
  if (!try_fuse(g, cap)) fail(FCC_ERR_BAD_ARG, std::string("einsum group not reducible to ") + std::to_string(cap) + " indices: " + spec);
}

int64_t gdim(const std::vector<Ix>& g) {
  int64_t d = 1;
  for (auto& x : g) d *= x.dim;
  return d;
}

// pad a group to exactly 3 levels (slowest first)
void pad3(std::vector<Ix>& g) { while (g.size() < 3) g.insert(g.begin(), Ix{1, {0, 0, 0}}); }

// Tensor-core evaluation of C = alpha * A.B + beta * C (no batch index).
void run_tc(TcEngine* tc, double alpha, const TView& A, const TView& B, double beta, const TView& C,
            std::vector<Ix> gm, std::vector<Ix> gn, std::vector<Ix> gk, cudaStream_t s) {
  // fastest-moving member last: the one with the smallest stride in the operand that is read along it
  auto order = [](std::vector<Ix>& g, int op) {
    std::stable_sort(g.begin(), g.end(), [op](const Ix& a, const Ix& b) { return std::llabs(a.s[op]) > std::llabs(b.s[op]); });
  };
  order(gm, 2);
  order(gn, 2);
  order(gk, 0);
  pad3(gm); pad3(gn); pad3(gk);
  const int64_t M = gdim(gm), N = gdim(gn), K = gdim(gk);
  if (tc->exact) {
    // exact-slice products: S digit slices of each operand, FP64 output
    const int G = tc->oz_groups, S = G - 1;
    const int64_t Kpad = oz_kpad(K), W = S * Kpad;
    if ((int64_t)tc->bufA.n < M * W) tc->bufA.alloc(M * W);
    if ((int64_t)tc->bufB.n < N * W) tc->bufB.alloc(N * W);
    if ((int64_t)tc->exA.n < M) tc->exA.alloc(M);
    if ((int64_t)tc->exB.n < N) tc->exB.alloc(N);
    PackSpec pa{M, K, W, gm[1].dim, gm[2].dim, gm[0].s[0], gm[1].s[0], gm[2].s[0],
                gk[1].dim, gk[2].dim, gk[0].s[0], gk[1].s[0], gk[2].s[0], S, 0};
    PackSpec pb{N, K, W, gn[1].dim, gn[2].dim, gn[0].s[1], gn[1].s[1], gn[2].s[1],
                gk[1].dim, gk[2].dim, gk[0].s[1], gk[1].s[1], gk[2].s[1], S, 0};
    pack_oz(A.p, pa, S, tc->bufA.p, tc->exA.p, s);
    pack_oz(B.p, pb, S, tc->bufB.p, tc->exB.p, s);
    EpiMap ep;
    ep.M = M; ep.N = N;
    ep.md2 = gm[1].dim; ep.md3 = gm[2].dim; ep.ms1 = gm[0].s[2]; ep.ms2 = gm[1].s[2]; ep.ms3 = gm[2].s[2];
    ep.nd2 = gn[1].dim; ep.nd3 = gn[2].dim; ep.ns1 = gn[0].s[2]; ep.ns2 = gn[1].s[2]; ep.ns3 = gn[2].s[2];
    ep.alpha = alpha; ep.beta = beta; ep.C = C.p; ep.mode = EPI_F64;
    const double npairs = (double)(G - 1) * (double)G / 2.0;
    ep.work = 2.0 * (double)M * (double)N * (double)K * npairs;
    gemm_oz(tc->bufA.p, M, tc->exA.p, tc->bufB.p, N, tc->exB.p, Kpad, G, ep, tc->err, s);
    tc->tc_calls++;
    tc->tc_flops += ep.work;
    return;
  }
  const SplitScheme sc = tc->scheme;
  const int64_t Kp = packed_kp(K, sc.P);
  if ((int64_t)tc->bufA.n < M * Kp) tc->bufA.alloc(M * Kp);
  if ((int64_t)tc->bufB.n < N * Kp) tc->bufB.alloc(N * Kp);
  PackSpec pa{M, K, Kp, gm[1].dim, gm[2].dim, gm[0].s[0], gm[1].s[0], gm[2].s[0],
              gk[1].dim, gk[2].dim, gk[0].s[0], gk[1].s[0], gk[2].s[0], sc.P, sc.code_a};
  PackSpec pb{N, K, Kp, gn[1].dim, gn[2].dim, gn[0].s[1], gn[1].s[1], gn[2].s[1],
              gk[1].dim, gk[2].dim, gk[0].s[1], gk[1].s[1], gk[2].s[1], sc.P, sc.code_b};
  pack_split(A.p, pa, tc->bufA.p, s);
  pack_split(B.p, pb, tc->bufB.p, s);
  EpiMap ep;
  ep.M = M; ep.N = N;
  ep.md2 = gm[1].dim; ep.md3 = gm[2].dim; ep.ms1 = gm[0].s[2]; ep.ms2 = gm[1].s[2]; ep.ms3 = gm[2].s[2];
  ep.nd2 = gn[1].dim; ep.nd3 = gn[2].dim; ep.ns1 = gn[0].s[2]; ep.ns2 = gn[1].s[2]; ep.ns3 = gn[2].s[2];
  ep.alpha = alpha; ep.beta = beta; ep.C = C.p; ep.mode = EPI_F64;
  ep.work = 2.0 * (double)M * (double)N * (double)K * sc.P;
  gemm_bf16x3(tc->bufA.p, M, 0, tc->bufB.p, N, 0, Kp, ep, tc->err, s);
  tc->tc_calls++;
  tc->tc_flops += 2.0 * (double)M * (double)N * (double)K * sc.P;
}

}  // namespace

static std::atomic<int64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

TcEngine*& tc_engine() {
  thread_local TcEngine* e = nullptr;
  return e;
}

void einsum(double alpha, const char* spec, const TView& A, const TView& B, double beta, const TView& C,
            cudaStream_t s) {
  std::vector<std::string> ins;
  std::string out;
  parse(spec, ins, out);
  if (ins.size() != 2) fail(FCC_ERR_BAD_ARG, std::string("einsum expects two operands: ") + spec);
  Operand oa{ins[0], &A}, ob{ins[1], &B}, oc{out, &C};
  if ((int)oa.idx.size() != A.rank || (int)ob.idx.size() != B.rank || (int)oc.idx.size() != C.rank)
    fail(FCC_ERR_BAD_ARG, std::string("einsum rank mismatch: ") + spec);
  std::string letters;
  for (auto& str : {oa.idx, ob.idx, oc.idx})
    for (char c : str)
      if (letters.find(c) == std::string::npos) letters += c;
  std::vector<Ix> gb, gm, gn, gk;
  for (char c : letters) {
    bool ia = oa.pos(c) >= 0, ib = ob.pos(c) >= 0, ic = oc.pos(c) >= 0;
    int64_t dim = std::max({oa.dim(c), ob.dim(c), oc.dim(c)});
    for (auto* op : {&oa, &ob, &oc})
      if (op->pos(c) >= 0 && op->dim(c) != dim)
        fail(FCC_ERR_BAD_ARG, std::string("einsum extent mismatch for '") + c + "': " + spec);
    Ix ix{dim, {oa.stride(c), ob.stride(c), oc.stride(c)}};
    if (ia && ib && ic) gb.push_back(ix);
    else if (ia && ic) gm.push_back(ix);
    else if (ib && ic) gn.push_back(ix);
    else if (ia && ib) gk.push_back(ix);
    else fail(FCC_ERR_BAD_ARG, std::string("einsum index in one operand only: ") + spec);
  }
  TcEngine* tc = tc_engine();
  if (tc && tc->enabled && gb.empty()) {
    const double flops = 2.0 * (double)gdim(gm) * (double)gdim(gn) * (double)gdim(gk);
    std::vector<Ix> m3 = gm, n3 = gn, k3 = gk;
    if (flops >= tc->min_flops && gdim(gm) >= tc->min_dim && gdim(gn) >= tc->min_dim && try_fuse(m3, 3) && try_fuse(n3, 3) &&
        try_fuse(k3, 3)) {
      run_tc(tc, alpha, A, B, beta, C, m3, n3, k3, s);
      return;
    }
  }
  fuse(gb, 1, spec);
  fuse(gm, 2, spec);
  fuse(gn, 2, spec);
  fuse(gk, 2, spec);
  if (tc) {
    tc->f64_calls++;
    tc->f64_flops += 2.0 * (double)gdim(gm) * (double)gdim(gn) * (double)gdim(gk) * (double)gdim(gb);
  }
  // order pairs so the faster-moving member (second) has the smallest stride
  auto order = [](std::vector<Ix>& g, int op) {
    if (g.size() == 2 && std::llabs(g[0].s[op]) < std::llabs(g[1].s[op])) std::swap(g[0], g[1]);
    while (g.size() < 2) g.insert(g.begin(), Ix{1, {0, 0, 0}});
  };
  order(gm, 0);
  order(gn, 1);
  order(gk, 0);
  if (gb.empty()) gb.push_back(Ix{1, {0, 0, 0}});
  CtrDesc d;
  d.M = gm[0].dim * gm[1].dim; d.M2 = gm[1].dim;
  d.N = gn[0].dim * gn[1].dim; d.N2 = gn[1].dim;
  d.K = gk[0].dim * gk[1].dim; d.K2 = gk[1].dim;
  d.batch = gb[0].dim;
  d.a_m1 = gm[0].s[0]; d.a_m2 = gm[1].s[0]; d.a_k1 = gk[0].s[0]; d.a_k2 = gk[1].s[0]; d.a_b = gb[0].s[0];
  d.b_k1 = gk[0].s[1]; d.b_k2 = gk[1].s[1]; d.b_n1 = gn[0].s[1]; d.b_n2 = gn[1].s[1]; d.b_b = gb[0].s[1];
  d.c_m1 = gm[0].s[2]; d.c_m2 = gm[1].s[2]; d.c_n1 = gn[0].s[2]; d.c_n2 = gn[1].s[2]; d.c_b = gb[0].s[2];
  d.alpha = alpha;
  d.beta = beta;
  contract_f64_launch(A.p, B.p, C.p, d, s);
}

void einsum1(double alpha, const char* spec, const TView& A, double beta, const TView& C, cudaStream_t s) {
  std::vector<std::string> ins;
  std::string out;
  parse(spec, ins, out);
  if (ins.size() != 1 || (int)ins[0].size() != A.rank || (int)out.size() != C.rank || A.rank != C.rank)
    fail(FCC_ERR_BAD_ARG, std::string("einsum1 spec mismatch: ") + spec);
  TView src;
  src.p = A.p;
  src.rank = 4;
  TView dst = C;
  for (int k = C.rank; k < 4; ++k) { dst.dim[k] = 1; dst.str[k] = 0; }
  for (int k = 0; k < 4; ++k) { src.dim[k] = 1; src.str[k] = 0; }
  for (int k = 0; k < C.rank; ++k) {
    auto p = ins[0].find(out[k]);
    if (p == std::string::npos) fail(FCC_ERR_BAD_ARG, std::string("einsum1 index missing: ") + spec);
    if (A.dim[p] != C.dim[k]) fail(FCC_ERR_BAD_ARG, std::string("einsum1 extent mismatch: ") + spec);
    src.dim[k] = A.dim[p];
    src.str[k] = A.str[p];
  }
  tensor_axpby_launch(src, dst, alpha, beta, s);
}

}  // namespace fcc

// ===================================================== allocation-free GEMM
// fcc_gemm_f64_noalloc: the split-K FP64 (DMMA) contraction for callers that
// must not allocate device memory -- code that runs while a CUDA graph is
// being captured, inside a host framework that owns every device allocation
// through its own pool, or on a latency-critical path where cudaMalloc's
// implicit synchronisation is not acceptable.  Such callers pass their own
// device inputs and output; the partial sums of the K slices live in the
// fixed file-scope array below instead of a cudaMalloc'd buffer.
//
// The array holds FCC_NOALLOC_SCRATCH doubles (16 MiB) and stays resident on
// every GPU that loads this library until the process exits.  Every call
// shares it and it keeps the last call's contents: each call writes every
// partial it later reads, so nothing needs clearing, but calls whose work
// overlaps on the GPU (different streams, or host threads without ordering)
// race on it and must be serialised by the caller.
namespace {

constexpr int64_t FCC_NOALLOC_SCRATCH = int64_t(1) << 21;
__device__ __align__(256) double g_noalloc_scratch[FCC_NOALLOC_SCRATCH];

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (a host-side reference to the symbol is not a device address).
double* noalloc_scratch_ptr(int& status) {
  static std::mutex mu;
  static double* ptr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { status = FCC_ERR_NO_DEVICE; return nullptr; }
  std::lock_guard<std::mutex> lock(mu);
  if (!ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) { status = FCC_ERR_CUDA; return nullptr; }
    ptr[dev] = static_cast<double*>(p);
  }
  status = FCC_OK;
  return ptr[dev];
}

}  // namespace

extern "C" int fcc_gemm_f64_noalloc(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* stream) {
  using namespace fcc;
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C || lda < K || ldb < N || ldc < N) return FCC_ERR_BAD_ARG;
  if (M * N > FCC_NOALLOC_SCRATCH / 2) return FCC_ERR_BAD_ARG;   // at least two K slices must fit
  int st = FCC_OK;
  double* scratch = noalloc_scratch_ptr(st);
  if (!scratch) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CtrDesc d;
  d.M = M; d.M2 = 1; d.N = N; d.N2 = N; d.K = K; d.K2 = K; d.batch = 1;
  d.a_m1 = lda; d.a_m2 = 0; d.a_k1 = 0; d.a_k2 = 1; d.a_b = 0;
  d.b_k1 = 0; d.b_k2 = ldb; d.b_n1 = 0; d.b_n2 = 1; d.b_b = 0;
  d.c_m1 = ldc; d.c_m2 = 0; d.c_n1 = 0; d.c_n2 = 1; d.c_b = 0;
  d.alpha = alpha;
  d.beta = beta;
  const int64_t gm = (M + BM - 1) / BM, gn = (N + BN - 1) / BN;
  if (gn > 65535) return FCC_ERR_BAD_ARG;
  int64_t splits = std::min<int64_t>(std::max<int64_t>(2, (2 * 152 + gm * gn - 1) / (gm * gn)), (K + BK - 1) / BK);
  splits = std::max<int64_t>(1, std::min<int64_t>(splits, FCC_NOALLOC_SCRATCH / (M * N)));
  const int64_t chunk = ((K + splits - 1) / splits + BK - 1) / BK * BK;
  splits = (K + chunk - 1) / chunk;
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)splits);
  contract_f64_kernel<<<grid, NT, 0, s>>>(A, B, C, d, 0, 1, chunk, scratch);
  if (cudaGetLastError() != cudaSuccess) return FCC_ERR_CUDA;
  note_launch();
  const int64_t MN = M * N;
  splitk_reduce_kernel<<<(unsigned)std::min<int64_t>((MN + 255) / 256, 152 * 8), 256, 0, s>>>(scratch, (int)splits, C, d);
  if (cudaGetLastError() != cudaSuccess) return FCC_ERR_CUDA;
  note_launch();
  return FCC_OK;
}
