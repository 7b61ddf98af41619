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

// Offsets of a 3-level index x = (x1*D2 + x2)*D3 + x3.
__device__ __forceinline__ int64_t off3(int64_t x, int64_t D2, int64_t D3, int64_t s1, int64_t s2, int64_t s3) {
  const int64_t x3 = x % D3, r = x / D3;
  const int64_t x2 = r % D2, x1 = r / D2;
  return x1 * s1 + x2 * s2 + x3 * s3;
}

// The k loop of one 64 x 64 output tile: stage A (BM x BK) and B (BK x BN)
// into shared memory, then 4 k-steps of m8n8k4 per 16-deep slab.  EDGE tiles
// (the last row or column tile of a ragged extent) skip the MMAs of 8-wide
// blocks that lie wholly outside the output, so a v = 152 extent (tiles of
// 64 + 64 + 24) issues no DMMA work for the 40 missing columns.
template <bool EDGE>
__device__ __forceinline__ void f64_mainloop(const double* __restrict__ A, const double* __restrict__ B,
                                             const CtrDesc& d, int a_mfast, int b_nfast, int64_t kbeg,
                                             int64_t kend, double (&As)[BK][LDS], double (&Bs)[BK][LDS],
                                             const int64_t* rowA, const int64_t* colB, const int8_t* rowOK,
                                             const int8_t* colOK, int64_t m0, int64_t n0,
                                             double (&acc)[4][4][2]) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  // row (column) blocks of 8 of this warp that lie inside the output
  int ni = 4, nj = 4;
  if (EDGE) {
    ni = (int)max((int64_t)0, min((int64_t)4, (d.M - m0 - wm + 7) / 8));
    nj = (int)max((int64_t)0, min((int64_t)4, (d.N - n0 - wn + 7) / 8));
  }
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
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
        for (int j = 0; j < 4; ++j)
          if (!EDGE || (i < ni && j < nj)) dmma884(acc[i][j][0], acc[i][j][1], af[i], bf[j]);   // warp-uniform
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(NT, 5) contract_f64_kernel(const double* __restrict__ A,
                                                          const double* __restrict__ B,
                                                          double* __restrict__ C, CtrDesc d,
                                                          int a_mfast, int b_nfast, int64_t k_chunk,
                                                          double* __restrict__ partial) {
  __shared__ double As[BK][LDS];
  __shared__ double Bs[BK][LDS];
  __shared__ int64_t rowA[BM], colB[BN], rowC[BM], colC[BN];
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
    const int64_t m = m0 + tid;
    const bool ok = m < d.M;
    rowA[tid] = ok ? off3(m, d.M2, d.M3, d.a_m1, d.a_m2, d.a_m3) : 0;
    rowC[tid] = ok ? off3(m, d.M2, d.M3, d.c_m1, d.c_m2, d.c_m3) : 0;
    rowOK[tid] = ok;
  } else {
    const int t = tid - BM;
    const int64_t n = n0 + t;
    const bool ok = n < d.N;
    colB[t] = ok ? off3(n, d.N2, d.N3, d.b_n1, d.b_n2, d.b_n3) : 0;
    colC[t] = ok ? off3(n, d.N2, d.N3, d.c_n1, d.c_n2, d.c_n3) : 0;
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

  if (m0 + BM <= d.M && n0 + BN <= d.N)
    f64_mainloop<false>(A, B, d, a_mfast, b_nfast, kbeg, kend, As, Bs, rowA, colB, rowOK, colOK, m0, n0, acc);
  else
    f64_mainloop<true>(A, B, d, a_mfast, b_nfast, kbeg, kend, As, Bs, rowA, colB, rowOK, colOK, m0, n0, acc);

  // ---- epilogue: C = alpha * acc + beta * C with general output strides
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int ml = wm + 8 * i + (lane >> 2);
    const int64_t m = m0 + ml;
    if (m >= d.M) continue;
    const int64_t crow = rowC[ml];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int nl = wn + 8 * j + 2 * (lane & 3) + h;
        const int64_t n = n0 + nl;
        if (n >= d.N) continue;
        if (partial) {   // split-K: raw partial sums, reduced in a fixed order later
          partial[((int64_t)blockIdx.z * d.M + m) * d.N + n] = acc[i][j][h];
          continue;
        }
        double* dst = C + crow + colC[nl];
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
    double* dst = C + off3(m, d.M2, d.M3, d.c_m1, d.c_m2, d.c_m3) + off3(n, d.N2, d.N3, d.c_n1, d.c_n2, d.c_n3);
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
    const double* a = A + off3(m, d.M2, d.M3, d.a_m1, d.a_m2, d.a_m3);
    double s = 0.0;
    for (int64_t k = lane; k < d.K; k += 32) {
      const int64_t k1 = k / d.K2, k2 = k - k1 * d.K2;
      s += a[k1 * d.a_k1 + k2 * d.a_k2] * B[k1 * d.b_k1 + k2 * d.b_k2];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      double* dst = C + off3(m, d.M2, d.M3, d.c_m1, d.c_m2, d.c_m3);
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
  // stage along M (N) when the fastest-moving M (N) index has unit stride
  const int a_fast = (d.M3 > 1 ? d.a_m3 : d.a_m2) == 1 ? 1 : 0;
  const int b_fast = (d.N3 > 1 ? d.b_n3 : d.b_n2) == 1 ? 1 : 0;
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
    DBuf<double> local;
    DBuf<double>* ws = f64_workspace();
    if (!ws) ws = &local;
    DBuf<double>& scratch = *ws;
    const int64_t need = splits * d.M * d.N;
    if ((int64_t)scratch.n < need) scratch.alloc(need);
    dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)splits);
    contract_f64_kernel<<<grid, NT, 0, s>>>(A, B, C, d, a_fast, b_fast, chunk, scratch.p);
    FCC_CHECK_LAUNCH();
    const int64_t MN = d.M * d.N;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>((MN + 255) / 256, 152 * 8), 256, 0, s>>>(scratch.p, (int)splits,
                                                                                                 C, d);
    FCC_CHECK_LAUNCH();
    prof_end(s, pidx, PROF_F64, pflops);
    return;
  }
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)d.batch);
  contract_f64_kernel<<<grid, NT, 0, s>>>(A, B, C, d, a_fast, b_fast, d.K, nullptr);
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

bool same_spec(const PackSpec& a, const PackSpec& b) {
  return a.R == b.R && a.K == b.K && a.Kp == b.Kp && a.rd2 == b.rd2 && a.rd3 == b.rd3 && a.rs1 == b.rs1 &&
         a.rs2 == b.rs2 && a.rs3 == b.rs3 && a.kd2 == b.kd2 && a.kd3 == b.kd3 && a.ks1 == b.ks1 && a.ks2 == b.ks2 &&
         a.ks3 == b.ks3 && a.P == b.P && a.code == b.code && a.scale == b.scale;
}

// The kept pack of operand A for (src, ps, S) when src is one of the
// engine's kept sources (nullptr otherwise); `fresh` is set when it has to be
// packed now.
TcEngine::KeptPack* kept_a(TcEngine* tc, const double* src, const PackSpec& ps, int S, bool& fresh) {
  fresh = false;
  for (int i = 0; i < 2; ++i) {
    if (!src || tc->keep_src[i] != src) continue;
    TcEngine::KeptPack& k = tc->kept[i];
    if (k.valid && k.S == S && same_spec(k.ps, ps)) return &k;
    k.ps = ps;
    k.S = S;
    k.valid = true;
    fresh = true;
    return &k;
  }
  return nullptr;
}

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
    bool fresh;
    TcEngine::KeptPack* ka = kept_a(tc, A.p, pa, S, fresh);
    __nv_bfloat16* pA = tc->bufA.p;
    int* eA = tc->exA.p;
    if (ka) {
      if (fresh) {
        if ((int64_t)ka->buf.n < M * W) ka->buf.alloc(M * W);
        if ((int64_t)ka->ex.n < M) ka->ex.alloc(M);
        pack_oz(A.p, pa, S, ka->buf.p, ka->ex.p, s);
      }
      pA = ka->buf.p;
      eA = ka->ex.p;
    } else {
      pack_oz(A.p, pa, S, pA, eA, s);
    }
    pack_oz(B.p, pb, S, tc->bufB.p, tc->exB.p, s);
    EpiMap ep;
    ep.M = M; ep.N = N;
    ep.md2 = gm[1].dim; ep.md3 = gm[2].dim; ep.ms1 = gm[0].s[2]; ep.ms2 = gm[1].s[2]; ep.ms3 = gm[2].s[2];
    ep.nd2 = gn[1].dim; ep.nd3 = gn[2].dim; ep.ns1 = gn[0].s[2]; ep.ns2 = gn[1].s[2]; ep.ns3 = gn[2].s[2];
    ep.alpha = alpha; ep.beta = beta; ep.C = C.p; ep.mode = EPI_F64;
    const double npairs = (double)(G - 1) * (double)G / 2.0;
    ep.work = 2.0 * (double)M * (double)N * (double)K * npairs;
    gemm_oz(pA, M, eA, tc->bufB.p, N, tc->exB.p, Kpad, G, ep, tc->err, s);
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
  bool fresh;
  TcEngine::KeptPack* ka = kept_a(tc, A.p, pa, 0, fresh);
  __nv_bfloat16* pA = tc->bufA.p;
  if (ka) {
    if (fresh) {
      if ((int64_t)ka->buf.n < M * Kp) ka->buf.alloc(M * Kp);
      pack_split(A.p, pa, ka->buf.p, s);
    }
    pA = ka->buf.p;
  } else {
    pack_split(A.p, pa, pA, s);
  }
  pack_split(B.p, pb, tc->bufB.p, s);
  EpiMap ep;
  ep.M = M; ep.N = N;
  ep.md2 = gm[1].dim; ep.md3 = gm[2].dim; ep.ms1 = gm[0].s[2]; ep.ms2 = gm[1].s[2]; ep.ms3 = gm[2].s[2];
  ep.nd2 = gn[1].dim; ep.nd3 = gn[2].dim; ep.ns1 = gn[0].s[2]; ep.ns2 = gn[1].s[2]; ep.ns3 = gn[2].s[2];
  ep.alpha = alpha; ep.beta = beta; ep.C = C.p; ep.mode = EPI_F64;
  ep.work = 2.0 * (double)M * (double)N * (double)K * sc.P;
  ep.no_loads = tc->no_loads_once;
  tc->no_loads_once = 0;
  gemm_bf16x3(pA, M, 0, tc->bufB.p, N, 0, Kp, ep, tc->err, s);
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

DBuf<double>*& f64_workspace() {
  thread_local DBuf<double>* w = nullptr;
  return w;
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
  fuse(gm, 3, spec);
  fuse(gn, 3, spec);
  fuse(gk, 2, spec);
  if (tc) {
    tc->f64_calls++;
    tc->f64_flops += 2.0 * (double)gdim(gm) * (double)gdim(gn) * (double)gdim(gk) * (double)gdim(gb);
  }
  // order each group slowest first (the last member has the smallest stride
  // in the operand read along it), padded at the front with unit indices
  auto order = [](std::vector<Ix>& g, int op, size_t levels) {
    std::stable_sort(g.begin(), g.end(), [op](const Ix& a, const Ix& b) { return std::llabs(a.s[op]) > std::llabs(b.s[op]); });
    while (g.size() < levels) g.insert(g.begin(), Ix{1, {0, 0, 0}});
  };
  order(gm, 0, 3);
  order(gn, 1, 3);
  order(gk, 0, 2);
  if (gb.empty()) gb.push_back(Ix{1, {0, 0, 0}});
  CtrDesc d;
  d.M = gdim(gm); d.M2 = gm[1].dim; d.M3 = gm[2].dim;
  d.N = gdim(gn); d.N2 = gn[1].dim; d.N3 = gn[2].dim;
  d.K = gk[0].dim * gk[1].dim; d.K2 = gk[1].dim;
  d.batch = gb[0].dim;
  d.a_m1 = gm[0].s[0]; d.a_m2 = gm[1].s[0]; d.a_m3 = gm[2].s[0];
  d.a_k1 = gk[0].s[0]; d.a_k2 = gk[1].s[0]; d.a_b = gb[0].s[0];
  d.b_k1 = gk[0].s[1]; d.b_k2 = gk[1].s[1];
  d.b_n1 = gn[0].s[1]; d.b_n2 = gn[1].s[1]; d.b_n3 = gn[2].s[1]; d.b_b = gb[0].s[1];
  d.c_m1 = gm[0].s[2]; d.c_m2 = gm[1].s[2]; d.c_m3 = gm[2].s[2];
  d.c_n1 = gn[0].s[2]; d.c_n2 = gn[1].s[2]; d.c_n3 = gn[2].s[2]; d.c_b = gb[0].s[2];
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
// cannot allocate device memory: a host framework that owns every device
// allocation through its own pool and forbids others, or a latency-critical
// path where cudaMalloc's implicit device synchronisation is not acceptable.
// Such callers pass their own device inputs and output; the partial sums of
// the K slices live in the fixed file-scope array below instead of a
// cudaMalloc'd buffer.
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
  // M and N are bounded one at a time first, so M * N cannot overflow
  if (M > FCC_NOALLOC_SCRATCH / 2 || N > FCC_NOALLOC_SCRATCH / 2) return FCC_ERR_BAD_ARG;
  if (M * N > FCC_NOALLOC_SCRATCH / 2) return FCC_ERR_BAD_ARG;   // at least two K slices must fit
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the scratch address is the current device's: the stream must belong to it
  if (s) {
    int cur = -1, sdev = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(s, &sdev) != cudaSuccess) return FCC_ERR_CUDA;
    if (cur != sdev) return FCC_ERR_BAD_ARG;
  }
  int st = FCC_OK;
  double* scratch = noalloc_scratch_ptr(st);
  if (!scratch) return st;
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
