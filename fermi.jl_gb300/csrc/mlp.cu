// Learned T2 initialiser: a 16 -> 128 -> 128 -> 1 GELU MLP that predicts, for
// every doubles amplitude, the CCSD correction to its MP2 value from
// per-element features (orbital energies, MP2 amplitude and integrals, DF pair
// norms).  It only seeds the iteration (RCCSDa.jl:92 accepts any guess); the
// converged energy is unaffected.
//
// Weights are BF16 for the forward/backward products with FP32 master copies
// updated by Adam.  Everything here is hand-written: the feature kernel, a
// BF16 tensor-core GEMM (mma.sync m16n8k16, FP32 accumulation, deterministic
// split-K) for the five layer products, an FP32 SIMT GEMM for the one-row
// output-layer gradient, bias+GELU forward and backward,
// the loss, bias-gradient reductions, Adam, and the inference kernel that
// writes the guess into a context.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <new>

#include "fcc_ctx.cuh"

namespace fcc {

namespace {

constexpr int NF = 16, H = 128;
// parameter vector: W1[H][NF] b1[H] W2[H][H] b2[H] w3[H] b3 mu[NF] sd[NF]
constexpr int64_t OFF_W1 = 0, OFF_B1 = OFF_W1 + H * NF, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
                  OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H, OFF_MU = OFF_B3 + 1, OFF_SD = OFF_MU + NF,
                  NPARAM = OFF_SD + NF;
constexpr int64_t NTRAIN = OFF_MU;   // trained parameters (mu, sd are fixed statistics)
constexpr double TARGET_FLOOR = 1e-4; // target = (t_cc - t_mp2) / (|t_mp2| + floor)

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

template <class T>
__device__ __forceinline__ float ld(const T* p, int64_t i);
template <>
__device__ __forceinline__ float ld<float>(const float* p, int64_t i) { return p[i]; }
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) { return __bfloat162float(p[i]); }

// C[m][n] = alpha * sum_k A(m,k) B(k,n) + beta * C[m][n]; A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn], C row-major with ldc.  64 x 64 tile, 16-deep K.
template <class TA, class TB>
__global__ void __launch_bounds__(256) sgemm_kernel(int M, int N, int K, float alpha, const TA* __restrict__ A,
                                                    int64_t sam, int64_t sak, const TB* __restrict__ B, int64_t sbk,
                                                    int64_t sbn, float beta, float* __restrict__ C, int64_t ldc) {
  __shared__ float As[16][64 + 1], Bs[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      int mm = e / 16, kk = e % 16;
      int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? ld(A, (int64_t)m * sam + (int64_t)k * sak) : 0.0f;
      int nn = e % 64, kb = e / 64;
      int n = n0 + nn, k2 = k0 + kb;
      Bs[kb][nn] = (n < N && k2 < K) ? ld(B, (int64_t)k2 * sbk + (int64_t)n * sbn) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int m = m0 + ty * 4 + r, n = n0 + tx * 4 + c;
      if (m < M && n < N) {
        float v = alpha * acc[r][c];
        if (beta != 0.0f) v += beta * C[(int64_t)m * ldc + n];
        C[(int64_t)m * ldc + n] = v;
      }
    }
}

template <class TA, class TB>
void sgemm(int M, int N, int K, float alpha, const TA* A, int64_t sam, int64_t sak, const TB* B, int64_t sbk,
           int64_t sbn, float beta, float* C, int64_t ldc, cudaStream_t s) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  sgemm_kernel<TA, TB><<<grid, 256, 0, s>>>(M, N, K, alpha, A, sam, sak, B, sbk, sbn, beta, C, ldc);
  FCC_CHECK_LAUNCH();
}

// ---- tensor-core GEMM of the network's products: operands rounded to BF16
// (nearest, ties to even) when staged, mma.sync m16n8k16 with FP32
// accumulation.  64 x 64 output tile, 32-deep K slab, four warps of 32 x 32.
// With `splits` > 1 the K range is cut into slices whose FP32 partial tiles
// are summed in slice order by hgemm_reduce_kernel (the gradient products
// reduce over the whole batch, K = 65536, into a 128 x 128 output).
constexpr int HT = 64, HK = 32, HLD = HK + 8;   // smem rows padded by 16 bytes

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <class T>
__device__ __forceinline__ __nv_bfloat16 to_bf(const T* p, int64_t i);
template <>
__device__ __forceinline__ __nv_bfloat16 to_bf<float>(const float* p, int64_t i) { return __float2bfloat16_rn(p[i]); }
template <>
__device__ __forceinline__ __nv_bfloat16 to_bf<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) { return p[i]; }

// C[m][n] = alpha * sum_k A(m,k) B(k,n) + beta * C (part == nullptr), or the
// raw partial of K slice blockIdx.z into part[z][m][n].
template <class TA, class TB>
__global__ void __launch_bounds__(128) hgemm_kernel(int M, int N, int K, int kchunk, float alpha,
                                                    const TA* __restrict__ A, int64_t sam, int64_t sak,
                                                    const TB* __restrict__ B, int64_t sbk, int64_t sbn, float beta,
                                                    float* __restrict__ C, int64_t ldc, float* __restrict__ part) {
  __shared__ __align__(16) __nv_bfloat16 As[HT][HLD];   // [m][k]
  __shared__ __align__(16) __nv_bfloat16 Bs[HT][HLD];   // [n][k]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * HT, n0 = blockIdx.x * HT;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, t4 = lane & 3;
  float acc[2][4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += HK) {
    // stage with the stride-1 index of each operand along the threads
    for (int e = tid; e < HT * HK; e += 128) {
      const int mm = sak == 1 ? e / HK : e % HT, kk = sak == 1 ? e % HK : e / HT;
      const int m = m0 + mm, k = k0 + kk;
      As[mm][kk] = (m < M && k < ke) ? to_bf(A, (int64_t)m * sam + (int64_t)k * sak) : __float2bfloat16_rn(0.0f);
      const int nn = sbk == 1 ? e / HK : e % HT, k2 = sbk == 1 ? e % HK : e / HT;
      const int n = n0 + nn, kk2 = k0 + k2;
      Bs[nn][k2] = (n < N && kk2 < ke) ? to_bf(B, (int64_t)kk2 * sbk + (int64_t)n * sbn) : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < HK; ks += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + 16 * i + g;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t4]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t4]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 8 + 2 * t4]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 8 + 2 * t4]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + 8 * j + g;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t4]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 8 + 2 * t4]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16_16816(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int m = m0 + wm + 16 * i + g + (h >> 1) * 8, n = n0 + wn + 8 * j + 2 * t4 + (h & 1);
        if (m >= M || n >= N) continue;
        if (part) {
          part[((int64_t)blockIdx.z * M + m) * N + n] = acc[i][j][h];
        } else {
          float v = alpha * acc[i][j][h];
          if (beta != 0.0f) v += beta * C[(int64_t)m * ldc + n];
          C[(int64_t)m * ldc + n] = v;
        }
      }
}

__global__ void hgemm_reduce_kernel(const float* __restrict__ part, int splits, int M, int N, float alpha,
                                    float beta, float* __restrict__ C, int64_t ldc) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)M * N; t += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += part[(int64_t)z * M * N + t];
    const int64_t m = t / N, n = t - m * N;
    float v = alpha * s;
    if (beta != 0.0f) v += beta * C[m * ldc + n];
    C[m * ldc + n] = v;
  }
}

// Tensor-core GEMM with the sgemm argument convention; splits K when the
// output has fewer tiles than the GPU has SMs (partials in `work`, grown as
// needed).
template <class TA, class TB>
void hgemm(int M, int N, int K, float alpha, const TA* A, int64_t sam, int64_t sak, const TB* B, int64_t sbk,
           int64_t sbn, float beta, float* C, int64_t ldc, DBuf<float>& work, cudaStream_t s) {
  const int tiles = ((N + HT - 1) / HT) * ((M + HT - 1) / HT);
  int splits = 1;
  if (tiles < 152 && K >= 8 * HK) splits = std::min((2 * 152 + tiles - 1) / tiles, K / (4 * HK));
  splits = std::max(1, std::min(splits, 256));
  const int kchunk = ((K + splits - 1) / splits + HK - 1) / HK * HK;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((N + HT - 1) / HT, (M + HT - 1) / HT, splits);
  if (splits == 1) {
    hgemm_kernel<TA, TB><<<grid, 128, 0, s>>>(M, N, K, kchunk, alpha, A, sam, sak, B, sbk, sbn, beta, C, ldc, nullptr);
    FCC_CHECK_LAUNCH();
    return;
  }
  const int64_t need = (int64_t)splits * M * N;
  if ((int64_t)work.n < need) work.alloc(need);
  hgemm_kernel<TA, TB><<<grid, 128, 0, s>>>(M, N, K, kchunk, alpha, A, sam, sak, B, sbk, sbn, beta, C, ldc, work.p);
  FCC_CHECK_LAUNCH();
  hgemm_reduce_kernel<<<(unsigned)std::min<int64_t>(((int64_t)M * N + 255) / 256, 152 * 4), 256, 0, s>>>(
      work.p, splits, M, N, alpha, beta, C, ldc);
  FCC_CHECK_LAUNCH();
}

// Z[b][h] += bias[h]; Hact = GELU(Z)
__global__ void bias_gelu_kernel(float* Z, float* Hact, const float* bias, int64_t B, int Hn) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < B * Hn; t += (int64_t)gridDim.x * blockDim.x) {
    float z = Z[t] + bias[t % Hn];
    Z[t] = z;
    Hact[t] = gelu(z);
  }
}

// dZ = dH * GELU'(Z)
__global__ void gelu_back_kernel(const float* Z, float* dH, int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dH[t] *= gelu_grad(Z[t]);
}

// y[b] = sum_h H2[b][h] w3[h] + b3; loss partials; dy = 2 (y - target) / B
__global__ void out_loss_kernel(const float* H2, const float* w3, const float* b3, const float* target, int64_t B,
                                float* y, float* dy, double* loss_part) {
  double l = 0.0;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < B; b += (int64_t)gridDim.x * blockDim.x) {
    float s = b3[0];
    for (int h = 0; h < H; ++h) s += H2[b * H + h] * w3[h];
    y[b] = s;
    if (target) {
      float d = s - target[b];
      l += (double)d * d;
      dy[b] = 2.0f * d / (float)B;
    }
  }
  if (loss_part) {
    __shared__ double sm[256];
    sm[threadIdx.x] = l;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = sm[0];
  }
}

// g[h] = sum_b X[b][h] (bias gradients), one block per h, fixed order.
__global__ void colsum_kernel(const float* X, int64_t B, int Hn, float* g) {
  const int h = blockIdx.x;
  double s = 0.0;
  for (int64_t b = threadIdx.x; b < B; b += blockDim.x) s += X[b * Hn + h];
  __shared__ double sm[256];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) g[h] = (float)sm[0];
}

// dH2[b][h] = dy[b] * w3[h]
__global__ void outer_kernel(const float* dy, const float* w3, int64_t B, float* dH2) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < B * H; t += (int64_t)gridDim.x * blockDim.x)
    dH2[t] = dy[t / H] * w3[t % H];
}

// Adam (Kingma & Ba 2015) on the FP32 masters, then the BF16 working copy.
__global__ void adam_kernel(float* p, const float* g, float* m1, float* m2, __nv_bfloat16* pb, int64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    float gi = g[t];
    float a = b1 * m1[t] + (1.0f - b1) * gi;
    float v = b2 * m2[t] + (1.0f - b2) * gi * gi;
    m1[t] = a;
    m2[t] = v;
    float upd = lr * (a / c1) / (sqrtf(v / c2) + eps);
    p[t] -= upd;
    pb[t] = __float2bfloat16_rn(p[t]);
  }
}

__global__ void to_bf16_kernel(const float* p, __nv_bfloat16* q, int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    q[t] = __float2bfloat16_rn(p[t]);
}

// Features of element e = ((i*o + j)*v + a)*v + b (normalised with mu, sd):
//  e_i e_j e_a e_b, D, t_mp2 = (ia|jb)/D, (ib|ja)/D, (ia|jb), (ib|ja),
//  |B_ia| |B_jb| |B_ib| |B_ja| (DF pair norms), d_ij, d_ab, 1/D.
struct FeatSrc {
  const double* eps;   // o + v
  const double* ovov;  // (ia|jb) [o][v][o][v]
  const double* pn;    // |B_ia| [o][v]
  int o, v;
};

__device__ void features(const FeatSrc& f, int64_t e, float* x, double& tmp2) {
  const int v = f.v, o = f.o;
  const int b = (int)(e % v);
  int64_t r = e / v;
  const int a = (int)(r % v);
  r /= v;
  const int j = (int)(r % o), i = (int)(r / o);
  const double ei = f.eps[i], ej = f.eps[j], ea = f.eps[o + a], eb = f.eps[o + b];
  const double D = ei + ej - ea - eb;
  const double iajb = f.ovov[(((int64_t)i * v + a) * o + j) * v + b];
  const double ibja = f.ovov[(((int64_t)i * v + b) * o + j) * v + a];
  tmp2 = iajb / D;
  x[0] = (float)ei; x[1] = (float)ej; x[2] = (float)ea; x[3] = (float)eb; x[4] = (float)D;
  x[5] = (float)(iajb / D); x[6] = (float)(ibja / D); x[7] = (float)iajb; x[8] = (float)ibja;
  x[9] = (float)f.pn[(int64_t)i * v + a]; x[10] = (float)f.pn[(int64_t)j * v + b];
  x[11] = (float)f.pn[(int64_t)i * v + b]; x[12] = (float)f.pn[(int64_t)j * v + a];
  x[13] = (float)(i == j); x[14] = (float)(a == b); x[15] = (float)(1.0 / D);
}

// Append samples (every stride-th element, offset by `phase`) with their raw
// features and targets.
__global__ void collect_kernel(FeatSrc f, const double* t2, int64_t total, int64_t stride, int64_t phase, float* X,
                               float* Y, int64_t base) {
  const int64_t ns = (total - phase + stride - 1) / stride;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = phase + s * stride;
    float x[NF];
    double tmp2;
    features(f, e, x, tmp2);
    for (int q = 0; q < NF; ++q) X[(base + s) * NF + q] = x[q];
    Y[base + s] = (float)((t2[e] - tmp2) / (fabs(tmp2) + TARGET_FLOOR));
  }
}

// Thresholded collection in two passes with a fixed sample order: candidate
// samples are the elements phase + s * stride; a candidate is kept when
// |t_MP2| >= thresh.  Pass 1 counts the kept candidates of each block's
// contiguous chunk; pass 2 (after an exclusive scan of the counts on the
// host) writes them at base + offset[block] + their rank inside the chunk.
constexpr int CT = 256;
__device__ __forceinline__ bool keep_elem(const FeatSrc& f, int64_t e, double thresh) {
  const int v = f.v, o = f.o;
  const int b = (int)(e % v);
  int64_t r = e / v;
  const int a = (int)(r % v);
  r /= v;
  const int j = (int)(r % o), i = (int)(r / o);
  const double D = f.eps[i] + f.eps[j] - f.eps[o + a] - f.eps[o + b];
  return fabs(f.ovov[(((int64_t)i * v + a) * o + j) * v + b] / D) >= thresh;
}

__global__ void __launch_bounds__(CT) collect_count_kernel(FeatSrc f, int64_t total, int64_t stride, int64_t phase,
                                                           int64_t chunk, double thresh, int* counts) {
  const int64_t ns = (total - phase + stride - 1) / stride;
  const int64_t s0 = (int64_t)blockIdx.x * chunk, s1 = min(ns, s0 + chunk);
  int c = 0;
  for (int64_t sidx = s0 + threadIdx.x; sidx < s1; sidx += CT) c += keep_elem(f, phase + sidx * stride, thresh);
  __shared__ int sm[CT / 32];
  for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < CT / 32; ++w) t += sm[w];
    counts[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(CT) collect_write_kernel(FeatSrc f, const double* t2, int64_t total, int64_t stride,
                                                           int64_t phase, int64_t chunk, double thresh,
                                                           const int64_t* offsets, float* X, float* Y, int64_t base) {
  const int64_t ns = (total - phase + stride - 1) / stride;
  const int64_t s0 = (int64_t)blockIdx.x * chunk, s1 = min(ns, s0 + chunk);
  __shared__ int wsum[CT / 32];
  __shared__ int64_t run;
  if (threadIdx.x == 0) run = base + offsets[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t c0 = s0; c0 < s1; c0 += CT) {
    const int64_t sidx = c0 + threadIdx.x;
    const int64_t e = phase + sidx * stride;
    const bool k = sidx < s1 && keep_elem(f, e, thresh);
    const unsigned bal = __ballot_sync(0xffffffffu, k);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    int before = 0, all = 0;
    for (int q = 0; q < CT / 32; ++q) { if (q < w) before += wsum[q]; all += wsum[q]; }
    const int64_t out = run + before + __popc(bal & ((1u << lane) - 1u));
    if (k) {
      float x[NF];
      double tmp2;
      features(f, e, x, tmp2);
      for (int q = 0; q < NF; ++q) X[out * NF + q] = x[q];
      Y[out] = (float)((t2[e] - tmp2) / (fabs(tmp2) + TARGET_FLOOR));
    }
    __syncthreads();
    if (threadIdx.x == 0) run += all;
    __syncthreads();
  }
}

// normalise raw features: (x - mu) / sd
__global__ void normalise_kernel(const float* Xraw, int64_t n, const float* mu, const float* sd, float* Xn) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * NF; t += (int64_t)gridDim.x * blockDim.x)
    Xn[t] = (Xraw[t] - mu[t % NF]) / sd[t % NF];
}

// gather a batch: rows idx[b] of the sample set
__global__ void gather_kernel(const float* X, const float* Y, int64_t B, uint64_t seed, int64_t nsamp, float* Xb,
                              float* Yb) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < B; b += (int64_t)gridDim.x * blockDim.x) {
    // SplitMix64 of (seed, b): a reproducible pseudo-random row
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(b + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int64_t r = (int64_t)(z % (uint64_t)nsamp);
    for (int q = 0; q < NF; ++q) Xb[b * NF + q] = X[r * NF + q];
    Yb[b] = Y[r];
  }
}

// t_ijab = t_jiba holds for the exact amplitudes; the network sees the two
// elements through different feature vectors, so average them.
__global__ void pair_symmetrise_kernel(double* t2, int o, int v) {
  const int64_t total = (int64_t)o * o * v * v;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % v);
    int64_t r = e / v;
    const int a = (int)(r % v);
    r /= v;
    const int j = (int)(r % o), i = (int)(r / o);
    const int64_t e2 = (((int64_t)j * o + i) * v + b) * v + a;
    if (e < e2) {
      const double m = 0.5 * (t2[e] + t2[e2]);
      t2[e] = m;
      t2[e2] = m;
    }
  }
}

// t2 = t_MP2 for every element; the elements with |t_MP2| >= thresh (the
// ones the correction is applied to) are appended to sel (in any order: each
// gets its own prediction, so the result does not depend on the order)
__global__ void mp2_select_kernel(FeatSrc f, int64_t total, double thresh, double* t2, int64_t* sel,
                                  unsigned long long* nsel) {
  __shared__ unsigned int cnt, base;
  for (int64_t e0 = (int64_t)blockIdx.x * blockDim.x; e0 < total; e0 += (int64_t)gridDim.x * blockDim.x) {
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    const int64_t e = e0 + threadIdx.x;
    unsigned int slot = 0;
    bool take = false;
    if (e < total) {
      float x[NF];
      double tmp2;
      features(f, e, x, tmp2);
      t2[e] = tmp2;
      take = fabs(tmp2) >= thresh;
      if (take) slot = atomicAdd(&cnt, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) base = cnt ? (unsigned int)atomicAdd(nsel, (unsigned long long)cnt) : 0u;
    __syncthreads();
    if (take) sel[(int64_t)base + slot] = e;
    __syncthreads();
  }
}

__global__ void infer_features_sel_kernel(FeatSrc f, const int64_t* sel, int64_t n, const float* mu, const float* sd,
                                          float* Xn) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    float x[NF];
    double tmp2;
    features(f, sel[s], x, tmp2);
    for (int q = 0; q < NF; ++q) Xn[s * NF + q] = (x[q] - mu[q]) / sd[q];
  }
}

// t2 += lam * correction for the selected elements
__global__ void infer_write_sel_kernel(const float* y, const int64_t* sel, int64_t n, double lam, double* t2) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = sel[s];
    const double tmp2 = t2[e];
    t2[e] = tmp2 + lam * (double)y[s] * (fabs(tmp2) + TARGET_FLOOR);
  }
}

__global__ void pair_norm_kernel(const double* B, int64_t Q, int64_t n, int o, int v, double* pn) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)o * v; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / v, a = t % v;
    double s = 0.0;
    for (int64_t q = 0; q < Q; ++q) {
      double x = B[(q * n + i) * n + o + a];
      s += x * x;
    }
    pn[t] = sqrt(s);
  }
}

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace

}  // namespace fcc

struct fcc_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  fcc::DBuf<float> p, g, m1, m2;          // FP32 masters, gradients, Adam moments
  fcc::DBuf<__nv_bfloat16> pb;            // BF16 working weights
  fcc::DBuf<float> X, Y;                  // collected raw samples
  int64_t nsamp = 0, cap = 0;
  int64_t adam_t = 0;
  bool stats = false;
  // batch work buffers
  fcc::DBuf<float> Xb, Yb, Z1, H1, Z2, H2, yb, dy, dH, dH1;
  fcc::DBuf<double> lpart;
  fcc::DBuf<float> work;                  // split-K partials of the tensor-core products
  int64_t bcap = 0;
};

namespace fcc {
namespace {

void ensure_batch(fcc_mlp* m, int64_t B) {
  if (B <= m->bcap) return;
  m->Xb.alloc(B * NF); m->Yb.alloc(B); m->Z1.alloc(B * H); m->H1.alloc(B * H); m->Z2.alloc(B * H);
  m->H2.alloc(B * H); m->yb.alloc(B); m->dy.alloc(B); m->dH.alloc(B * H); m->dH1.alloc(B * H);
  m->lpart.alloc(304);
  m->bcap = B;
}

// forward on normalised Xb (B rows); pred into yb; with target: loss, dy and
// the full backward into m->g.
double fwd_bwd(fcc_mlp* m, int64_t B, const float* target, bool backward) {
  cudaStream_t s = m->stream;
  const __nv_bfloat16* W1 = m->pb.p + OFF_W1;
  const __nv_bfloat16* W2 = m->pb.p + OFF_W2;
  const float* b1 = m->p.p + OFF_B1;
  const float* b2 = m->p.p + OFF_B2;
  // layer 1: Z1 = Xb W1^T   (B x H), K = NF; tensor cores, BF16 operands
  hgemm<float, __nv_bfloat16>((int)B, H, NF, 1.0f, m->Xb.p, NF, 1, W1, 1, NF, 0.0f, m->Z1.p, H, m->work, s);
  bias_gelu_kernel<<<grid_of(B * H), 256, 0, s>>>(m->Z1.p, m->H1.p, b1, B, H);
  FCC_CHECK_LAUNCH();
  hgemm<float, __nv_bfloat16>((int)B, H, H, 1.0f, m->H1.p, H, 1, W2, 1, H, 0.0f, m->Z2.p, H, m->work, s);
  bias_gelu_kernel<<<grid_of(B * H), 256, 0, s>>>(m->Z2.p, m->H2.p, b2, B, H);
  FCC_CHECK_LAUNCH();
  // output layer (w3 FP32 master used directly: 128 weights)
  out_loss_kernel<<<304, 256, 0, s>>>(m->H2.p, m->p.p + OFF_W3, m->p.p + OFF_B3, target, B, m->yb.p, m->dy.p,
                                      target ? m->lpart.p : nullptr);
  FCC_CHECK_LAUNCH();
  double loss = 0.0;
  if (target) {
    std::vector<double> lp(304);
    FCC_CUDA(cudaMemcpyAsync(lp.data(), m->lpart.p, sizeof(double) * 304, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    for (double x : lp) loss += x;
    loss /= (double)B;
  }
  if (!backward) return loss;
  float* g = m->g.p;
  // dL/dw3[h] = sum_b dy[b] H2[b][h];  dL/db3 = sum_b dy[b]
  sgemm<float, float>(1, H, (int)B, 1.0f, m->dy.p, 0, 1, m->H2.p, H, 1, 0.0f, g + OFF_W3, H, s);
  colsum_kernel<<<1, 256, 0, s>>>(m->dy.p, B, 1, g + OFF_B3);
  FCC_CHECK_LAUNCH();
  // dH2 = dy w3^T, dZ2 = dH2 * GELU'(Z2)
  outer_kernel<<<grid_of(B * H), 256, 0, s>>>(m->dy.p, m->p.p + OFF_W3, B, m->dH.p);
  FCC_CHECK_LAUNCH();
  gelu_back_kernel<<<grid_of(B * H), 256, 0, s>>>(m->Z2.p, m->dH.p, B * H);
  FCC_CHECK_LAUNCH();
  // dW2 = dZ2^T H1 (H x H, K = B), db2 = colsum(dZ2)
  hgemm<float, float>(H, H, (int)B, 1.0f, m->dH.p, 1, H, m->H1.p, H, 1, 0.0f, g + OFF_W2, H, m->work, s);
  colsum_kernel<<<H, 256, 0, s>>>(m->dH.p, B, H, g + OFF_B2);
  FCC_CHECK_LAUNCH();
  // dH1 = dZ2 W2 (B x H), dZ1 = dH1 * GELU'(Z1)
  hgemm<float, __nv_bfloat16>((int)B, H, H, 1.0f, m->dH.p, H, 1, W2, H, 1, 0.0f, m->dH1.p, H, m->work, s);
  gelu_back_kernel<<<grid_of(B * H), 256, 0, s>>>(m->Z1.p, m->dH1.p, B * H);
  FCC_CHECK_LAUNCH();
  // dW1 = dZ1^T X (H x NF), db1 = colsum(dZ1)
  hgemm<float, float>(H, NF, (int)B, 1.0f, m->dH1.p, 1, H, m->Xb.p, NF, 1, 0.0f, g + OFF_W1, NF, m->work, s);
  colsum_kernel<<<H, 256, 0, s>>>(m->dH1.p, B, H, g + OFF_B1);
  FCC_CHECK_LAUNCH();
  return loss;
}

FeatSrc feat_src(fcc_ctx* c, DBuf<double>& pn) {
  pn.alloc(c->o * c->v);
  pair_norm_kernel<<<grid_of(c->o * c->v), 256, 0, c->stream>>>(c->B.p, c->Q, c->n, (int)c->o, (int)c->v, pn.p);
  FCC_CHECK_LAUNCH();
  FeatSrc f;
  f.eps = c->eps.p; f.ovov = c->ovov.p; f.pn = pn.p; f.o = (int)c->o; f.v = (int)c->v;
  return f;
}

template <class F>
int guard(F&& f) {
  try {
    return f();
  } catch (const Error& e) {
    return e.code;
  } catch (...) {
    return FCC_ERR_CUDA;
  }
}

}  // namespace
}  // namespace fcc

using namespace fcc;

extern "C" {

int64_t fcc_mlp_num_params(void) { return NPARAM; }

int fcc_mlp_create(fcc_mlp** out, int32_t device) {
  if (!out) return FCC_ERR_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return FCC_ERR_NO_DEVICE;
  fcc_mlp* m = new (std::nothrow) fcc_mlp();
  if (!m) return FCC_ERR_OOM;
  m->device = device;
  int rc = guard([&]() {
    FCC_CUDA(cudaSetDevice(device));
    FCC_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    m->p.alloc(NPARAM); m->g.alloc(NPARAM); m->m1.alloc(NPARAM); m->m2.alloc(NPARAM); m->pb.alloc(NPARAM);
    // deterministic initialisation: uniform(-1/sqrt(fan_in), +) weights, zero biases
    std::vector<float> h(NPARAM, 0.0f);
    uint64_t z = 0x1234567ull;
    auto uni = [&]() {
      z += 0x9E3779B97F4A7C15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      x ^= x >> 31;
      return (double)(x >> 11) / 9007199254740992.0 * 2.0 - 1.0;
    };
    for (int64_t t = 0; t < H * NF; ++t) h[OFF_W1 + t] = (float)(uni() / std::sqrt((double)NF));
    for (int64_t t = 0; t < H * H; ++t) h[OFF_W2 + t] = (float)(uni() / std::sqrt((double)H));
    for (int64_t t = 0; t < H; ++t) h[OFF_W3 + t] = (float)(0.1 * uni() / std::sqrt((double)H));
    for (int q = 0; q < NF; ++q) h[OFF_SD + q] = 1.0f;
    FCC_CUDA(cudaMemcpyAsync(m->p.p, h.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, m->stream));
    m->m1.zero(m->stream);
    m->m2.zero(m->stream);
    m->g.zero(m->stream);
    to_bf16_kernel<<<grid_of(NPARAM), 256, 0, m->stream>>>(m->p.p, m->pb.p, NPARAM);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaStreamSynchronize(m->stream));
    return FCC_OK;
  });
  if (rc != FCC_OK) { delete m; return rc; }
  *out = m;
  return FCC_OK;
}

void fcc_mlp_destroy(fcc_mlp* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  cudaStream_t s = m->stream;
  if (s) cudaStreamSynchronize(s);
  delete m;
  if (s) cudaStreamDestroy(s);
}

int fcc_mlp_get_params(const fcc_mlp* m, float* params, int64_t n) {
  if (!m || !params || n != NPARAM) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    FCC_CUDA(cudaMemcpy(params, m->p.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    return FCC_OK;
  });
}

int fcc_mlp_set_params(fcc_mlp* m, const float* params, int64_t n) {
  if (!m || !params || n != NPARAM) return FCC_ERR_BAD_ARG;
  for (int q = 0; q < NF; ++q)
    if (!(params[OFF_SD + q] > 0.0f)) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    FCC_CUDA(cudaMemcpy(m->p.p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    to_bf16_kernel<<<grid_of(NPARAM), 256, 0, m->stream>>>(m->p.p, m->pb.p, NPARAM);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaStreamSynchronize(m->stream));
    m->stats = true;
    return FCC_OK;
  });
}

int fcc_mlp_collect(fcc_mlp* m, fcc_ctx* c, int32_t stride) {
  if (!m || !c || stride < 1) return FCC_ERR_BAD_ARG;
  if (!c->have_ccsd) return FCC_ERR_STATE;
  if (c->device != m->device) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    FCC_CUDA(cudaStreamSynchronize(m->stream));
    const int64_t total = c->o * c->o * c->v * c->v;
    const int64_t phase = (int64_t)(m->nsamp % stride);
    const int64_t ns = (total - phase + stride - 1) / stride;
    if (m->nsamp + ns > m->cap) {
      int64_t ncap = std::max<int64_t>(2 * m->cap, m->nsamp + ns);
      DBuf<float> X2, Y2;
      X2.alloc(ncap * NF);
      Y2.alloc(ncap);
      if (m->nsamp) {
        FCC_CUDA(cudaMemcpy(X2.p, m->X.p, sizeof(float) * m->nsamp * NF, cudaMemcpyDeviceToDevice));
        FCC_CUDA(cudaMemcpy(Y2.p, m->Y.p, sizeof(float) * m->nsamp, cudaMemcpyDeviceToDevice));
      }
      m->X = std::move(X2);
      m->Y = std::move(Y2);
      m->cap = ncap;
    }
    DBuf<double> pn;
    FeatSrc f = feat_src(c, pn);
    collect_kernel<<<grid_of(ns), 256, 0, c->stream>>>(f, c->t2.p, total, stride, phase, m->X.p, m->Y.p, m->nsamp);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaStreamSynchronize(c->stream));
    m->nsamp += ns;
    return FCC_OK;
  });
}

int fcc_mlp_collect_ex(fcc_mlp* m, fcc_ctx* c, int32_t stride, double thresh) {
  if (!m || !c || stride < 1 || !(thresh >= 0)) return FCC_ERR_BAD_ARG;
  if (!c->have_ccsd) return FCC_ERR_STATE;
  if (c->device != m->device) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    FCC_CUDA(cudaStreamSynchronize(m->stream));
    cudaStream_t s = c->stream;
    const int64_t total = c->o * c->o * c->v * c->v;
    const int64_t phase = (int64_t)(m->nsamp % stride);
    const int64_t ns = (total - phase + stride - 1) / stride;
    const int64_t nblk = std::max<int64_t>(1, std::min<int64_t>(152 * 8, (ns + CT - 1) / CT));
    const int64_t chunk = (ns + nblk - 1) / nblk;
    DBuf<double> pn;
    FeatSrc f = feat_src(c, pn);
    DBuf<int> counts;
    counts.alloc(nblk);
    collect_count_kernel<<<(unsigned)nblk, CT, 0, s>>>(f, total, stride, phase, chunk, thresh, counts.p);
    FCC_CHECK_LAUNCH();
    std::vector<int> hc(nblk);
    FCC_CUDA(cudaMemcpyAsync(hc.data(), counts.p, sizeof(int) * nblk, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    std::vector<int64_t> off(nblk);
    int64_t kept = 0;
    for (int64_t b = 0; b < nblk; ++b) { off[b] = kept; kept += hc[b]; }
    if (kept == 0) return FCC_OK;
    if (m->nsamp + kept > m->cap) {
      int64_t ncap = std::max<int64_t>(m->cap + m->cap / 2, m->nsamp + kept);
      DBuf<float> X2, Y2;
      X2.alloc(ncap * NF);
      Y2.alloc(ncap);
      if (m->nsamp) {
        FCC_CUDA(cudaMemcpy(X2.p, m->X.p, sizeof(float) * m->nsamp * NF, cudaMemcpyDeviceToDevice));
        FCC_CUDA(cudaMemcpy(Y2.p, m->Y.p, sizeof(float) * m->nsamp, cudaMemcpyDeviceToDevice));
      }
      m->X = std::move(X2);
      m->Y = std::move(Y2);
      m->cap = ncap;
    }
    DBuf<int64_t> doff;
    doff.alloc(nblk);
    FCC_CUDA(cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * nblk, cudaMemcpyHostToDevice, s));
    collect_write_kernel<<<(unsigned)nblk, CT, 0, s>>>(f, c->t2.p, total, stride, phase, chunk, thresh, doff.p, m->X.p,
                                                       m->Y.p, m->nsamp);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaStreamSynchronize(s));
    m->nsamp += kept;
    return FCC_OK;
  });
}

int64_t fcc_mlp_num_samples(const fcc_mlp* m) { return m ? m->nsamp : -1; }

// Adam training on the collected samples; the first call fixes the feature
// normalisation (mean and standard deviation of the collected features).
int fcc_mlp_train(fcc_mlp* m, int32_t steps, int32_t batch, double lr, uint64_t seed, double* loss_log) {
  if (!m || steps < 0 || batch < 1 || !(lr > 0)) return FCC_ERR_BAD_ARG;
  if (m->nsamp < 1) return FCC_ERR_STATE;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    cudaStream_t s = m->stream;
    if (!m->stats) {
      // statistics over an evenly spaced subset of at most 2^20 samples
      const int64_t step = std::max<int64_t>(1, m->nsamp >> 20);
      const int64_t ns = (m->nsamp + step - 1) / step;
      // only the rows used are copied: rows 0, step, 2 step, ...
      std::vector<float> X(ns * NF);
      FCC_CUDA(cudaMemcpy2D(X.data(), sizeof(float) * NF, m->X.p, sizeof(float) * NF * step, sizeof(float) * NF, ns,
                            cudaMemcpyDeviceToHost));
      std::vector<float> ms(2 * NF);
      for (int q = 0; q < NF; ++q) {
        double s1 = 0, s2 = 0;
        for (int64_t r = 0; r < ns; ++r) { double x = X[r * NF + q]; s1 += x; s2 += x * x; }
        double mu = s1 / ns, var = s2 / ns - mu * mu;
        ms[q] = (float)mu;
        ms[NF + q] = (float)(var > 1e-20 ? std::sqrt(var) : 1.0);
      }
      FCC_CUDA(cudaMemcpy(m->p.p + OFF_MU, ms.data(), sizeof(float) * 2 * NF, cudaMemcpyHostToDevice));
      m->stats = true;
    }
    ensure_batch(m, batch);
    DBuf<float> Xraw;
    Xraw.alloc((int64_t)batch * NF);
    for (int st = 0; st < steps; ++st) {
      gather_kernel<<<grid_of(batch), 256, 0, s>>>(m->X.p, m->Y.p, batch, seed + (uint64_t)st * 0x632BE59BD9B4E019ull,
                                                   m->nsamp, Xraw.p, m->Yb.p);
      FCC_CHECK_LAUNCH();
      normalise_kernel<<<grid_of((int64_t)batch * NF), 256, 0, s>>>(Xraw.p, batch, m->p.p + OFF_MU, m->p.p + OFF_SD,
                                                                     m->Xb.p);
      FCC_CHECK_LAUNCH();
      double loss = fwd_bwd(m, batch, m->Yb.p, true);
      if (loss_log) loss_log[st] = loss;
      ++m->adam_t;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.0f - std::pow(b1, (float)m->adam_t), c2 = 1.0f - std::pow(b2, (float)m->adam_t);
      adam_kernel<<<grid_of(NTRAIN), 256, 0, s>>>(m->p.p, m->g.p, m->m1.p, m->m2.p, m->pb.p, NTRAIN, (float)lr, b1, b2,
                                                   1e-8f, c1, c2);
      FCC_CHECK_LAUNCH();
    }
    FCC_CUDA(cudaStreamSynchronize(s));
    return FCC_OK;
  });
}

// One forward/backward on given raw samples (n x 16 features, targets):
// gradient of the mean squared error w.r.t. the trained parameters (the
// gradient check), loss returned.
int fcc_mlp_grad(fcc_mlp* m, const float* X, const float* y, int32_t n, float* grad, double* loss) {
  if (!m || !X || !y || n < 1 || !grad) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    cudaStream_t s = m->stream;
    ensure_batch(m, n);
    DBuf<float> Xraw;
    Xraw.alloc((int64_t)n * NF);
    FCC_CUDA(cudaMemcpyAsync(Xraw.p, X, sizeof(float) * n * NF, cudaMemcpyHostToDevice, s));
    FCC_CUDA(cudaMemcpyAsync(m->Yb.p, y, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    normalise_kernel<<<grid_of((int64_t)n * NF), 256, 0, s>>>(Xraw.p, n, m->p.p + OFF_MU, m->p.p + OFF_SD, m->Xb.p);
    FCC_CHECK_LAUNCH();
    double l = fwd_bwd(m, n, m->Yb.p, true);
    FCC_CUDA(cudaMemcpyAsync(grad, m->g.p, sizeof(float) * NTRAIN, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = l;
    return FCC_OK;
  });
}

// T1 = 0 and T2 = MP2 + lam * learned correction (applied where
// |t_MP2| >= thresh), built on the device.
int fcc_mlp_guess_ex(fcc_ctx* c, const fcc_mlp* mc, double lam, double thresh) {
  fcc_mlp* m = const_cast<fcc_mlp*>(mc);
  if (!c || !m) return FCC_ERR_BAD_ARG;
  if (!c->have_ints) return FCC_ERR_STATE;
  if (c->device != m->device) return FCC_ERR_BAD_ARG;
  return guard([&]() {
    FCC_CUDA(cudaSetDevice(m->device));
    FCC_CUDA(cudaStreamSynchronize(c->stream));
    cudaStream_t s = m->stream;
    const int64_t total = c->o * c->o * c->v * c->v;
    const int64_t chunk = 1 << 18;
    ensure_batch(m, chunk);
    DBuf<double> pn;
    FeatSrc f = feat_src(c, pn);
    FCC_CUDA(cudaStreamSynchronize(c->stream));
    // MP2 everywhere; the network runs only on the elements whose correction
    // is applied (|t_MP2| >= thresh), compacted into sel
    DBuf<int64_t> sel;
    DBuf<unsigned long long> nsel;
    sel.alloc(total);
    nsel.alloc(1);
    FCC_CUDA(cudaMemsetAsync(nsel.p, 0, sizeof(unsigned long long), s));
    mp2_select_kernel<<<grid_of(total), 256, 0, s>>>(f, total, thresh, c->t2.p, sel.p, nsel.p);
    FCC_CHECK_LAUNCH();
    unsigned long long hsel = 0;
    FCC_CUDA(cudaMemcpyAsync(&hsel, nsel.p, sizeof(hsel), cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    const int64_t nsel_h = (int64_t)hsel;
    for (int64_t base = 0; base < nsel_h && lam != 0.0; base += chunk) {
      const int64_t nb = std::min(chunk, nsel_h - base);
      infer_features_sel_kernel<<<grid_of(nb), 256, 0, s>>>(f, sel.p + base, nb, m->p.p + OFF_MU, m->p.p + OFF_SD,
                                                            m->Xb.p);
      FCC_CHECK_LAUNCH();
      fwd_bwd(m, nb, nullptr, false);
      infer_write_sel_kernel<<<grid_of(nb), 256, 0, s>>>(m->yb.p, sel.p + base, nb, lam, c->t2.p);
      FCC_CHECK_LAUNCH();
    }
    pair_symmetrise_kernel<<<grid_of(total), 256, 0, s>>>(c->t2.p, (int)c->o, (int)c->v);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaMemsetAsync(c->t1.p, 0, sizeof(double) * c->o * c->v, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    c->have_guess = true;
    c->have_ccsd = false;
    return FCC_OK;
  });
}

// Default inference settings: full correction on the amplitudes with
// |t_MP2| >= 3e-4, MP2 elsewhere (on the many tiny amplitudes the network's
// error is of the size of their correction).
int fcc_mlp_guess(fcc_ctx* c, const fcc_mlp* m) { return fcc_mlp_guess_ex(c, m, 1.0, 3e-4); }

}  // extern "C"
