// RCCSD / DF-RCCSD amplitude iteration on one GPU.
//
// Algorithm: Fermi.jl's closed-shell CCSD (src/Methods/CoupledCluster/RCCSD/
// RCCSDHelper.jl:8-349, driver RCCSDa.jl:92-244, DIIS src/Core/DIIS.jl).  The
// residual is evaluated in the T1-dressed density-fitted form (Koch et al.,
// J. Chem. Phys. 100, 4393 (1994); DePrince & Sherrill, J. Chem. Theory
// Comput. 9, 2687 (2013)): the three-index factors are dressed with T1 once
// per iteration and every T1 term of the reference equations is carried by
// them, leaving CCD-like doubles equations.  It is the same function of
// (T1, T2) as the reference's term-by-term sum (RCCSDHelper.jl:57-192); the
// test suite checks the two against each other for arbitrary amplitudes.
//
// Jacobi update, rms, DIIS cadence and the energy follow RCCSDa.jl exactly;
// the update, rms, DIIS error vectors and dot products and the energy are one
// fused bandwidth-bound pass (update_t2_kernel).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/fermicc_testing.h"
#include "fcc_ctx.cuh"

namespace fcc {

namespace {

constexpr int RED_BLOCKS = 608;  // 152 SMs x 4: fixed, so reductions are deterministic
constexpr int RED_THREADS = 256;
constexpr int MAX_DIIS = 8;
// partial-sum layout per block: [0] sum dT^2, [1] energy, [2..2+MAX_DIIS) dots
constexpr int NPART = 2 + MAX_DIIS;

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// Block-reduce NPART values held per thread into part[blockIdx.x*NPART + k].
__device__ void block_reduce_store(double (&vals)[NPART], int nvals, double* part) {
  __shared__ double sm[RED_THREADS / 32][NPART];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = 0; k < nvals; ++k) {
    double s = warp_sum(vals[k]);
    if (lane == 0) sm[w][k] = s;
  }
  __syncthreads();
  if (threadIdx.x < nvals) {
    double s = 0.0;
    for (int i = 0; i < RED_THREADS / 32; ++i) s += sm[i][threadIdx.x];
    part[blockIdx.x * NPART + threadIdx.x] = s;
  }
}

// Sum the per-block partials (fixed order) into out[k].
__global__ void finish_reduce_kernel(const double* part, int nblocks, int nvals, double* out) {
  int k = threadIdx.x;
  if (k >= nvals) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[b * NPART + k];
  out[k] = s;
}

struct ErrSlots {
  const float* s[MAX_DIIS];
  const double* d[MAX_DIIS];
  int n;
};

// Fused amplitude update (kernel (c)): for every element
//   dT = R / D, D = e_i + e_j - e_a - e_b (or e_i - e_a for T1),
//   Tnew = T + dT, accumulate dT^2, store dT as the DIIS error (FP32 or FP64),
//   accumulate dot(dT, e_k) with the other stored errors, and the energy
//   contribution Lt * (Tnew + t1new_ia t1new_jb) (T2 only).
// rank 2: index e -> (i, a); rank 4: e -> (i, j, a, b), b fastest.  For T2
// each warp takes whole rows (i, j, a) so the index arithmetic and
// e_i + e_j - e_a are per row; lanes read consecutive pairs of b with 128-bit
// loads (v even) or single elements.
__device__ __forceinline__ void update_one(int64_t e, double t, double r, double D, double t1ab, const double* Lt,
                                           float* err_s, double* err_d, const ErrSlots& others, double& tn,
                                           double (&vals)[NPART]) {
  const double dt = r / D;
  tn = t + dt;
  vals[0] += dt * dt;
  if (Lt) vals[1] += Lt[e] * (tn + t1ab);
  double ev;
  if (err_s) { const float f = (float)dt; err_s[e] = f; ev = (double)f; }
  else if (err_d) { err_d[e] = dt; ev = dt; }
  else ev = dt;
  for (int k = 0; k < others.n; ++k) vals[2 + k] += ev * (others.s[k] ? (double)others.s[k][e] : others.d[k][e]);
}

__global__ void __launch_bounds__(RED_THREADS) update_kernel(
    int rank, const double* __restrict__ T, const double* __restrict__ R, const double* __restrict__ eps,
    int o, int v, double* __restrict__ Tnew, float* __restrict__ err_s, double* __restrict__ err_d,
    ErrSlots others, const double* __restrict__ Lt, const double* __restrict__ t1new, double* part) {
  double vals[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) vals[k] = 0.0;
  if (rank == 2) {
    const int total = o * v;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
      const int i = e / v, a = e - i * v;
      double tn;
      update_one(e, T[e], R[e], eps[i] - eps[o + a], 0.0, nullptr, err_s, err_d, others, tn, vals);
      Tnew[e] = tn;
    }
  } else {
    const int lane = threadIdx.x & 31;
    const int64_t nrows = (int64_t)o * o * v;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool pairs = (v & 1) == 0;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += nw) {
      const int a = (int)(row % v);
      const int64_t ij = row / v;
      const int j = (int)(ij % o), i = (int)(ij / o);
      const double Drow = eps[i] + eps[j] - eps[o + a];
      const double t1ia = Lt ? t1new[(int64_t)i * v + a] : 0.0;
      const double* t1j = t1new + (int64_t)j * v;
      const double* ev = eps + o;
      const int64_t base = row * v;
      if (pairs) {
        for (int b = 2 * lane; b < v; b += 64) {
          const int64_t e = base + b;
          const double2 tv = *reinterpret_cast<const double2*>(T + e);
          const double2 rv = *reinterpret_cast<const double2*>(R + e);
          double2 tn;
          update_one(e, tv.x, rv.x, Drow - ev[b], Lt ? t1ia * t1j[b] : 0.0, Lt, err_s, err_d, others, tn.x, vals);
          update_one(e + 1, tv.y, rv.y, Drow - ev[b + 1], Lt ? t1ia * t1j[b + 1] : 0.0, Lt, err_s, err_d, others,
                     tn.y, vals);
          *reinterpret_cast<double2*>(Tnew + e) = tn;
        }
      } else {
        for (int b = lane; b < v; b += 32) {
          const int64_t e = base + b;
          double tn;
          update_one(e, T[e], R[e], Drow - ev[b], Lt ? t1ia * t1j[b] : 0.0, Lt, err_s, err_d, others, tn, vals);
          Tnew[e] = tn;
        }
      }
    }
  }
  block_reduce_store(vals, 2 + others.n, part);
}

// Self dot of the stored error (its norm^2 in the stored precision).
__global__ void __launch_bounds__(RED_THREADS) selfdot_kernel(int64_t total, const float* es, const double* ed,
                                                              double* part) {
  double vals[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) vals[k] = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    double x = es ? (double)es[e] : ed[e];
    vals[0] += x * x;
  }
  block_reduce_store(vals, 1, part);
}

// DIIS extrapolation: out = sum_k c_k (vec_k + add_res * err_k); for T2 also
// accumulates the energy with the already extrapolated t1.
struct VecSlots {
  const double* vec[MAX_DIIS];
  const float* es[MAX_DIIS];
  const double* ed[MAX_DIIS];
  int n;
};

__global__ void __launch_bounds__(RED_THREADS) extrapolate_kernel(int rank, int o, int v, VecSlots sl,
                                                                  const double* __restrict__ coef,
                                                                  double* __restrict__ out,
                                                                  const double* __restrict__ Lt,
                                                                  const double* __restrict__ t1new, double* part) {
  double vals[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) vals[k] = 0.0;
  double c[MAX_DIIS];
  for (int k = 0; k < sl.n; ++k) c[k] = coef[k];
  auto combine = [&](int64_t e) {
    double s = 0.0;
    for (int k = 0; k < sl.n; ++k) {
      const double ev = sl.es[k] ? (double)sl.es[k][e] : sl.ed[k][e];
      s += c[k] * sl.vec[k][e] + c[k] * ev;
    }
    out[e] = s;
    return s;
  };
  if (rank == 2) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < o * v; e += gridDim.x * blockDim.x) combine(e);
  } else {
    // whole rows (i, j, a) per warp, lanes along b
    const int lane = threadIdx.x & 31;
    const int64_t nrows = (int64_t)o * o * v;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += nw) {
      const int a = (int)(row % v);
      const int64_t ij = row / v;
      const int j = (int)(ij % o), i = (int)(ij / o);
      const double t1ia = Lt ? t1new[(int64_t)i * v + a] : 0.0;
      for (int b = lane; b < v; b += 32) {
        const int64_t e = row * v + b;
        const double s = combine(e);
        if (Lt) vals[1] += Lt[e] * (s + t1ia * t1new[(int64_t)j * v + b]);
      }
    }
  }
  block_reduce_store(vals, 2, part);
}

// Energy of given amplitudes: sum Lt * (t2 + t1 t1), whole rows (i, j, a) per warp.
__global__ void __launch_bounds__(RED_THREADS) energy_kernel(int o, int v, const double* __restrict__ t2,
                                                             const double* __restrict__ t1,
                                                             const double* __restrict__ Lt, double* part) {
  double vals[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) vals[k] = 0.0;
  const int lane = threadIdx.x & 31;
  const int64_t nrows = (int64_t)o * o * v;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += nw) {
    const int a = (int)(row % v);
    const int64_t ij = row / v;
    const int j = (int)(ij % o), i = (int)(ij / o);
    const double t1ia = t1[(int64_t)i * v + a];
    for (int b = lane; b < v; b += 32) {
      const int64_t e = row * v + b;
      vals[1] += Lt[e] * (t2[e] + t1ia * t1[(int64_t)j * v + b]);
    }
  }
  block_reduce_store(vals, 2, part);
}

// DF-MP2 correlation energy from (ia|jb) (RMP2a.jl:91-140 forms the same sum
// pair by pair from the factors): sum (ia|jb) [2 (ia|jb) - (ib|ja)] / D_ijab,
// whole rows (i, j, a) per warp, lanes along b.
__global__ void __launch_bounds__(RED_THREADS) mp2_energy_kernel(int o, int v, const double* __restrict__ ovov,
                                                                 const double* __restrict__ eps, double* part) {
  double vals[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) vals[k] = 0.0;
  const int lane = threadIdx.x & 31;
  const int64_t nrows = (int64_t)o * o * v;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += nw) {
    const int a = (int)(row % v);
    const int64_t ij = row / v;
    const int j = (int)(ij % o), i = (int)(ij / o);
    const double Dia = eps[i] + eps[j] - eps[o + a];
    const double* iajb = ovov + (((int64_t)i * v + a) * o + j) * v;   // (ia|jb) over b
    for (int b = lane; b < v; b += 32) {
      const double x = iajb[b];
      const double y = ovov[(((int64_t)i * v + b) * o + j) * v + a];   // (ib|ja)
      vals[1] += x * (2.0 * x - y) / (Dia - eps[o + b]);
    }
  }
  block_reduce_store(vals, 2, part);
}

// Solve the bordered DIIS system B c = (0,..,0,1) in FP64 with partial
// pivoting (DIIS.jl:66-87); one thread, N <= MAX_DIIS + 1.
__global__ void diis_solve_kernel(const double* Bm, int N, double* coef, int* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double A[MAX_DIIS + 1][MAX_DIIS + 2];
  for (int r = 0; r < N; ++r) {
    for (int c = 0; c < N; ++c) A[r][c] = Bm[r * N + c];
    A[r][N] = (r == N - 1) ? 1.0 : 0.0;
  }
  int st = 0;
  for (int col = 0; col < N; ++col) {
    int piv = col;
    for (int r = col + 1; r < N; ++r)
      if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
    if (A[piv][col] == 0.0) { st = 1; break; }
    if (piv != col)
      for (int c = 0; c <= N; ++c) { double t = A[col][c]; A[col][c] = A[piv][c]; A[piv][c] = t; }
    for (int r = col + 1; r < N; ++r) {
      double f = A[r][col] / A[col][col];
      for (int c = col; c <= N; ++c) A[r][c] -= f * A[col][c];
    }
  }
  if (!st) {
    for (int r = N - 1; r >= 0; --r) {
      double s = A[r][N];
      for (int c = r + 1; c < N; ++c) s -= A[r][c] * coef[c];
      coef[r] = s / A[r][r];
    }
  }
  *status = st;
}

// t2 <- OVOV-derived MP2 numerator / D2 (RCCSDa.jl:53-89); t1 <- 0.
__global__ void divide_d2_kernel(double* t2, const double* eps, int o, int v) {
  int64_t total = (int64_t)o * o * v * v;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e % v, r = e / v, a = r % v;
    r /= v;
    int64_t j = r % o, i = r / o;
    t2[e] /= (eps[i] + eps[j] - eps[o + a] - eps[o + b]);
  }
}

// X = 1 - T, Y = 1 + T^T with T[a,i] = t1[i,a] (n x n, row-major).
__global__ void dress_mats_kernel(const double* t1, int o, int v, double* X, double* Y) {
  int n = o + v;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
    int p = e / n, q = e % n;
    double xv = (p == q) ? 1.0 : 0.0, yv = xv;
    if (p >= o && q < o) xv -= t1[q * v + (p - o)];   // X[a,i] = -t_ia
    if (p < o && q >= o) yv += t1[p * v + (q - o)];   // Y[i,a] = +t_ia
    X[e] = xv;
    Y[e] = yv;
  }
}

__global__ void fill_kernel(double* p, int64_t n, double val) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) p[e] = val;
}

__global__ void add_diag_kernel(double* M, const double* d, int n, double scale) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) M[(int64_t)e * n + e] += scale * d[e];
}

__global__ void axpby_flat_kernel(double* y, const double* x, int64_t n, double a, double b) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = a * y[e] + b * x[e];
}

// ---- symmetric / antisymmetric particle-particle ladder
// (Scuseria, Janssen & Schaefer, J. Chem. Phys. 89, 7382 (1988)):
//   L_ij^ab = sum_cd t_ij^cd (ac|bd) = X+ + X-, with
//   X+ = sum_{c<=d} t+_ij^cd W+_ab^cd,  X- = sum_{c<d} t-_ij^cd W-_ab^cd,
//   t+- = (t^cd +- t^dc)/2 (t+^cc = t^cc),  W+- = W^cd +- W^dc (W+^cc = W^cc),
// X+ symmetric and X- antisymmetric under (i<->j) and under (a<->b), so only
// i <= j, a <= b (i < j, a < b for X-) are formed.

// Tp[p][q] = t+ over (i<=j, c<=d), Tm[p'][q'] = t- over (i<j, c<d)
__global__ void build_tpm_kernel(const double* __restrict__ t2, int o, int v, const int2* __restrict__ ijP,
                                 const int2* __restrict__ ijM, const int2* __restrict__ cdP,
                                 const int2* __restrict__ cdM, int64_t nP, int64_t nM, int64_t nij_p,
                                 int64_t nij_m, double* __restrict__ Tp, double* __restrict__ Tm) {
  const int64_t totP = nij_p * nP, totM = nij_m * nM;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totP + totM; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < totP) {
      const int64_t p = t / nP, q = t - p * nP;
      const int2 ij = ijP[p], cd = cdP[q];
      const double* tr = t2 + ((int64_t)ij.x * o + ij.y) * v * v;
      Tp[t] = (cd.x == cd.y) ? tr[(int64_t)cd.x * v + cd.y]
                             : 0.5 * (tr[(int64_t)cd.x * v + cd.y] + tr[(int64_t)cd.y * v + cd.x]);
    } else {
      const int64_t u = t - totP;
      const int64_t p = u / nM, q = u - p * nM;
      const int2 ij = ijM[p], cd = cdM[q];
      const double* tr = t2 + ((int64_t)ij.x * o + ij.y) * v * v;
      Tm[u] = 0.5 * (tr[(int64_t)cd.x * v + cd.y] - tr[(int64_t)cd.y * v + cd.x]);
    }
  }
}

// W+- rows for the pairs (a,b) of the current block from the slab
// W[a-a0][c][b-a0][d] = (ac|bd), b in [a0, v).
__global__ void build_wpm_kernel(const double* __restrict__ W, int v, int a0, int64_t vb, const int2* __restrict__ abP,
                                 const int2* __restrict__ abM, int64_t rP0, int64_t nrP, int64_t rM0, int64_t nrM,
                                 const int2* __restrict__ cdP, const int2* __restrict__ cdM, int64_t nP, int64_t nM,
                                 double* __restrict__ Wp, double* __restrict__ Wm) {
  const int64_t totP = nrP * nP, totM = nrM * nM;
  auto Wat = [&](int a, int c, int b, int d) -> double {
    return W[(((int64_t)(a - a0) * v + c) * vb + (b - a0)) * v + d];
  };
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totP + totM; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < totP) {
      const int64_t r = t / nP, q = t - r * nP;
      const int2 ab = abP[rP0 + r], cd = cdP[q];
      Wp[t] = (cd.x == cd.y) ? Wat(ab.x, cd.x, ab.y, cd.y) : Wat(ab.x, cd.x, ab.y, cd.y) + Wat(ab.x, cd.y, ab.y, cd.x);
    } else {
      const int64_t u = t - totP;
      const int64_t r = u / nM, q = u - r * nM;
      const int2 ab = abM[rM0 + r], cd = cdM[q];
      Wm[u] = Wat(ab.x, cd.x, ab.y, cd.y) - Wat(ab.x, cd.y, ab.y, cd.x);
    }
  }
}

// R2 += L for the four index orders of every (i<=j, a<=b) of the block.
__global__ void ladder_scatter_kernel(const double* __restrict__ Xp, const double* __restrict__ Xm, int o, int v,
                                      const int2* __restrict__ ijP, const int2* __restrict__ abP, int64_t nij_p,
                                      int64_t rP0, int64_t nrP, int64_t rM0, int64_t nrM, double* __restrict__ R2) {
  const int64_t tot = nij_p * nrP;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / nrP, r = t - p * nrP;
    const int2 ij = ijP[p], ab = abP[rP0 + r];
    const int i = ij.x, j = ij.y, a = ab.x, b = ab.y;
    const double xp = Xp[p * nrP + r];
    double xm = 0.0;
    if (i < j && a < b) {
      // positions in the (i<j) and (a<b) lists, both row-major
      const int64_t pm = (int64_t)i * o - (int64_t)i * (i + 1) / 2 + (j - i - 1);
      const int64_t rm = (int64_t)a * v - (int64_t)a * (a + 1) / 2 + (b - a - 1) - rM0;
      xm = Xm[pm * nrM + rm];
    }
    const int64_t vv = (int64_t)v * v;
    R2[((int64_t)i * o + j) * vv + (int64_t)a * v + b] += xp + xm;
    if (a != b) R2[((int64_t)i * o + j) * vv + (int64_t)b * v + a] += xp - xm;
    if (i != j) R2[((int64_t)j * o + i) * vv + (int64_t)a * v + b] += xp - xm;
    if (i != j && a != b) R2[((int64_t)j * o + i) * vv + (int64_t)b * v + a] += xp + xm;
  }
}

int grid_for(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

// ------------------------------------------------------------------- setup
// Constant tensors derived once from the three-index factors.
void setup_integrals(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  TView Bf = rm(c->B.p, {Q, n, n});
  TView Bov = slice(slice(Bf, 1, 0, o), 2, o, v);
  c->ovov.alloc(o * v * o * v);
  c->Lldkc.alloc(o * v * o * v);
  c->Lt.alloc(o * o * v * v);
  TView ovov = rm(c->ovov.p, {o, v, o, v});
  einsum(1.0, "Qkc,Qld->kcld", Bov, Bov, 0.0, ovov, s);
  TView L = rm(c->Lldkc.p, {o, v, o, v});
  einsum1(2.0, "ldkc->ldkc", ovov, 0.0, L, s);
  einsum1(-1.0, "lckd->ldkc", ovov, 1.0, L, s);
  TView Lt = rm(c->Lt.p, {o, o, v, v});
  einsum1(2.0, "kcld->klcd", ovov, 0.0, Lt, s);
  einsum1(-1.0, "kdlc->klcd", ovov, 1.0, Lt, s);
  c->V2.alloc(o * o * v * v);
  einsum1(1.0, "kcld->klcd", ovov, 0.0, rm(c->V2.p, {o, o, v, v}), s);

  // one-body part h = diag(eps) - G(B), G_pq = 2 sum_Qk (pq|kk) - (pk|kq)
  c->h.alloc(n * n);
  c->F.alloc(n * n);
  c->Xm.alloc(n * n);
  c->Ym.alloc(n * n);
  c->tmpnn.alloc(n * n);
  c->ones.alloc(std::max<int64_t>(o, 1));
  c->gam.alloc(Q);
  fill_kernel<<<1, 256, 0, s>>>(c->ones.p, c->ones.n, 1.0);
  FCC_CHECK_LAUNCH();
  TView h = rm(c->h.p, {n, n});
  // gamma_Q = sum_k B[Q,k,k]
  TView diag;
  diag.p = c->B.p; diag.rank = 2; diag.dim[0] = Q; diag.dim[1] = o; diag.str[0] = n * n; diag.str[1] = n + 1;
  TView onesv = rm(c->ones.p, {o});
  TView gam = rm(c->gam.p, {Q});
  einsum(1.0, "Qk,k->Q", diag, onesv, 0.0, gam, s);
  einsum(-2.0, "Qpq,Q->pq", Bf, gam, 0.0, h, s);
  einsum(1.0, "Qpk,Qkq->pq", slice(Bf, 2, 0, o), slice(Bf, 1, 0, o), 1.0, h, s);
  add_diag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c->h.p, c->eps.p, (int)n, 1.0);
  FCC_CHECK_LAUNCH();

  // work tensors
  c->t1.alloc(o * v);
  c->t2.alloc(o * o * v * v);
  c->r1.alloc(o * v);
  c->r2.alloc(o * o * v * v);
  c->u.alloc(o * o * v * v);
  c->P.alloc(o * o * v * v);
  c->Cint.alloc(o * o * v * v);
  c->Dint.alloc(o * o * v * v);
  c->Fring.alloc(o * o * v * v);
  c->Xo.alloc(o * o * o * o);
  c->Xq.alloc(Q * o * v);
  c->Yq.alloc(Q * o * v);
  c->Fvv.alloc(v * v);
  c->Foo.alloc(o * o);
  c->Bt.alloc(Q * n * n);
  c->red.alloc(RED_BLOCKS * NPART + 64);
  // ladder: (ac|bd) slab for a block of virtuals a (b >= block start), blocks
  // of a sized to ~512 MB; pair tables of the symmetric/antisymmetric channels
  int64_t per_a = v * v * v;
  c->ladder_block = std::max<int64_t>(1, std::min<int64_t>(v, (int64_t)(64ll << 20) / std::max<int64_t>(per_a, 1)));
  c->Wslab.alloc(c->ladder_block * per_a);
  auto tri = [&](DBuf<int2>& dst, int64_t nx, bool diag) {
    std::vector<int2> h;
    for (int64_t x = 0; x < nx; ++x)
      for (int64_t y = diag ? x : x + 1; y < nx; ++y) h.push_back(make_int2((int)x, (int)y));
    dst.alloc(std::max<size_t>(h.size(), 1));
    if (!h.empty()) FCC_CUDA(cudaMemcpy(dst.p, h.data(), sizeof(int2) * h.size(), cudaMemcpyHostToDevice));
  };
  tri(c->pairP_v, v, true);
  tri(c->pairM_v, v, false);
  tri(c->pairP_o, o, true);
  tri(c->pairM_o, o, false);
  const int64_t nP = v * (v + 1) / 2, nM = v * (v - 1) / 2;
  const int64_t nijP = o * (o + 1) / 2, nijM = o * (o - 1) / 2;
  c->Tp.alloc(nijP * nP);
  c->Tm.alloc(std::max<int64_t>(1, nijM * nM));
  const int64_t rows_max = c->ladder_block * v;
  c->Wp.alloc(rows_max * nP);
  c->Wm.alloc(std::max<int64_t>(1, rows_max * nM));
  c->LXp.alloc(nijP * rows_max);
  c->LXm.alloc(std::max<int64_t>(1, nijM * rows_max));
}

void make_mp2_guess(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v;
  FCC_CUDA(cudaMemsetAsync(c->t1.p, 0, sizeof(double) * o * v, s));
  einsum1(1.0, "iajb->ijab", rm(c->ovov.p, {o, v, o, v}), 0.0, rm(c->t2.p, {o, o, v, v}), s);
  divide_d2_kernel<<<grid_for(o * o * v * v), 256, 0, s>>>(c->t2.p, c->eps.p, (int)o, (int)v);
  FCC_CHECK_LAUNCH();
}

double cc_energy(fcc_ctx* c, const double* t1, const double* t2) {
  cudaStream_t s = c->stream;
  energy_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>((int)c->o, (int)c->v, t2, t1, c->Lt.p, c->red.p);
  FCC_CHECK_LAUNCH();
  double* out = c->red.p + RED_BLOCKS * NPART;
  finish_reduce_kernel<<<1, 32, 0, s>>>(c->red.p, RED_BLOCKS, 2, out);
  FCC_CHECK_LAUNCH();
  double h[2];
  FCC_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  return h[1];
}

double mp2_energy(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  mp2_energy_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>((int)c->o, (int)c->v, c->ovov.p, c->eps.p, c->red.p);
  FCC_CHECK_LAUNCH();
  double* out = c->red.p + RED_BLOCKS * NPART;
  finish_reduce_kernel<<<1, 32, 0, s>>>(c->red.p, RED_BLOCKS, 2, out);
  FCC_CHECK_LAUNCH();
  double h[2];
  FCC_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  return h[1];
}

// ---------------------------------------------------------------- residual
// Full CCSD residuals r1 = Omega_ia, r2 = Omega_ijab (zero at convergence) for
// the current t1, t2; the reference's pre-denominator amplitudes are
// r + D * t (RCCSDHelper.jl:304-349).
void residual(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  TView t1 = rm(c->t1.p, {o, v});
  TView t2 = rm(c->t2.p, {o, o, v, v});
  TView B = rm(c->B.p, {Q, n, n});
  TView Bt = rm(c->Bt.p, {Q, n, n});
  auto blk = [](TView t, int64_t r0, int64_t nr, int64_t c0, int64_t nc) {
    return slice(slice(t, 1, r0, nr), 2, c0, nc);
  };
  TView Boo = blk(B, 0, o, 0, o), Bov = blk(B, 0, o, o, v), Bvo = blk(B, o, v, 0, o), Bvv = blk(B, o, v, o, v);
  TView Btoo = blk(Bt, 0, o, 0, o), Btov = blk(Bt, 0, o, o, v), Btvo = blk(Bt, o, v, 0, o), Btvv = blk(Bt, o, v, o, v);

  // ---- T1-dressed factors: Bt = X B Y^T blockwise
  einsum1(1.0, "Qij->Qij", Boo, 0.0, Btoo, s);
  einsum(1.0, "Qib,jb->Qij", Bov, t1, 1.0, Btoo, s);
  einsum1(1.0, "Qia->Qia", Bov, 0.0, Btov, s);
  einsum1(1.0, "Qab->Qab", Bvv, 0.0, Btvv, s);
  einsum(-1.0, "ka,Qkb->Qab", t1, Bov, 1.0, Btvv, s);
  einsum1(1.0, "Qai->Qai", Bvo, 0.0, Btvo, s);
  einsum(-1.0, "ka,Qki->Qai", t1, Boo, 1.0, Btvo, s);
  einsum(1.0, "Qac,ic->Qai", Btvv, t1, 1.0, Btvo, s);

  // ---- dressed Fock F = X h Y^T + G(Bt)
  dress_mats_kernel<<<grid_for(n * n), 256, 0, s>>>(c->t1.p, (int)o, (int)v, c->Xm.p, c->Ym.p);
  FCC_CHECK_LAUNCH();
  TView X = rm(c->Xm.p, {n, n}), Y = rm(c->Ym.p, {n, n}), H = rm(c->h.p, {n, n});
  TView tmp = rm(c->tmpnn.p, {n, n}), F = rm(c->F.p, {n, n});
  einsum(1.0, "pr,rs->ps", X, H, 0.0, tmp, s);
  einsum(1.0, "ps,qs->pq", tmp, Y, 0.0, F, s);
  TView diag;
  diag.p = c->Bt.p; diag.rank = 2; diag.dim[0] = Q; diag.dim[1] = o; diag.str[0] = n * n; diag.str[1] = n + 1;
  TView gam = rm(c->gam.p, {Q});
  einsum(1.0, "Qk,k->Q", diag, rm(c->ones.p, {o}), 0.0, gam, s);
  einsum(2.0, "Qpq,Q->pq", Bt, gam, 1.0, F, s);
  einsum(-1.0, "Qpk,Qkq->pq", slice(Bt, 2, 0, o), slice(Bt, 1, 0, o), 1.0, F, s);
  TView Foo_ = blk(rm(c->F.p, {1, n, n}), 0, o, 0, o), Fov_ = blk(rm(c->F.p, {1, n, n}), 0, o, o, v);
  TView Fvo_ = blk(rm(c->F.p, {1, n, n}), o, v, 0, o), Fvv_ = blk(rm(c->F.p, {1, n, n}), o, v, o, v);
  auto drop0 = [](TView t) {  // remove the leading unit index
    TView r; r.p = t.p; r.rank = t.rank - 1;
    for (int k = 1; k < t.rank; ++k) { r.dim[k - 1] = t.dim[k]; r.str[k - 1] = t.str[k]; }
    return r;
  };
  TView Foo = drop0(Foo_), Fov = drop0(Fov_), Fvo = drop0(Fvo_), Fvv = drop0(Fvv_);

  TView ovov = rm(c->ovov.p, {o, v, o, v});
  TView L = rm(c->Lldkc.p, {o, v, o, v});
  TView u = rm(c->u.p, {o, o, v, v});
  TView R2 = rm(c->r2.p, {o, o, v, v});
  TView R1 = rm(c->r1.p, {o, v});
  TView P = rm(c->P.p, {o, o, v, v});
  TView Ci = rm(c->Cint.p, {o, o, v, v});   // [k][i][a][c]
  TView Di = rm(c->Dint.p, {v, o, o, v});   // [a][i][k][c]
  TView Xo = rm(c->Xo.p, {o, o, o, o});     // [k][i][l][j]

  // u_ijab = 2 t_ijab - t_jiab
  einsum1(2.0, "ijab->ijab", t2, 0.0, u, s);
  einsum1(-1.0, "jiab->ijab", t2, 1.0, u, s);

  // ---- doubles
  einsum(1.0, "Qai,Qbj->ijab", Btvo, Btvo, 0.0, R2, s);                 // (ai|bj)
  // particle-particle ladder in the symmetric / antisymmetric channels, one
  // block of virtual a at a time (no vvvv is ever stored)
  {
    const int64_t nP = v * (v + 1) / 2, nM = v * (v - 1) / 2;
    const int64_t nijP = o * (o + 1) / 2, nijM = o * (o - 1) / 2;
    build_tpm_kernel<<<grid_for(nijP * nP + nijM * nM), 256, 0, s>>>(c->t2.p, (int)o, (int)v, c->pairP_o.p,
                                                                    c->pairM_o.p, c->pairP_v.p, c->pairM_v.p, nP, nM,
                                                                    nijP, nijM, c->Tp.p, c->Tm.p);
    FCC_CHECK_LAUNCH();
    // Tp and Tm are the A operands of every block's ladder product: packed once
    KeepPackedA keep(tc_engine(), c->Tp.p, c->Tm.p);
    auto startP = [&](int64_t a) { return a * v - a * (a - 1) / 2; };   // first (a, b>=a) row
    auto startM = [&](int64_t a) { return a * v - a * (a + 1) / 2; };   // first (a, b>a) row
    // On the tensor cores every block's (ac|bd) = sum_Q Bt[Q][a][c] Bt[Q][b][d]
    // takes its rows (a, c) for a in the block and (b, d) for b >= a0 from one
    // packing of Bt over all (x, y) (row x * v + y, K = Q): two row ranges of
    // the same packed array, instead of packing both slices for every block.
    TcEngine* tc = tc_engine();
    const bool tcw = tc && tc->enabled;
    const int64_t R = v * v;
    int64_t Wk = 0;   // packed row length
    if (tcw) {
      PackSpec ps{};
      ps.R = R; ps.K = Q;
      ps.rd2 = 1; ps.rd3 = v; ps.rs1 = n; ps.rs2 = 0; ps.rs3 = 1;
      ps.kd2 = 1; ps.kd3 = Q; ps.ks1 = 0; ps.ks2 = 0; ps.ks3 = n * n;
      if (tc->exact) {
        const int S = tc->oz_groups - 1;
        Wk = S * oz_kpad(Q);
        ps.Kp = Wk;
        if ((int64_t)c->bvvA.n < R * Wk) c->bvvA.alloc(R * Wk);
        if ((int64_t)c->bvvEx.n < R) c->bvvEx.alloc(R);
        pack_oz(Btvv.p, ps, S, c->bvvA.p, c->bvvEx.p, s);
      } else {
        Wk = packed_kp(Q, tc->scheme.P);
        ps.Kp = Wk;
        ps.P = tc->scheme.P;
        if ((int64_t)c->bvvA.n < R * Wk) c->bvvA.alloc(R * Wk);
        if ((int64_t)c->bvvB.n < R * Wk) c->bvvB.alloc(R * Wk);
        ps.code = tc->scheme.code_a;
        pack_split(Btvv.p, ps, c->bvvA.p, s);
        ps.code = tc->scheme.code_b;
        pack_split(Btvv.p, ps, c->bvvB.p, s);
      }
    }
    for (int64_t a0 = 0; a0 < v; a0 += c->ladder_block) {
      const int64_t na = std::min<int64_t>(c->ladder_block, v - a0);
      const int64_t vb = v - a0;
      TView W = rm(c->Wslab.p, {na, v, vb, v});                            // [a][c][b-a0][d]
      if (tcw) {
        EpiMap ep;
        ep.M = na * v;
        ep.N = vb * v;
        ep.ms1 = vb * v;   // W[(a, c)][(b, d)]
        ep.ns1 = 1;
        ep.alpha = 1.0; ep.beta = 0.0; ep.C = c->Wslab.p; ep.mode = EPI_F64;
        const int64_t r0 = a0 * v;
        if (tc->exact) {
          const int G = tc->oz_groups;
          ep.work = 2.0 * (double)ep.M * (double)ep.N * (double)Q * ((double)(G - 1) * (double)G / 2.0);
          gemm_oz(c->bvvA.p + r0 * Wk, ep.M, c->bvvEx.p + r0, c->bvvA.p + r0 * Wk, ep.N, c->bvvEx.p + r0, Wk / (G - 1),
                  G, ep, tc->err, s);
        } else {
          ep.work = 2.0 * (double)ep.M * (double)ep.N * (double)Q * tc->scheme.P;
          ep.no_loads = tc->no_loads_once;
          tc->no_loads_once = 0;
          gemm_bf16x3(c->bvvA.p, R, r0, c->bvvB.p, R, r0, Wk, ep, tc->err, s);
        }
        tc->tc_calls++;
        tc->tc_flops += ep.work;
      } else {
        einsum(1.0, "Qac,Qbd->acbd", slice(Btvv, 1, a0, na), slice(Btvv, 1, a0, vb), 0.0, W, s);
      }
      const int64_t rP0 = startP(a0), nrP = startP(a0 + na) - rP0;
      const int64_t rM0 = startM(a0), nrM = startM(a0 + na) - rM0;
      build_wpm_kernel<<<grid_for(nrP * nP + nrM * nM), 256, 0, s>>>(c->Wslab.p, (int)v, (int)a0, vb, c->pairP_v.p,
                                                                    c->pairM_v.p, rP0, nrP, rM0, nrM, c->pairP_v.p,
                                                                    c->pairM_v.p, nP, nM, c->Wp.p, c->Wm.p);
      FCC_CHECK_LAUNCH();
      einsum(1.0, "pq,rq->pr", rm(c->Tp.p, {nijP, nP}), rm(c->Wp.p, {nrP, nP}), 0.0, rm(c->LXp.p, {nijP, nrP}), s);
      if (nijM > 0 && nrM > 0)
        einsum(1.0, "pq,rq->pr", rm(c->Tm.p, {nijM, nM}), rm(c->Wm.p, {nrM, nM}), 0.0, rm(c->LXm.p, {nijM, nrM}), s);
      ladder_scatter_kernel<<<grid_for(nijP * nrP), 256, 0, s>>>(c->LXp.p, c->LXm.p, (int)o, (int)v, c->pairP_o.p,
                                                                c->pairP_v.p, nijP, rP0, nrP, rM0, nrM, c->r2.p);
      FCC_CHECK_LAUNCH();
    }
  }
  // hole-hole ladder
  einsum(1.0, "Qki,Qlj->kilj", Btoo, Btoo, 0.0, Xo, s);
  einsum(1.0, "ijcd,kcld->kilj", t2, ovov, 1.0, Xo, s);
  einsum(1.0, "klab,kilj->ijab", t2, Xo, 1.0, R2, s);
  // C and D intermediates
  einsum(1.0, "Qki,Qac->kiac", Btoo, Btvv, 0.0, Ci, s);                 // (ki|ac)
  einsum(2.0, "Qai,Qkc->aikc", Btvo, Btov, 0.0, Di, s);                 // 2 (ai|kc)
  einsum1(-1.0, "kiac->aikc", Ci, 1.0, Di, s);                          // - (ac|ki)
  einsum(0.5, "ilad,ldkc->aikc", u, L, 1.0, Di, s);
  einsum(-0.5, "liad,kdlc->kiac", t2, ovov, 1.0, Ci, s);
  // -1/2 t_kj^bc C_ki^ac - t_ki^bc C_kj^ac = -1/2 F_ijab - F_jiab with
  // F_ijab = t_kj^bc C_ki^ac: one o^3 v^3 contraction instead of two
  TView Fr = rm(c->Fring.p, {o, o, v, v});
  einsum(1.0, "kjbc,kiac->ijab", t2, Ci, 0.0, Fr, s);
  einsum1(-0.5, "ijab->ijab", Fr, 0.0, P, s);
  einsum1(-1.0, "jiab->ijab", Fr, 1.0, P, s);
  einsum(0.5, "jkbc,aikc->ijab", u, Di, 1.0, P, s);
  // Fock-like terms
  TView Fvvp = rm(c->Fvv.p, {v, v}), Foop = rm(c->Foo.p, {o, o});
  einsum1(1.0, "bc->bc", Fvv, 0.0, Fvvp, s);
  TView V2 = rm(c->V2.p, {o, o, v, v});
  einsum(-1.0, "klbd,klcd->bc", u, V2, 1.0, Fvvp, s);
  einsum1(1.0, "kj->kj", Foo, 0.0, Foop, s);
  einsum(1.0, "jlcd,klcd->kj", u, V2, 1.0, Foop, s);
  einsum(1.0, "ijac,bc->ijab", t2, Fvvp, 1.0, P, s);
  einsum(-1.0, "ikab,kj->ijab", t2, Foop, 1.0, P, s);
  einsum1(1.0, "ijab->ijab", P, 1.0, R2, s);
  einsum1(1.0, "jiba->ijab", P, 1.0, R2, s);

  // ---- singles
  einsum1(1.0, "ai->ia", Fvo, 0.0, R1, s);
  TView Xq = rm(c->Xq.p, {Q, o, v}), Yq = rm(c->Yq.p, {Q, o, v});
  einsum(1.0, "kicd,Qkc->Qid", u, Btov, 0.0, Xq, s);
  einsum(1.0, "Qad,Qid->ia", Btvv, Xq, 1.0, R1, s);
  einsum(1.0, "klac,Qlc->Qka", u, Btov, 0.0, Yq, s);
  einsum(-1.0, "Qki,Qka->ia", Btoo, Yq, 1.0, R1, s);
  einsum(1.0, "ikac,kc->ia", u, Fov, 1.0, R1, s);
}

// --------------------------------------------------------------- iteration
namespace {

struct DiisState {
  int ndiis = 0;
  bool fp32 = true;
  int64_t len = 0;
  std::vector<int> valid;          // slot -> 1 if occupied
  std::vector<double> norm2;       // ||e_k||^2 in stored precision
  std::vector<std::vector<double>> dot;  // dot[i][j]
  std::vector<int> age;            // insertion order, for a stable ordering of the subspace
  int counter = 0;
  int count() const { int n = 0; for (int x : valid) n += x; return n; }
};

double* vec_slot(DBuf<double>& vecs, int64_t len, int k) { return vecs.p + (int64_t)k * len; }

}  // namespace

int ccsd_run(fcc_ctx* c, const fcc_opts* opt, fcc_iter_stats* log, int32_t log_cap, fcc_ccsd_result* res) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v;
  const int64_t len1 = o * v, len2 = o * o * v * v;
  fcc_opts op = *opt;
  if (op.max_iter < 0 || op.ndiis < 1 || op.ndiis > MAX_DIIS || op.diis_relax < 1 || op.damp < 0 || op.damp >= 1)
    fail(FCC_ERR_BAD_ARG, "invalid CC options");
  if (op.precision != FCC_PREC_FP64 && op.precision != FCC_PREC_MIXED && op.precision != FCC_PREC_EXACT)
    fail(FCC_ERR_BAD_ARG, "precision must be FCC_PREC_FP64, FCC_PREC_MIXED or FCC_PREC_EXACT");
  if (op.precision == FCC_PREC_MIXED && !(op.mixed_switch_rms > 0))
    fail(FCC_ERR_BAD_ARG, "mixed_switch_rms must be positive");
  if (op.mixed_finish != FCC_FINISH_EXACT && op.mixed_finish != FCC_FINISH_FP64)
    fail(FCC_ERR_BAD_ARG, "mixed_finish must be FCC_FINISH_EXACT or FCC_FINISH_FP64");
  int phase = op.precision;  // mixed: split-BF16 contractions until the switch, then exact-slice, then the finish
  if (!c->dev_err.p) c->dev_err.alloc(1);
  FCC_CUDA(cudaMemsetAsync(c->dev_err.p, 0, sizeof(int), s));
  c->tc.err = c->dev_err.p;
  double best_rms = 1e300;
  int stalled = 0;
  int exact_groups = 0;   // exact-slice width of the last exact-slice iteration
  bool diis = op.diis != 0;
  bool fp32err = op.diis_prec != 64;

  // amplitude buffers: "cur" = newT of the reference loop
  DBuf<double> tn1, tn2, tx1, tx2;
  tn1.alloc(len1); tn2.alloc(len2);
  DiisState D1s, D2s;
  if (diis) {
    c->dvec1.alloc(len1 * op.ndiis);
    c->dvec2.alloc(len2 * op.ndiis);
    if (fp32err) { c->derr1s.alloc(len1 * op.ndiis); c->derr2s.alloc(len2 * op.ndiis); }
    else { c->derr1d.alloc(len1 * op.ndiis); c->derr2d.alloc(len2 * op.ndiis); }
    tx1.alloc(len1); tx2.alloc(len2);
    for (auto* d : {&D1s, &D2s}) {
      d->ndiis = op.ndiis; d->fp32 = fp32err;
      d->valid.assign(op.ndiis, 0); d->norm2.assign(op.ndiis, 0.0);
      d->dot.assign(op.ndiis, std::vector<double>(op.ndiis, 0.0)); d->age.assign(op.ndiis, 0);
    }
    D1s.len = len1; D2s.len = len2;
  }
  // newT starts as the guess held in c->t1/c->t2
  FCC_CUDA(cudaMemcpyAsync(tn1.p, c->t1.p, sizeof(double) * len1, cudaMemcpyDeviceToDevice, s));
  FCC_CUDA(cudaMemcpyAsync(tn2.p, c->t2.p, sizeof(double) * len2, cudaMemcpyDeviceToDevice, s));
  double* cur1 = tn1.p;
  double* cur2 = tn2.p;

  double Ecc = cc_energy(c, cur1, cur2);                                   // RCCSDa.jl:168
  double Eguess = Ecc + c->e_ref;
  double dE = 1.0, rms = 1.0;
  int ite = 1, nlog = 0;
  double* hred = nullptr;
  FCC_CUDA(cudaMallocHost(&hred, sizeof(double) * 64));
  struct HostFree { double* p; ~HostFree() { if (p) cudaFreeHost(p); } } hf{hred};
  DBuf<double> dB, dcoef;
  DBuf<int> dstat;
  dB.alloc((MAX_DIIS + 1) * (MAX_DIIS + 1));
  dcoef.alloc(MAX_DIIS + 1);
  dstat.alloc(4);
  cudaEvent_t ev0, ev1;
  FCC_CUDA(cudaEventCreate(&ev0));
  FCC_CUDA(cudaEventCreate(&ev1));
  struct EvFree { cudaEvent_t a, b; ~EvFree() { cudaEventDestroy(a); cudaEventDestroy(b); } } evf{ev0, ev1};
  double* dout = c->red.p + RED_BLOCKS * NPART;

  auto run_update = [&](int rank, DiisState& ds, DBuf<double>& vecs, DBuf<float>& es, DBuf<double>& ed,
                        const double* T, const double* R, DBuf<double>& plain, double** cur, const double* t1new,
                        double* out_sumsq, double* out_energy) {
    int64_t len = rank == 2 ? len1 : len2;
    ErrSlots others{};
    int target = -1;
    std::vector<int> other_ids;
    if (diis) {
      // DIIS.jl:38-50: evict the slot with the largest error norm when full
      if (ds.count() + 1 > ds.ndiis) {
        int worst = -1;
        for (int k = 0; k < ds.ndiis; ++k)
          if (ds.valid[k] && (worst < 0 || ds.norm2[k] > ds.norm2[worst])) worst = k;
        ds.valid[worst] = 0;
        target = worst;
      } else {
        for (int k = 0; k < ds.ndiis; ++k) if (!ds.valid[k]) { target = k; break; }
      }
      for (int k = 0; k < ds.ndiis; ++k)
        if (ds.valid[k]) {
          others.s[others.n] = ds.fp32 ? es.p + (int64_t)k * len : nullptr;
          others.d[others.n] = ds.fp32 ? nullptr : ed.p + (int64_t)k * len;
          other_ids.push_back(k);
          others.n++;
        }
    }
    double* dst = diis ? vec_slot(vecs, len, target) : plain.p;
    float* errs = (diis && ds.fp32) ? es.p + (int64_t)target * len : nullptr;
    double* errd = (diis && !ds.fp32) ? ed.p + (int64_t)target * len : nullptr;
    update_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(rank, T, R, c->eps.p, (int)o, (int)v, dst, errs, errd, others,
                                                     rank == 4 ? c->Lt.p : nullptr, t1new, c->red.p);
    FCC_CHECK_LAUNCH();
    finish_reduce_kernel<<<1, 32, 0, s>>>(c->red.p, RED_BLOCKS, 2 + others.n, dout);
    FCC_CHECK_LAUNCH();
    int nself = 0;
    if (diis) {
      selfdot_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(len, errs, errd, c->red.p);
      FCC_CHECK_LAUNCH();
      finish_reduce_kernel<<<1, 32, 0, s>>>(c->red.p, RED_BLOCKS, 1, dout + 2 + MAX_DIIS);
      FCC_CHECK_LAUNCH();
      nself = 1;
    }
    FCC_CUDA(cudaMemcpyAsync(hred, dout, sizeof(double) * (2 + MAX_DIIS + nself), cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    *out_sumsq = hred[0];
    *out_energy = hred[1];
    if (diis) {
      ds.valid[target] = 1;
      ds.age[target] = ++ds.counter;
      ds.norm2[target] = hred[2 + MAX_DIIS];
      ds.dot[target][target] = hred[2 + MAX_DIIS];
      for (size_t q = 0; q < other_ids.size(); ++q) {
        ds.dot[target][other_ids[q]] = hred[2 + q];
        ds.dot[other_ids[q]][target] = hred[2 + q];
      }
    }
    *cur = dst;
  };

  auto extrapolate = [&](int rank, DiisState& ds, DBuf<double>& vecs, DBuf<float>& es, DBuf<double>& ed,
                         DBuf<double>& outbuf, const double* t1new, double* out_energy) -> bool {
    int64_t len = rank == 2 ? len1 : len2;
    std::vector<int> ids;
    for (int k = 0; k < ds.ndiis; ++k) if (ds.valid[k]) ids.push_back(k);
    std::sort(ids.begin(), ids.end(), [&](int a, int b) { return ds.age[a] < ds.age[b]; });
    int m = (int)ids.size();
    if (m < 2) fail(FCC_ERR_STATE, "DIIS cannot extrapolate from one vector");
    int N = m + 1;
    std::vector<double> Bm(N * N, 1.0);
    Bm[N * N - 1] = 0.0;
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b) Bm[a * N + b] = ds.dot[ids[a]][ids[b]];
    FCC_CUDA(cudaMemcpyAsync(dB.p, Bm.data(), sizeof(double) * N * N, cudaMemcpyHostToDevice, s));
    diis_solve_kernel<<<1, 1, 0, s>>>(dB.p, N, dcoef.p, dstat.p);
    FCC_CHECK_LAUNCH();
    VecSlots sl{};
    for (int a = 0; a < m; ++a) {
      sl.vec[a] = vec_slot(vecs, len, ids[a]);
      sl.es[a] = ds.fp32 ? es.p + (int64_t)ids[a] * len : nullptr;
      sl.ed[a] = ds.fp32 ? nullptr : ed.p + (int64_t)ids[a] * len;
    }
    sl.n = m;
    extrapolate_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(rank, (int)o, (int)v, sl, dcoef.p, outbuf.p,
                                                          rank == 4 ? c->Lt.p : nullptr, t1new, c->red.p);
    FCC_CHECK_LAUNCH();
    finish_reduce_kernel<<<1, 32, 0, s>>>(c->red.p, RED_BLOCKS, 2, dout);
    FCC_CHECK_LAUNCH();
    int st = 0;
    FCC_CUDA(cudaMemcpyAsync(hred, dout, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaMemcpyAsync(&st, dstat.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    if (st) fail(FCC_ERR_NAN, "singular DIIS matrix");
    *out_energy = hred[1];
    return true;
  };

  int status = FCC_OK;
  bool conv_final = false;
  // Iteration kinds: FP64 residual (DMMA); split-BF16 residual with three
  // products (mixed form, first phase); exact-slice BF16 residual at 6-8
  // weight groups (mixed form, second phase: Ozaki-scheme products whose
  // error, ~1e-11 absolute in the residual, is far below the convergence
  // criteria); exact-slice residual at 9 weight groups, whose truncation
  // (below 2^-47 of max|A_r| max|B_c| per term) and exact accumulation give
  // FP64-class contractions.  A run ends only on an iteration of its finish
  // kind that meets the criteria: FP64 for the FP64 form and for the mixed
  // form with FCC_FINISH_FP64, the 9-group exact-slice residual for
  // FCC_PREC_EXACT and for the mixed form with FCC_FINISH_EXACT, so the
  // converged amplitudes are the fixed point of an FP64-accurate residual.
  enum { K_F64 = 0, K_MIX = 1, K_EXACT = 2, K_EXACT9 = 3 };
  constexpr int OZ_G_FINISH = 9;
  const int finish = (phase == FCC_PREC_FP64) ? K_F64
                     : (phase == FCC_PREC_EXACT) ? K_EXACT9
                     : (op.mixed_finish == FCC_FINISH_FP64 ? K_F64 : K_EXACT9);
  int kind = (phase == FCC_PREC_MIXED) ? K_MIX : finish;
  while (true) {
    if (ite > op.max_iter) { status = FCC_NO_CONVERGE; break; }            // :179-182
    FCC_CUDA(cudaEventRecord(ev0, s));
    // T1 .= newT1; T2 .= newT2                                              // :185-186
    if (cur1 != c->t1.p) FCC_CUDA(cudaMemcpyAsync(c->t1.p, cur1, sizeof(double) * len1, cudaMemcpyDeviceToDevice, s));
    if (cur2 != c->t2.p) FCC_CUDA(cudaMemcpyAsync(c->t2.p, cur2, sizeof(double) * len2, cudaMemcpyDeviceToDevice, s));
    double oldE = Ecc;
    const int iter_kind = kind;
    {
      TcScope scope(kind == K_F64 ? nullptr : &c->tc);
      c->tc.enabled = kind != K_F64;
      c->tc.exact = kind == K_EXACT || kind == K_EXACT9;
      if (kind == K_EXACT9) c->tc.oz_groups = OZ_G_FINISH;
      // exact-slice width by the size of the step: 6 weight groups (15 slice
      // pairs; noise floor in the Jacobi step ~1e-8 at (H2O)8) while the step
      // is above 100 max_rms, then 7 groups (21 pairs, floor ~1e-10, two
      // orders below the criteria) until the finish.  The width only grows,
      // so the phase cannot cycle.
      if (kind == K_EXACT) {
        const int want = rms < 100.0 * op.max_rms ? OZ_G_DEFAULT - 1 : OZ_G_DEFAULT - 2;
        const int groups = std::max(exact_groups, want);
        if (groups != exact_groups) { best_rms = 1e300; stalled = 0; }
        exact_groups = groups;
        c->tc.oz_groups = groups;
      }
      c->tc.scheme = SPLIT3;
      if (c->test_fault == FCC_TEST_FAULT_NO_LOADS && kind == K_MIX) {
        c->tc.no_loads_once = 1;
        c->test_fault = 0;
      }
      residual(c);                                                         // :190
      if (c->test_fault == FCC_TEST_FAULT_NAN) {
        const double nan = std::nan("");
        FCC_CUDA(cudaMemcpyAsync(c->r2.p, &nan, sizeof(double), cudaMemcpyHostToDevice, s));
        FCC_CUDA(cudaStreamSynchronize(s));
        c->test_fault = 0;
      }
    }
    double ss1, ss2, e_dummy, e_new;
    run_update(2, D1s, c->dvec1, c->derr1s, c->derr1d, c->t1.p, c->r1.p, tn1, &cur1, nullptr, &ss1, &e_dummy);
    run_update(4, D2s, c->dvec2, c->derr2s, c->derr2d, c->t2.p, c->r2.p, tn2, &cur2, cur1, &ss2, &e_new);
    double r1 = std::sqrt(ss1 / (double)len1), r2 = std::sqrt(ss2 / (double)len2);   // :193-194
    bool did = false;
    if (diis && ite >= op.diis_start && ite % op.diis_relax == 0 && D1s.count() >= 2 && D2s.count() >= 2) {   // :204
      double e1d;
      extrapolate(2, D1s, c->dvec1, c->derr1s, c->derr1d, tx1, nullptr, &e1d);
      extrapolate(4, D2s, c->dvec2, c->derr2s, c->derr2d, tx2, tx1.p, &e_new);
      cur1 = tx1.p;
      cur2 = tx2.p;
      did = true;
    }
    if (op.damp > 0) {                                                     // :213-216
      double dp = op.damp;
      double* d1 = (cur1 == tx1.p) ? tx1.p : tn1.p;
      double* d2 = (cur2 == tx2.p) ? tx2.p : tn2.p;
      if (cur1 != d1) FCC_CUDA(cudaMemcpyAsync(d1, cur1, sizeof(double) * len1, cudaMemcpyDeviceToDevice, s));
      if (cur2 != d2) FCC_CUDA(cudaMemcpyAsync(d2, cur2, sizeof(double) * len2, cudaMemcpyDeviceToDevice, s));
      axpby_flat_kernel<<<grid_for(len1), 256, 0, s>>>(d1, c->t1.p, len1, 1 - dp, dp);
      axpby_flat_kernel<<<grid_for(len2), 256, 0, s>>>(d2, c->t2.p, len2, 1 - dp, dp);
      FCC_CHECK_LAUNCH();
      cur1 = d1;
      cur2 = d2;
      e_new = cc_energy(c, cur1, cur2);
    }
    Ecc = e_new;                                                           // :218
    rms = std::max(r1, r2);                                                // :220
    const double prev_dE = dE;
    dE = Ecc - oldE;                                                       // :221
    bool converged = iter_kind == finish && std::fabs(dE) < op.e_conv && rms < op.max_rms;   // :178
    if (phase == FCC_PREC_MIXED && !converged) {
      // leave a reduced-precision phase once its residual is below the
      // threshold (split-BF16: mixed_switch_rms; exact-slice: the reference's
      // own criteria, checked next by an FP64 evaluation), or when it stops
      // improving (its noise floor)
      if (rms < best_rms * 0.7) { best_rms = rms; stalled = 0; }
      else ++stalled;
      if (iter_kind == K_MIX && (rms < op.mixed_switch_rms || stalled >= 3)) {
        kind = K_EXACT;
        best_rms = 1e300;
        stalled = 0;
      } else if (iter_kind == K_EXACT) {
        // FP64 finish (one DMMA residual costs ~25 exact-slice ones): switch
        // when the criteria hold ten times over on this iteration and hold on
        // the previous one, so that the FP64 step that follows (whose energy
        // change is the next step of the same convergence) meets them at
        // once.  Exact-slice finish (~1.5 exact-slice iterations): switch
        // once the step is below max_rms with the energy change within ten
        // times e_conv, i.e. when the next step is expected to meet the
        // criteria (an exact-slice step that met them would be one wasted
        // iteration); a finish step that misses them is followed by another.
        const bool ready = finish == K_F64
                               ? (rms < 0.1 * op.max_rms && std::fabs(dE) < 0.1 * op.e_conv &&
                                  std::fabs(prev_dE) < op.e_conv)
                               : (rms < op.max_rms && std::fabs(dE) < 10.0 * op.e_conv);
        if (ready || stalled >= 5) kind = finish;
      }
    }
    FCC_CUDA(cudaEventRecord(ev1, s));
    FCC_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    FCC_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    if (!std::isfinite(Ecc) || !std::isfinite(rms)) { status = FCC_ERR_NAN; }
    if (iter_kind != K_F64) {
      int herr = 0;
      FCC_CUDA(cudaMemcpy(&herr, c->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost));
      if (herr) { status = FCC_ERR_TIMEOUT; }
    }
    if (c->ckpt_every > 0 && ite % c->ckpt_every == 0)
      checkpoint_write(c, c->ckpt_path, cur1, cur2, Ecc, ite, 0);
    if (log && nlog < log_cap) {
      fcc_iter_stats& L = log[nlog];
      L.ite = ite; L.diis = did; L.precision = iter_kind; L.pad = 0;
      L.energy = Ecc; L.dE = dE; L.rms = rms; L.seconds = ms * 1e-3;
    }
    ++nlog;
    ++ite;
    if (status == FCC_ERR_NAN || status == FCC_ERR_TIMEOUT) break;
    if (converged) { conv_final = true; break; }
  }
  // keep the final amplitudes in c->t1 / c->t2
  if (cur1 != c->t1.p) FCC_CUDA(cudaMemcpyAsync(c->t1.p, cur1, sizeof(double) * len1, cudaMemcpyDeviceToDevice, s));
  if (cur2 != c->t2.p) FCC_CUDA(cudaMemcpyAsync(c->t2.p, cur2, sizeof(double) * len2, cudaMemcpyDeviceToDevice, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  c->dvec1.release(); c->dvec2.release(); c->derr1s.release(); c->derr2s.release();
  c->derr1d.release(); c->derr2d.release();
  if (res) {
    res->guessenergy = Eguess;
    res->correlation = Ecc;
    res->energy = Ecc + c->e_ref;
    res->e_conv = dE;
    res->t_conv = rms;
    res->iterations = nlog;
    res->converged = conv_final ? 1 : 0;                                   // :231
  }
  c->have_ccsd = true;
  c->last_ecc = Ecc;
  c->last_iters = nlog;
  c->last_converged = conv_final ? 1 : 0;
  if (c->ckpt_every > 0) checkpoint_write(c, c->ckpt_path, c->t1.p, c->t2.p, Ecc, nlog, conv_final ? 1 : 0);
  return status;
}

}  // namespace fcc
