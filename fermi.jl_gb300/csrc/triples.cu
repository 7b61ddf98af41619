// RCCSD(T) perturbative triples on one GPU, FP64 form.
//
// Algorithm: Fermi.jl's default (T), src/Methods/CoupledCluster/
// PerturbativeTriples/ijk.jl:20-149.  For every occupied triplet i >= j >= k
// the v^3 intermediate W is the sum of the twelve contractions of
// ijk.jl:109-114 (six over a virtual index d, six over an occupied index l),
// V = W + the three T1 x (ia|jb) products of ijk.jl:116, and the energy is the
// six-fold permutation sum of ijk.jl:121-137 with weight
// (2 - d_ij - d_jk) / (D_ijkabc (1 + d_ab + d_bc)) over a >= b >= c.
//
// W is built by the DMMA contraction kernel (twelve launches per triplet,
// index permutations folded into the operand strides); the energy kernel
// forms V on the fly from W, T1 and (ia|jb) and reduces in FP64 into
// per-block partials that are summed in a fixed order at the end.
#include <cmath>

#include "fcc_ctx.cuh"

namespace fcc {

namespace {

constexpr int EB = 256;          // threads per energy block
constexpr int EBLOCKS = 304;     // fixed grid (152 SMs x 2) for a deterministic sum

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// V[x,y,z] for the current triplet from W and the T1 / (ia|jb) products.
struct TripCtx {
  const double* W;
  const double* t1i; const double* t1j; const double* t1k;   // t1[i,:] etc.
  const double* Mjk; const double* Mik; const double* Mij;   // (j x|k y) etc. as v x v with row stride
  int64_t mstr;                                              // stride of the first virtual index
  int v;
};

__device__ __forceinline__ double Wat(const TripCtx& t, int x, int y, int z) {
  return t.W[((int64_t)x * t.v + y) * t.v + z];
}
__device__ __forceinline__ double Vat(const TripCtx& t, int x, int y, int z) {
  // V[a,b,c] = W[a,b,c] + t1_ia (jb|kc) + (ia|kc) t1_jb + (ia|jb) t1_kc
  return Wat(t, x, y, z) + t.t1i[x] * t.Mjk[(int64_t)y * t.mstr + z] + t.Mik[(int64_t)x * t.mstr + z] * t.t1j[y] +
         t.Mij[(int64_t)x * t.mstr + y] * t.t1k[z];
}

__global__ void __launch_bounds__(EB) triples_energy_kernel(TripCtx t, const double* __restrict__ eps, int o,
                                                            int i, int j, int k, double* part) {
  const int v = t.v;
  const int64_t npair = (int64_t)v * (v + 1) / 2;
  const double Dijk = eps[i] + eps[j] + eps[k];
  const double* fv = eps + o;
  double acc = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += (int64_t)gridDim.x * blockDim.x) {
    int a = (int)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
    while ((int64_t)a * (a + 1) / 2 > p) --a;
    while ((int64_t)(a + 1) * (a + 2) / 2 <= p) ++a;
    int b = (int)(p - (int64_t)a * (a + 1) / 2);
    const double Dab = Dijk - fv[a] - fv[b];
    for (int c = 0; c <= b; ++c) {
      double Wabc = Wat(t, a, b, c), Wacb = Wat(t, a, c, b), Wbac = Wat(t, b, a, c);
      double Wbca = Wat(t, b, c, a), Wcab = Wat(t, c, a, b), Wcba = Wat(t, c, b, a);
      double Vabc = Vat(t, a, b, c), Vacb = Vat(t, a, c, b), Vbac = Vat(t, b, a, c);
      double Vbca = Vat(t, b, c, a), Vcab = Vat(t, c, a, b), Vcba = Vat(t, c, b, a);
      double X = Wabc * Vabc + Wacb * Vacb + Wbac * Vbac + Wbca * Vbca + Wcab * Vcab + Wcba * Vcba;
      double Y = Vabc + Vbca + Vcab;
      double Z = Vacb + Vbac + Vcba;
      double Ef = (Y - 2 * Z) * (Wabc + Wbca + Wcab) + (Z - 2 * Y) * (Wacb + Wbac + Wcba) + 3 * X;
      double Dd = Dab - fv[c];
      double w = 1.0 + (a == b) + (b == c);
      acc += Ef / (Dd * w);
    }
  }
  __shared__ double sm[EB / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < EB / 32; ++w) s += sm[w];
    double wt = 2.0 - (i == j) - (j == k);
    part[blockIdx.x] += wt * s;
  }
}

__global__ void sum_kernel(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < n; ++b) s += part[b];
    *out = s;
  }
}

}  // namespace

double triples_fp64(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  TView B = rm(c->B.p, {Q, n, n});
  TView Boo = slice(slice(B, 1, 0, o), 2, 0, o);
  TView Bov = slice(slice(B, 1, 0, o), 2, o, v);
  TView Bvv = slice(slice(B, 1, o, v), 2, o, v);
  c->ovvv.alloc(o * v * v * v);
  c->ooov.alloc(o * o * o * v);
  c->Wt.alloc(v * v * v);
  TView ovvv = rm(c->ovvv.p, {o, v, v, v});   // (ia|bd) [i][a][b][d]
  TView ooov = rm(c->ooov.p, {o, o, o, v});   // (li|jb) [l][i][j][b]
  einsum(1.0, "Qia,Qbd->iabd", Bov, Bvv, 0.0, ovvv, s);
  einsum(1.0, "Qli,Qjb->lijb", Boo, Bov, 0.0, ooov, s);
  TView t2 = rm(c->t2.p, {o, o, v, v});
  TView W = rm(c->Wt.p, {v, v, v});
  DBuf<double> part, out;
  part.alloc(EBLOCKS);
  out.alloc(1);
  part.zero(s);

  auto ov3 = [&](int64_t i) {  // ovvv[i] as (x, y, d)
    TView r; r.p = c->ovvv.p + i * v * v * v; r.rank = 3;
    r.dim[0] = v; r.dim[1] = v; r.dim[2] = v; r.str[0] = v * v; r.str[1] = v; r.str[2] = 1;
    return r;
  };
  auto t2pair = [&](int64_t i, int64_t j) {  // t2[i][j] as (x, y)
    TView r; r.p = c->t2.p + (i * o + j) * v * v; r.rank = 2;
    r.dim[0] = v; r.dim[1] = v; r.str[0] = v; r.str[1] = 1;
    return r;
  };
  auto t2row = [&](int64_t i) {  // t2[i] as (l, x, y)
    TView r; r.p = c->t2.p + i * o * v * v; r.rank = 3;
    r.dim[0] = o; r.dim[1] = v; r.dim[2] = v; r.str[0] = v * v; r.str[1] = v; r.str[2] = 1;
    return r;
  };
  auto oo = [&](int64_t x, int64_t y) {  // ooov[:, x, y, :] as (l, b)
    TView r; r.p = c->ooov.p + (x * o + y) * v; r.rank = 2;
    r.dim[0] = o; r.dim[1] = v; r.str[0] = o * o * v; r.str[1] = 1;
    return r;
  };
  (void)t2;
  for (int64_t i = 0; i < o; ++i)
    for (int64_t j = 0; j <= i; ++j)
      for (int64_t k = 0; k <= j; ++k) {
        if (i == j && j == k) continue;   // weight 2 - d_ij - d_jk = 0
        einsum(1.0, "abd,cd->abc", ov3(i), t2pair(k, j), 0.0, W, s);     // :109
        einsum(-1.0, "lb,lca->abc", oo(i, j), t2row(k), 1.0, W, s);
        einsum(1.0, "bad,cd->abc", ov3(j), t2pair(k, i), 1.0, W, s);     // :110
        einsum(-1.0, "la,lcb->abc", oo(j, i), t2row(k), 1.0, W, s);
        einsum(1.0, "cad,bd->abc", ov3(k), t2pair(j, i), 1.0, W, s);     // :111
        einsum(-1.0, "la,lbc->abc", oo(k, i), t2row(j), 1.0, W, s);
        einsum(1.0, "cbd,da->abc", ov3(k), t2pair(j, i), 1.0, W, s);     // :112
        einsum(-1.0, "lb,lac->abc", oo(k, j), t2row(i), 1.0, W, s);
        einsum(1.0, "acd,db->abc", ov3(i), t2pair(k, j), 1.0, W, s);     // :113
        einsum(-1.0, "lc,lba->abc", oo(i, k), t2row(j), 1.0, W, s);
        einsum(1.0, "bcd,da->abc", ov3(j), t2pair(k, i), 1.0, W, s);     // :114
        einsum(-1.0, "lc,lab->abc", oo(j, k), t2row(i), 1.0, W, s);
        TripCtx t;
        t.W = c->Wt.p;
        t.t1i = c->t1.p + i * v; t.t1j = c->t1.p + j * v; t.t1k = c->t1.p + k * v;
        // ovov[x][a][y][b] = (xa|yb): M_xy[a][b] has row stride o*v
        t.Mjk = c->ovov.p + (j * v * o + k) * v;
        t.Mik = c->ovov.p + (i * v * o + k) * v;
        t.Mij = c->ovov.p + (i * v * o + j) * v;
        t.mstr = o * v;
        t.v = (int)v;
        triples_energy_kernel<<<EBLOCKS, EB, 0, s>>>(t, c->eps.p, (int)o, (int)i, (int)j, (int)k, part.p);
        FCC_CHECK_LAUNCH();
      }
  sum_kernel<<<1, 1, 0, s>>>(part.p, EBLOCKS, out.p);
  FCC_CHECK_LAUNCH();
  double et = 0.0;
  FCC_CUDA(cudaMemcpyAsync(&et, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  c->ovvv.release();
  c->ooov.release();
  c->Wt.release();
  return et;
}

}  // namespace fcc
