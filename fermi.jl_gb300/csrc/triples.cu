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
// For a pair i >= j and a run of k <= j, each of the twelve contractions is
// ONE DMMA launch over the whole run: the occupied index k joins the rows or
// columns of the product (k-run views of (ia|bd), (li|jb) or t2), so W[k][a]
// [b][c] for up to 32 k is built by twelve launches per pair instead of
// twelve per triplet, with the index permutations in the operand and output
// strides.  The energy kernel then works on 8 x 8 x 8 sub-cubes (blocks
// A >= B >= C): it stages the six permutations of a sub-cube of W in shared
// memory with loads along W's stride-1 index, forms V from T1 and (ia|jb)
// blocks staged beside them, and reduces in FP64 into per-(k, sub-cube)
// partials that are summed in a fixed order at the end.
#include <cmath>

#include "fcc_ctx.cuh"

namespace fcc {

namespace {

constexpr int EB = 256;          // threads per energy block

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

constexpr int ET = 8;            // sub-cube edge of the energy kernel

struct TileTri {
  int16_t a, b, c, pad;
};

// Energy of the triplets (i, j, k0 + blockIdx.y) on the sub-cube
// tiles[blockIdx.x] (blocks A >= B >= C), from W[kq][a][b][c].
// part[k * ntiles + tile] accumulates over the calls in a fixed order.
__global__ void __launch_bounds__(EB) triples_energy_f64_kernel(const double* __restrict__ W,
                                                                const TileTri* __restrict__ tiles, int ntiles,
                                                                const double* __restrict__ t1,
                                                                const double* __restrict__ ovov,
                                                                const double* __restrict__ eps, int o, int v, int i,
                                                                int j, int k0, double* __restrict__ part) {
  __shared__ double Wt[6][ET][ET][ET + 1];   // W on the six permutations of the sub-cube
  __shared__ double Mjk[3][3][ET][ET + 1];   // (j y|k z) for y in block r1, z in block r2
  __shared__ double Mik[3][3][ET][ET + 1];
  __shared__ double Mij[3][3][ET][ET + 1];
  __shared__ double T1[3][3][ET];            // t1 of i, j, k on block r
  __shared__ double epsv[3][ET];
  __shared__ double red[EB / 32];
  const int kq = blockIdx.y, k = k0 + kq;
  if (i == j && j == k) return;              // weight 2 - d_ij - d_jk = 0
  const TileTri tt = tiles[blockIdx.x];
  const int oa = tt.a * ET, ob = tt.b * ET, oc = tt.c * ET;
  auto org = [&](int r) { return r == 0 ? oa : (r == 1 ? ob : oc); };
  const int64_t v2 = (int64_t)v * v;
  const double* Wk = W + (int64_t)kq * v2 * v;
  // permutation p: roles (rx, ry, rz) of the sub-cube blocks, 2 bits each:
  // (0,1,2) (0,2,1) (1,0,2) (1,2,0) (2,0,1) (2,1,0)
  constexpr uint64_t PRC = (0ull | 1ull << 2 | 2ull << 4) | (0ull | 2ull << 2 | 1ull << 4) << 8 |
                           (1ull | 0ull << 2 | 2ull << 4) << 16 | (1ull | 2ull << 2 | 0ull << 4) << 24 |
                           (2ull | 0ull << 2 | 1ull << 4) << 32 | (2ull | 1ull << 2 | 0ull << 4) << 40;
  auto role = [](int p, int r) { return (int)((PRC >> (8 * p + 2 * r)) & 3); };
  const int t = threadIdx.x;
  // every thread issues all its global loads first, then writes shared memory
  constexpr int NE = 6 * ET * ET * ET / EB;
  constexpr int NM = (9 * ET * ET + EB - 1) / EB;
  double w[NE], mjk[NM], mik[NM], mij[NM];
  const int64_t mstr = (int64_t)o * v;
#pragma unroll
  for (int q = 0; q < NE; ++q) {
    const int e = t + q * EB;
    const int p = e / (ET * ET * ET), r = e % (ET * ET * ET);
    const int x = org(role(p, 0)) + r / (ET * ET), y = org(role(p, 1)) + (r / ET) % ET, z = org(role(p, 2)) + r % ET;
    w[q] = (x < v && y < v && z < v) ? Wk[((int64_t)x * v + y) * v + z] : 0.0;
  }
#pragma unroll
  for (int q = 0; q < NM; ++q) {
    const int e = t + q * EB;
    mjk[q] = mik[q] = mij[q] = 0.0;
    if (e < 9 * ET * ET) {
      const int rr = e / (ET * ET), qq = e % (ET * ET);
      const int Y = org(rr / 3) + qq / ET, Z = org(rr % 3) + qq % ET;
      if (Y < v && Z < v) {
        // ovov[p][y][q][z] = (p y|q z), row stride o*v
        mjk[q] = ovov[((int64_t)j * v + Y) * mstr + (int64_t)k * v + Z];
        mik[q] = ovov[((int64_t)i * v + Y) * mstr + (int64_t)k * v + Z];
        mij[q] = ovov[((int64_t)i * v + Y) * mstr + (int64_t)j * v + Z];
      }
    }
  }
  if (t < 3 * ET) {
    const int r = t / ET, x = t % ET, X = org(r) + x;
    T1[0][r][x] = X < v ? t1[(int64_t)i * v + X] : 0.0;
    T1[1][r][x] = X < v ? t1[(int64_t)j * v + X] : 0.0;
    T1[2][r][x] = X < v ? t1[(int64_t)k * v + X] : 0.0;
    epsv[r][x] = X < v ? eps[o + X] : 0.0;
  }
#pragma unroll
  for (int q = 0; q < NM; ++q) {
    const int e = t + q * EB;
    if (e < 9 * ET * ET) {
      const int rr = e / (ET * ET), qq = e % (ET * ET);
      Mjk[rr / 3][rr % 3][qq / ET][qq % ET] = mjk[q];
      Mik[rr / 3][rr % 3][qq / ET][qq % ET] = mik[q];
      Mij[rr / 3][rr % 3][qq / ET][qq % ET] = mij[q];
    }
  }
#pragma unroll
  for (int q = 0; q < NE; ++q) {
    const int e = t + q * EB;
    const int p = e / (ET * ET * ET), r = e % (ET * ET * ET);
    Wt[p][r / (ET * ET)][(r / ET) % ET][r % ET] = w[q];
  }
  __syncthreads();
  // V(x,y,z) for x in block rx at lx etc.: W + t1_ix (jy|kz) + (ix|kz) t1_jy + (ix|jy) t1_kz  (ijk.jl:116)
  auto V = [&](int rx, int lx, int ry, int ly, int rz, int lz, double wv) -> double {
    return wv + T1[0][rx][lx] * Mjk[ry][rz][ly][lz] + Mik[rx][rz][lx][lz] * T1[1][ry][ly] +
           Mij[rx][ry][lx][ly] * T1[2][rz][lz];
  };
  const double Dijk = eps[i] + eps[j] + eps[k];
  double acc = 0.0;
  for (int e = t; e < ET * ET * ET; e += EB) {
    const int la = e / (ET * ET), lb = (e / ET) % ET, lc = e % ET;
    const int a = oa + la, b = ob + lb, c = oc + lc;
    if (a >= v || b >= v || c >= v || b > a || c > b) continue;
    const double Wabc = Wt[0][la][lb][lc], Wacb = Wt[1][la][lc][lb], Wbac = Wt[2][lb][la][lc];
    const double Wbca = Wt[3][lb][lc][la], Wcab = Wt[4][lc][la][lb], Wcba = Wt[5][lc][lb][la];
    const double Vabc = V(0, la, 1, lb, 2, lc, Wabc), Vacb = V(0, la, 2, lc, 1, lb, Wacb);
    const double Vbac = V(1, lb, 0, la, 2, lc, Wbac), Vbca = V(1, lb, 2, lc, 0, la, Wbca);
    const double Vcab = V(2, lc, 0, la, 1, lb, Wcab), Vcba = V(2, lc, 1, lb, 0, la, Wcba);
    const double X = Wabc * Vabc + Wacb * Vacb + Wbac * Vbac + Wbca * Vbca + Wcab * Vcab + Wcba * Vcba;   // :129
    const double Y = Vabc + Vbca + Vcab;                                                                   // :130
    const double Z = Vacb + Vbac + Vcba;                                                                   // :131
    const double Ef = (Y - 2.0 * Z) * (Wabc + Wbca + Wcab) + (Z - 2.0 * Y) * (Wacb + Wbac + Wcba) + 3.0 * X;
    const double Dd = Dijk - epsv[0][la] - epsv[1][lb] - epsv[2][lc];
    acc += Ef / (Dd * (1.0 + (a == b) + (b == c)));                                                       // :133
  }
  acc = warp_sum(acc);
  if ((t & 31) == 0) red[t >> 5] = acc;
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int q = 0; q < EB / 32; ++q) s += red[q];
    part[(int64_t)k * ntiles + blockIdx.x] += (2.0 - (i == j) - (j == k)) * s;
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

double triples_fp64(fcc_ctx* c, const std::vector<int3>* subset, std::vector<double>* each) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  const int64_t v2 = v * v, v3 = v2 * v, ov2 = o * v2, o2v = o * o * v;
  TView B = rm(c->B.p, {Q, n, n});
  TView Boo = slice(slice(B, 1, 0, o), 2, 0, o);
  TView Bov = slice(slice(B, 1, 0, o), 2, o, v);
  TView Bvv = slice(slice(B, 1, o, v), 2, o, v);
  c->ovvv.alloc(o * v3);
  c->ooov.alloc(o * o2v);
  einsum(1.0, "Qia,Qbd->iabd", Bov, Bvv, 0.0, rm(c->ovvv.p, {o, v, v, v}), s);   // (ia|bd) [i][a][b][d]
  einsum(1.0, "Qli,Qjb->lijb", Boo, Bov, 0.0, rm(c->ooov.p, {o, o, o, v}), s);   // (li|jb) [l][i][j][b]
  // runs of up to KC values of k: W holds KC * v^3 doubles (at most ~2 GB)
  const int64_t KC = std::max<int64_t>(1, std::min<int64_t>(o, (int64_t)(2ll << 30) / (8 * v3)));
  c->Wt.alloc(KC * v3);
  const int nt = (int)((v + ET - 1) / ET);
  std::vector<TileTri> th;
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b <= a; ++b)
      for (int cc = 0; cc <= b; ++cc) th.push_back(TileTri{(int16_t)a, (int16_t)b, (int16_t)cc, 0});
  const int ntiles = (int)th.size();
  DBuf<TileTri> tiles;
  tiles.alloc(ntiles);
  FCC_CUDA(cudaMemcpyAsync(tiles.p, th.data(), sizeof(TileTri) * ntiles, cudaMemcpyHostToDevice, s));
  DBuf<double> part, out;
  part.alloc(o * ntiles);
  out.alloc(1);
  part.zero(s);

  double* ovvv = c->ovvv.p;
  double* ooov = c->ooov.p;
  double* t2 = c->t2.p;
  auto view = [](double* p, std::initializer_list<int64_t> dims, std::initializer_list<int64_t> strides) {
    TView r;
    r.p = p;
    r.rank = (int)dims.size();
    int q = 0;
    for (auto d : dims) r.dim[q++] = d;
    q = 0;
    for (auto st : strides) r.str[q++] = st;
    return r;
  };
  // W[k][a][b][c] for k in [k0, k0 + nk) from the twelve terms of ijk.jl:109-114
  auto build_w = [&](int64_t i, int64_t j, int64_t k0, int64_t nk) {
    TView W = rm(c->Wt.p, {nk, v, v, v});
    auto ov3 = [&](int64_t x) { return view(ovvv + x * v3, {v, v, v}, {v2, v, 1}); };             // (x a|b d)
    TView ov3k = view(ovvv + k0 * v3, {nk, v, v, v}, {v3, v2, v, 1});                              // (k a|b d)
    auto t2pair = [&](int64_t x, int64_t y) { return view(t2 + (x * o + y) * v2, {v, v}, {v, 1}); };
    auto t2pairk = [&](int64_t y) { return view(t2 + (k0 * o + y) * v2, {nk, v, v}, {ov2, v, 1}); };   // t(k,y)
    auto t2row = [&](int64_t x) { return view(t2 + x * ov2, {o, v, v}, {v2, v, 1}); };              // t(x, l)
    TView t2rowk = view(t2 + k0 * ov2, {nk, o, v, v}, {ov2, v2, v, 1});                            // t(k, l)
    auto oo = [&](int64_t x, int64_t y) { return view(ooov + (x * o + y) * v, {o, v}, {o2v, 1}); };   // (l x|y b)
    auto oo_k_y = [&](int64_t y) { return view(ooov + (k0 * o + y) * v, {o, nk, v}, {o2v, o * v, 1}); };   // (l k|y b)
    auto oo_x_k = [&](int64_t x) { return view(ooov + (x * o + k0) * v, {o, nk, v}, {o2v, v, 1}); };       // (l x|k b)
    einsum(1.0, "abd,kcd->kabc", ov3(i), t2pairk(j), 0.0, W, s);     // :109
    einsum(-1.0, "lb,klca->kabc", oo(i, j), t2rowk, 1.0, W, s);
    einsum(1.0, "bad,kcd->kabc", ov3(j), t2pairk(i), 1.0, W, s);     // :110
    einsum(-1.0, "la,klcb->kabc", oo(j, i), t2rowk, 1.0, W, s);
    einsum(1.0, "kcad,bd->kabc", ov3k, t2pair(j, i), 1.0, W, s);     // :111
    einsum(-1.0, "lka,lbc->kabc", oo_k_y(i), t2row(j), 1.0, W, s);
    einsum(1.0, "kcbd,da->kabc", ov3k, t2pair(j, i), 1.0, W, s);     // :112
    einsum(-1.0, "lkb,lac->kabc", oo_k_y(j), t2row(i), 1.0, W, s);
    einsum(1.0, "acd,kdb->kabc", ov3(i), t2pairk(j), 1.0, W, s);     // :113
    einsum(-1.0, "lkc,lba->kabc", oo_x_k(i), t2row(j), 1.0, W, s);
    einsum(1.0, "bcd,kda->kabc", ov3(j), t2pairk(i), 1.0, W, s);     // :114
    einsum(-1.0, "lkc,lab->kabc", oo_x_k(j), t2row(i), 1.0, W, s);
  };
  auto energy = [&](int64_t i, int64_t j, int64_t k0, int64_t nk) {
    const int pe = prof_begin(s);
    dim3 g((unsigned)ntiles, (unsigned)nk);
    triples_energy_f64_kernel<<<g, EB, 0, s>>>(c->Wt.p, tiles.p, ntiles, c->t1.p, c->ovov.p, c->eps.p, (int)o, (int)v,
                                               (int)i, (int)j, (int)k0, part.p);
    FCC_CHECK_LAUNCH();
    prof_end(s, pe, PROF_TRIPLES, (double)nk * (double)v * (v + 1) * (v + 2) / 6.0);
  };
  if (subset) {
    // one triplet at a time, each energy read separately
    each->assign(subset->size(), 0.0);
    for (size_t q = 0; q < subset->size(); ++q) {
      const int3 t = (*subset)[q];
      part.zero(s);
      build_w(t.x, t.y, t.z, 1);
      energy(t.x, t.y, t.z, 1);
      sum_kernel<<<1, 1, 0, s>>>(part.p, (int)(o * ntiles), out.p);
      FCC_CHECK_LAUNCH();
      FCC_CUDA(cudaMemcpyAsync(&(*each)[q], out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    FCC_CUDA(cudaStreamSynchronize(s));
  } else {
    for (int64_t i = 0; i < o; ++i)
      for (int64_t j = 0; j <= i; ++j)
        for (int64_t k0 = 0; k0 <= j; k0 += KC) {
          const int64_t nk = std::min<int64_t>(KC, j + 1 - k0);
          if (i == j && j == k0 && nk == 1) continue;   // i = j = k only: weight 0
          build_w(i, j, k0, nk);
          energy(i, j, k0, nk);
        }
  }
  sum_kernel<<<1, 1, 0, s>>>(part.p, (int)(o * ntiles), out.p);
  FCC_CHECK_LAUNCH();
  double et = 0.0;
  FCC_CUDA(cudaMemcpyAsync(&et, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  c->ovvv.release();
  c->ooov.release();
  c->Wt.release();
  return subset ? 0.0 : et;
}

}  // namespace fcc
