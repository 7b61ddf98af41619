// RCCSD(T) in the mixed form: split-BF16 tensor-core contractions with FP32
// accumulation for W; V, the permutation sums and the quotient by the
// denominator in FP32; the denominators and the energy reduction in FP64.
//
// Same algorithm as the FP64 form (PerturbativeTriples/ijk.jl:20-149),
// arranged for the tensor cores.  For a pair i >= j and a run of k <= j, the
// twelve contractions of ijk.jl:109-114 are three grouped products (one per
// lone virtual index, gemm_t3.cu), written once as G_g[k] over (pair, lone)
// in 8 x 8 x 8 sub-cube blocks (t3_blk):
//   W_ijk(a,b,c) = G0[k](a,b|c) + G1[k](a,c|b) + G2[k](b,c|a).
// The energy kernel works on 8 x 8 x 8 sub-cubes (a-, b-, c-blocks A >= B >= C):
// it stages the sub-blocks of G0, G1, G2 for the six permutations of the
// sub-cube in shared memory with coalesced loads, forms W there, and
// evaluates every a >= b >= c of the sub-cube from shared memory.
//
// Packed split-BF16 operands (rows x K, built once per call):
//   OVA [x][y][z] = (xy|zd)      OVTA[x][y][z] = (xz|yd)        (A side, K = d)
//   P3A [x][y][z] = -t(x,l,y,z)  P3TA[x][y][z] = -t(x,l,z,y)    (A side, K = l)
//   P1B [x][k][c] = t(k,x,c,d)   P2B [x][k][b] = t(x,k,b,d)     (B side, K = d)
//   OORB[y][x][a] = (ly|xa)                                     (B side, K = l)
#include <cmath>
#include <cstring>
#include <vector>

#include "fcc_ctx.cuh"
#include "fcc_t3.cuh"

namespace fcc {

namespace {

constexpr int ET = 8;          // sub-cube edge of the energy kernel
constexpr int ETH = 256;       // threads per energy block

struct TileTri {
  int16_t a, b, c, pad;
};

// x = hi + lo, two floats (hi = x rounded, lo = the rest rounded): ~2^-48 relative
__device__ __forceinline__ float2 split_f2(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
// a + b and its rounding error e (Knuth's TwoSum, no condition on the magnitudes)
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}
// (x.hi + x.lo) - (y.hi + y.lo) rounded to one float
__device__ __forceinline__ float diff_f2(float2 x, float2 y) {
  float e;
  const float s = two_sum(x.x, -y.x, e);
  return __fadd_rn(s, __fadd_rn(e, __fsub_rn(x.y, y.y)));
}

// Energy of the triplets (i, j, k0 + blockIdx.y) on the sub-cube
// tiles[blockIdx.x] (tile blocks A >= B >= C).  part[k * ntiles + tile]
// accumulates over the calls in a fixed order.
__global__ void __launch_bounds__(ETH) triples_energy_tiled_kernel(
    const float* __restrict__ G, int nk, const TileTri* __restrict__ tiles, int ntiles, const float* __restrict__ t1f,
    const float* __restrict__ ovovf, const double* __restrict__ eps, int o, int v, int i, int j, int k0,
    double* __restrict__ part) {
  __shared__ float Wt[6][ET][ET][ET + 1];   // W on the six permutations of the sub-cube
  __shared__ float Mjk[3][3][ET][ET + 1];   // (j y|k z) for y in block r1, z in block r2
  __shared__ float Mik[3][3][ET][ET + 1];
  __shared__ float Mij[3][3][ET][ET + 1];
  __shared__ float T1[3][3][ET];            // t1 of i, j, k on block r
  __shared__ float2 ecf[ET];                // e_c of block C as an unevaluated float sum (hi, lo)
  __shared__ float2 Dabf[ET][ET];           // e_i + e_j + e_k - e_a - e_b likewise
  __shared__ double red[ETH / 32];
  const int kq = blockIdx.y, k = k0 + kq;
  if (i == j && j == k) return;
  const TileTri tt = tiles[blockIdx.x];
  const int oa = tt.a * ET, ob = tt.b * ET, oc = tt.c * ET;
  auto org = [&](int r) { return r == 0 ? oa : (r == 1 ? ob : oc); };
  const int64_t nbk = t3_nb(v), slab = t3_slab(v);
  const float* G0 = G + ((int64_t)0 * nk + kq) * slab;   // (a, b | c), blocked
  const float* G1 = G + ((int64_t)1 * nk + kq) * slab;   // (a, c | b)
  const float* G2 = G + ((int64_t)2 * nk + kq) * slab;   // (b, c | a)
  // permutation p: roles (rx, ry, rz) of the sub-cube blocks, 2 bits each:
  // (0,1,2) (0,2,1) (1,0,2) (1,2,0) (2,0,1) (2,1,0)
  constexpr uint64_t PRC = (0ull | 1ull << 2 | 2ull << 4) | (0ull | 2ull << 2 | 1ull << 4) << 8 |
                           (1ull | 0ull << 2 | 2ull << 4) << 16 | (1ull | 2ull << 2 | 0ull << 4) << 24 |
                           (2ull | 0ull << 2 | 1ull << 4) << 32 | (2ull | 1ull << 2 | 0ull << 4) << 40;
  auto role = [](int p, int r) { return (int)((PRC >> (8 * p + 2 * r)) & 3); };
  const int t = threadIdx.x;

  // ---- stage W = G0[x][y][z] + G1[x][z][y] + G2[y][z][x] and the
  // integral blocks: every thread first issues all its global loads, then
  // writes shared memory, so one global latency covers the whole staging.
  // The block origins are multiples of 8, so each (permutation, group) source
  // is one whole 512-float sub-cube of its G, read in order as 128 float4
  // (element r = hi * 64 + mid * 8 + lo of the sub-cube): thread t reads
  // float4 (t & 127) of the sources q = 0..8, group g = q / 3 and permutation
  // p = 2 (q - 3g) + (t >> 7).  In the sub-cube, G0 runs over (x, y | z),
  // G1 over (x, z | y) and G2 over (y, z | x) as (hi, mid, lo).  Elements
  // past v (v not a multiple of 8: the padding of the blocked layout, inside
  // the slab but never written) are replaced by zeros.
  constexpr int NQ = 18 * ET * ET * ET / 4 / ETH;      // float4 per thread (9)
  constexpr int NM = (9 * ET * ET + ETH - 1) / ETH;    // integral elements per thread
  static_assert(NQ == 9 && ETH == 256, "staging assumes 256 threads");
  float4 gv[NQ];
  float mjk[NM], mik[NM], mij[NM];
  const int64_t mstr = (int64_t)o * v;
  const int r0 = (t & 127) << 2;
  const int shi = r0 >> 6, smid = (r0 >> 3) & 7, slo = r0 & 7;
  const bool edge = (v & 7) != 0;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int g = q / 3, p = 2 * (q - 3 * g) + (t >> 7);
    const int o0 = org(role(p, 0)), o1 = org(role(p, 1)), o2 = org(role(p, 2));
    // sub-cube origin of the source in its own index order (hi, mid, lo)
    const int b0 = g == 2 ? o1 : o0, b1 = g == 0 ? o1 : o2, b2 = g == 0 ? o2 : (g == 1 ? o1 : o0);
    const float* src = (g == 0 ? G0 : (g == 1 ? G1 : G2)) + t3_blk(b0, b1, b2, nbk) + r0;
    float4 x = *reinterpret_cast<const float4*>(src);
    if (edge) {
      const bool ok = b0 + shi < v && b1 + smid < v;
      x.x = ok && b2 + slo < v ? x.x : 0.0f;
      x.y = ok && b2 + slo + 1 < v ? x.y : 0.0f;
      x.z = ok && b2 + slo + 2 < v ? x.z : 0.0f;
      x.w = ok && b2 + slo + 3 < v ? x.w : 0.0f;
    }
    gv[q] = x;
  }
#pragma unroll
  for (int q = 0; q < NM; ++q) {
    const int e = t + q * ETH;
    mjk[q] = mik[q] = mij[q] = 0.0f;
    if (e < 9 * ET * ET) {
      const int rr = e / (ET * ET), qq = e % (ET * ET);
      const int Y = org(rr / 3) + qq / ET, Z = org(rr % 3) + qq % ET;
      if (Y < v && Z < v) {
        // ovovf[p][y][q][z] = (p y|q z), row stride o*v
        mjk[q] = ovovf[((int64_t)j * v + Y) * mstr + (int64_t)k * v + Z];
        mik[q] = ovovf[((int64_t)i * v + Y) * mstr + (int64_t)k * v + Z];
        mij[q] = ovovf[((int64_t)i * v + Y) * mstr + (int64_t)j * v + Z];
      }
    }
  }
  if (t < 3 * ET) {
    const int r = t / ET, x = t % ET, X = org(r) + x;
    T1[0][r][x] = X < v ? t1f[(int64_t)i * v + X] : 0.0f;
    T1[1][r][x] = X < v ? t1f[(int64_t)j * v + X] : 0.0f;
    T1[2][r][x] = X < v ? t1f[(int64_t)k * v + X] : 0.0f;
    if (r == 2) ecf[x] = split_f2(X < v ? eps[o + X] : 0.0);
  }
#pragma unroll
  for (int q = 0; q < NM; ++q) {
    const int e = t + q * ETH;
    if (e < 9 * ET * ET) {
      const int rr = e / (ET * ET), qq = e % (ET * ET);
      Mjk[rr / 3][rr % 3][qq / ET][qq % ET] = mjk[q];
      Mik[rr / 3][rr % 3][qq / ET][qq % ET] = mik[q];
      Mij[rr / 3][rr % 3][qq / ET][qq % ET] = mij[q];
    }
  }
  // G0 element (hi, mid, lo) is W[p][hi][mid][lo]; G1's is W[p][hi][lo][mid]
  // (x, z, y order); G2's is W[p][lo][hi][mid] (y, z, x order)
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int p = 2 * q + (t >> 7);
    Wt[p][shi][smid][slo] = gv[q].x;
    Wt[p][shi][smid][slo + 1] = gv[q].y;
    Wt[p][shi][smid][slo + 2] = gv[q].z;
    Wt[p][shi][smid][slo + 3] = gv[q].w;
  }
  __syncthreads();
#pragma unroll
  for (int q = 3; q < 6; ++q) {
    const int p = 2 * (q - 3) + (t >> 7);
    Wt[p][shi][slo][smid] += gv[q].x;
    Wt[p][shi][slo + 1][smid] += gv[q].y;
    Wt[p][shi][slo + 2][smid] += gv[q].z;
    Wt[p][shi][slo + 3][smid] += gv[q].w;
  }
  __syncthreads();
#pragma unroll
  for (int q = 6; q < 9; ++q) {
    const int p = 2 * (q - 6) + (t >> 7);
    Wt[p][slo][shi][smid] += gv[q].x;
    Wt[p][slo + 1][shi][smid] += gv[q].y;
    Wt[p][slo + 2][shi][smid] += gv[q].z;
    Wt[p][slo + 3][shi][smid] += gv[q].w;
  }
  if (t < ET * ET)
    Dabf[t / ET][t % ET] = split_f2(eps[i] + eps[j] + eps[k] - eps[o + oa + t / ET] - eps[o + ob + t % ET]);
  __syncthreads();

  // V(x,y,z) for x in block rx at lx etc.: W + t1_ix (jy|kz) + (ix|kz) t1_jy + (ix|jy) t1_kz
  auto V = [&](int rx, int lx, int ry, int ly, int rz, int lz, float w) -> float {
    return w + T1[0][rx][lx] * Mjk[ry][rz][ly][lz] + Mik[rx][rz][lx][lz] * T1[1][ry][ly] +
           Mij[rx][ry][lx][ly] * T1[2][rz][lz];
  };
  float accf = 0.0f;   // two (a,b,c) per thread; the reductions over threads and blocks are FP64
  for (int e = t; e < ET * ET * ET; e += ETH) {
    const int la = e / (ET * ET), lb = (e / ET) % ET, lc = e % ET;
    const int a = oa + la, b = ob + lb, c = oc + lc;
    if (a >= v || b >= v || c >= v || b > a || c > b) continue;
    const float Wabc = Wt[0][la][lb][lc], Wacb = Wt[1][la][lc][lb], Wbac = Wt[2][lb][la][lc];
    const float Wbca = Wt[3][lb][lc][la], Wcab = Wt[4][lc][la][lb], Wcba = Wt[5][lc][lb][la];
    const float Vabc = V(0, la, 1, lb, 2, lc, Wabc), Vacb = V(0, la, 2, lc, 1, lb, Wacb);
    const float Vbac = V(1, lb, 0, la, 2, lc, Wbac), Vbca = V(1, lb, 2, lc, 0, la, Wbca);
    const float Vcab = V(2, lc, 0, la, 1, lb, Wcab), Vcba = V(2, lc, 1, lb, 0, la, Wcba);
    const float X = Wabc * Vabc + Wacb * Vacb + Wbac * Vbac + Wbca * Vbca + Wcab * Vcab + Wcba * Vcba;
    const float Y = Vabc + Vbca + Vcab;
    const float Z = Vacb + Vbac + Vcba;
    const float Ef = (Y - 2.0f * Z) * (Wabc + Wbca + Wcab) + (Z - 2.0f * Y) * (Wacb + Wbac + Wcba) + 3.0f * X;
    // denominator from the FP64 orbital energies, carried as float pairs
    // (~2^-48 relative) and rounded once to FP32; the quotient of the FP32 Ef
    // in FP32 (the FP64 pipe is 1/64 rate on this part: FP64 denominators
    // and reductions kept it 35% busy)
    const float D = diff_f2(Dabf[la][lb], ecf[lc]);
    const float wgt = 1.0f + (float)(a == b) + (float)(b == c);
    accf += __fdiv_rn(Ef, D * wgt);
  }
  // warp sum in double-float (TwoSum), then FP64 over warps and blocks
  float sh = accf, sl = 0.0f;
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, sh, off), ol = __shfl_down_sync(0xffffffffu, sl, off);
    float e;
    const float h = two_sum(sh, oh, e);
    sl = __fadd_rn(__fadd_rn(sl, ol), e);
    sh = two_sum(h, sl, sl);
  }
  if ((t & 31) == 0) red[t >> 5] = (double)sh + (double)sl;
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int w = 0; w < ETH / 32; ++w) s += red[w];
    part[(int64_t)k * ntiles + blockIdx.x] += (2.0 - (i == j) - (j == k)) * s;
  }
}

__global__ void to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] = (float)x[t];
}

__global__ void sum_parts_kernel(const double* part, int64_t n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int64_t b = 0; b < n; ++b) s += part[b];
    *out = s;
  }
}

// 3-level row spec for packing: rows (x, y, z) with strides, K with stride.
PackSpec pspec(int64_t d1, int64_t d2, int64_t d3, int64_t s1, int64_t s2, int64_t s3, int64_t K, int64_t ks,
               uint32_t code, double scale = 1.0) {
  PackSpec p;
  p.R = d1 * d2 * d3;
  p.K = K;
  p.Kp = packed_kp(K, SPLIT3.P);
  p.P = SPLIT3.P;
  p.code = code;
  p.scale = scale;
  p.rd2 = d2; p.rd3 = d3; p.rs1 = s1; p.rs2 = s2; p.rs3 = s3;
  p.kd2 = 1; p.kd3 = K; p.ks1 = 0; p.ks2 = 0; p.ks3 = ks;
  return p;
}

}  // namespace

double triples_mixed(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  const int bn = c->t3_bn_override ? c->t3_bn_override : t3_bn((int)v);
  TView B = rm(c->B.p, {Q, n, n});
  TView Boo = slice(slice(B, 1, 0, o), 2, 0, o);
  TView Bov = slice(slice(B, 1, 0, o), 2, o, v);
  TView Bvv = slice(slice(B, 1, o, v), 2, o, v);
  if (!c->dev_err.p) c->dev_err.alloc(1);
  FCC_CUDA(cudaMemsetAsync(c->dev_err.p, 0, sizeof(int), s));
  int* err = c->dev_err.p;
  // (ia|bd) and (li|jb) from the factors by exact-slice products
  DBuf<double> ovvv, ooov;
  ovvv.alloc(o * v * v * v);
  ooov.alloc(o * o * o * v);
  {
    TcScope scope(&c->tc);
    c->tc.enabled = true;
    c->tc.exact = true;
    c->tc.err = err;
    einsum(1.0, "Qia,Qbd->iabd", Bov, Bvv, 0.0, rm(ovvv.p, {o, v, v, v}), s);
    einsum(1.0, "Qli,Qjb->lijb", Boo, Bov, 0.0, rm(ooov.p, {o, o, o, v}), s);
    c->tc.exact = false;
  }
  const int64_t v2 = v * v, v3 = v2 * v;
  const uint32_t CA = SPLIT3.code_a, CB = SPLIT3.code_b;
  const double* t2 = c->t2.p;   // t2[i][j][a][b]: strides o*v2, v2, v, 1
  // ovvv[x][y][z][d] = (xy|zd); ooov[l][y][x][a] = (ly|xa)
  PackSpec sOVA = pspec(o, v, v, v3, v2, v, v, 1, CA);
  PackSpec sOVTA = pspec(o, v, v, v3, v, v2, v, 1, CA);
  PackSpec sP3A = pspec(o, v, v, o * v2, v, 1, o, v2, CA, -1.0);
  PackSpec sP3TA = pspec(o, v, v, o * v2, 1, v, o, v2, CA, -1.0);
  PackSpec sP1B = pspec(o, o, v, v2, o * v2, v, v, 1, CB);
  PackSpec sP2B = pspec(o, o, v, o * v2, v2, v, v, 1, CB);
  PackSpec sOORB = pspec(o, o, v, o * v, v, 1, o, o * o * v, CB);
  const PackSpec* specs[7] = {&sOVA, &sOVTA, &sP3A, &sP3TA, &sP1B, &sP2B, &sOORB};
  const double* srcs[7] = {ovvv.p, ovvv.p, t2, t2, t2, t2, ooov.p};
  DBuf<__nv_bfloat16> packed[7];
  for (int q = 0; q < 7; ++q) {
    packed[q].alloc(specs[q]->R * specs[q]->Kp);
    pack_split(srcs[q], *specs[q], packed[q].p, s);
  }
  ovvv.release();
  ooov.release();

  T3Params P;
  std::memset(&P, 0, sizeof(P));
  for (int q = 0; q < 7; ++q) P.maps[q] = tma_map_bf16(packed[q].p, specs[q]->R, specs[q]->Kp, q < 4 ? 128 : bn);
  enum { OVA = 0, OVTA = 1, P3A = 2, P3TA = 3, P1B = 4, P2B = 5, OORB = 6 };
  enum { SI = 0, SJ = 1, SK = 2 };
  const int16_t kbv = (int16_t)(sOVA.Kp / 64), kbo = (int16_t)(sP3A.Kp / 64);
  auto seg = [&](int amap, int asel, int bmap, int b1, int b2) {
    return T3Seg{(int8_t)amap, (int8_t)asel, (int8_t)bmap, (int8_t)b1, (int8_t)b2, (amap <= OVTA) ? kbv : kbo};
  };
  // group 0: rows (a,b), lone c: :109a (ia|bd)t(kj,cd), :110a (jb|ad)t(ki,cd),
  //          :113b -(li|kc)t(jl,ba), :114b -(lj|kc)t(il,ab)
  P.seg[0][0] = seg(OVA, SI, P1B, SJ, SK);
  P.seg[0][1] = seg(OVTA, SJ, P1B, SI, SK);
  P.seg[0][2] = seg(P3TA, SJ, OORB, SI, SK);
  P.seg[0][3] = seg(P3A, SI, OORB, SJ, SK);
  // group 1: rows (a,c), lone b: :111a (kc|ad)t(ji,bd), :113a (ia|cd)t(kj,db),
  //          :112b -(lk|jb)t(il,ac), :109b -(li|jb)t(kl,ca)
  P.seg[1][0] = seg(OVTA, SK, P1B, SI, SJ);
  P.seg[1][1] = seg(OVA, SI, P2B, SJ, SK);
  P.seg[1][2] = seg(P3A, SI, OORB, SK, SJ);
  P.seg[1][3] = seg(P3TA, SK, OORB, SI, SJ);
  // group 2: rows (b,c), lone a: :112a (kc|bd)t(ji,da), :114a (jb|cd)t(ki,da),
  //          :111b -(lk|ia)t(jl,bc), :110b -(lj|ia)t(kl,cb)
  P.seg[2][0] = seg(OVTA, SK, P1B, SJ, SI);
  P.seg[2][1] = seg(OVA, SJ, P2B, SI, SK);
  P.seg[2][2] = seg(P3A, SJ, OORB, SK, SI);
  P.seg[2][3] = seg(P3TA, SK, OORB, SJ, SI);
  P.o = (int)o;
  P.v = (int)v;
  P.bn = bn;
  P.err = err;

  // sub-cube list of the energy kernel
  const int nt = (int)((v + ET - 1) / ET);
  std::vector<TileTri> th;
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b <= a; ++b)
      for (int cc = 0; cc <= b; ++cc) th.push_back(TileTri{(int16_t)a, (int16_t)b, (int16_t)cc, 0});
  const int ntiles = (int)th.size();
  DBuf<TileTri> tiles;
  tiles.alloc(ntiles);
  FCC_CUDA(cudaMemcpyAsync(tiles.p, th.data(), sizeof(TileTri) * ntiles, cudaMemcpyHostToDevice, s));

  DBuf<float> t1f, ovovf;
  t1f.alloc(o * v);
  ovovf.alloc(o * v * o * v);
  to_f32_kernel<<<152 * 4, 256, 0, s>>>(c->t1.p, t1f.p, o * v);
  FCC_CHECK_LAUNCH();
  to_f32_kernel<<<152 * 16, 256, 0, s>>>(c->ovov.p, ovovf.p, o * v * o * v);
  FCC_CHECK_LAUNCH();
  DBuf<double> part, out;
  part.alloc(o * ntiles);
  out.alloc(1);
  part.zero(s);
  // runs of up to KC values of k per launch (G holds 3 * KC * v^3 FP32, at
  // most ~2 GB); long runs keep the launches large and reuse the i- and
  // j-operands across the run.  Measured (T) at (H2O)8: 32 k 0.308 s, 16 k
  // 0.312 s, 8 k 0.320 s; with the earlier tile order 16 k took 0.318 s and
  // 2 k (G small enough to stay in L2) 0.377 s.
  int64_t KC = std::max<int64_t>(1, std::min<int64_t>(32, (2ll << 30) / (3 * t3_slab(v) * 4)));
  if (c->t3_kc_override > 0) KC = c->t3_kc_override;
  DBuf<float> G;
  G.alloc(3 * KC * t3_slab(v));
  P.G = G.p;
  for (int64_t i = 0; i < o; ++i)
    for (int64_t j = 0; j <= i; ++j)
      for (int64_t k0 = 0; k0 <= j; k0 += KC) {
        const int64_t nk = std::min<int64_t>(KC, j + 1 - k0);
        P.i = (int)i;
        P.j = (int)j;
        P.k0 = (int)k0;
        P.nk = (int)nk;
        gemm_t3(P, s);
        dim3 g((unsigned)ntiles, (unsigned)nk);
        const int pe = prof_begin(s);
        triples_energy_tiled_kernel<<<g, ETH, 0, s>>>(G.p, (int)nk, tiles.p, ntiles, t1f.p, ovovf.p, c->eps.p, (int)o,
                                                      (int)v, (int)i, (int)j, (int)k0, part.p);
        FCC_CHECK_LAUNCH();
        prof_end(s, pe, PROF_TRIPLES, (double)nk * (double)v * (v + 1) * (v + 2) / 6.0);
      }
  sum_parts_kernel<<<1, 1, 0, s>>>(part.p, o * ntiles, out.p);
  FCC_CHECK_LAUNCH();
  double et = 0.0;
  int herr = 0;
  FCC_CUDA(cudaMemcpyAsync(&et, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  FCC_CUDA(cudaStreamSynchronize(s));
  if (herr) fail(FCC_ERR_TIMEOUT, "a tensor-core wait gave up in (T)");
  return et;
}

}  // namespace fcc
