// RCCSD(T) in the mixed form: split-BF16 tensor-core contractions with FP32
// accumulation for W; V and the permutation sums in FP32; the denominators,
// the division and the energy reduction in FP64.
//
// Same algorithm as the FP64 form (PerturbativeTriples/ijk.jl:20-149), batched
// for the tensor cores: for every pair i >= j the intermediates W_k for all
// k <= j are built together, so each of the twelve contractions of
// ijk.jl:109-114 is ONE GEMM whose N (or M) dimension runs over k.  Every
// operand is split and packed once per (T) call into the row layouts the
// GEMMs read with 2-D TMA boxes:
//   OVp[x][y][z][d]   = (xy|zd)         (A and B patterns)
//   OVpT[x][y][z][d]  = (xz|yd)         (B)
//   P1[x][k][c][d]    = t(k,x,c,d)      (B)
//   P2[x][k][b][d]    = t(x,k,b,d)      (A)
//   P3[x][c][a][l]    = t(x,l,c,a)      (A and B)
//   P3T[x][y][z][l]   = t(x,l,z,y)      (B)
//   OOq[x][y][a][l]   = (ly|xa)         (A)
//   OOr[y][x][a][l]   = (ly|xa)         (B)
// and each GEMM's epilogue scatters into W[k][a][b][c] (FP32) with the index
// permutation of its term; every GEMM is oriented so its N index ends in c.
#include <cmath>

#include "fcc_ctx.cuh"

namespace fcc {

namespace {

constexpr int EB = 256;
constexpr int EBLOCKS = 152;

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// Energy of the triplets (i, j, k), k = 0..nk-1, from W[k][a][b][c] (FP32).
// V = W + t1_ia (jb|kc) + (ia|kc) t1_jb + (ia|jb) t1_kc and the six-fold
// permutation sums are FP32 (W itself is an FP32-accumulated split-BF16
// result); the orbital-energy denominators, the division and the reduction
// are FP64.  part[k*gridDim.x + block] accumulates across calls in a fixed
// order.
__global__ void __launch_bounds__(EB) triples_energy_batch_kernel(const float* __restrict__ Wb,
                                                                  const float* __restrict__ t1f,
                                                                  const float* __restrict__ ovovf,
                                                                  const double* __restrict__ eps, int o, int v,
                                                                  int i, int j, int k0, double* part) {
  const int k = k0 + blockIdx.y;
  if (i == j && j == k) return;
  const float* W = Wb + (int64_t)blockIdx.y * v * v * v;
  const int64_t mstr = (int64_t)o * v;
  const float* Mjk = ovovf + ((int64_t)j * v * o + k) * v;
  const float* Mik = ovovf + ((int64_t)i * v * o + k) * v;
  const float* Mij = ovovf + ((int64_t)i * v * o + j) * v;
  const float* t1i = t1f + (int64_t)i * v;
  const float* t1j = t1f + (int64_t)j * v;
  const float* t1k = t1f + (int64_t)k * v;
  auto Wat = [&](int x, int y, int z) -> float { return W[((int64_t)x * v + y) * v + z]; };
  auto Vat = [&](int x, int y, int z, float w) -> float {
    return w + t1i[x] * Mjk[(int64_t)y * mstr + z] + Mik[(int64_t)x * mstr + z] * t1j[y] +
           Mij[(int64_t)x * mstr + y] * t1k[z];
  };
  const double Dijk = eps[i] + eps[j] + eps[k];
  const double* fv = eps + o;
  const int64_t npair = (int64_t)v * (v + 1) / 2;
  double acc = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += (int64_t)gridDim.x * blockDim.x) {
    int a = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while ((int64_t)a * (a + 1) / 2 > p) --a;
    while ((int64_t)(a + 1) * (a + 2) / 2 <= p) ++a;
    const int b = (int)(p - (int64_t)a * (a + 1) / 2);
    const double Dab = Dijk - fv[a] - fv[b];
    for (int c = 0; c <= b; ++c) {
      const float Wabc = Wat(a, b, c), Wacb = Wat(a, c, b), Wbac = Wat(b, a, c);
      const float Wbca = Wat(b, c, a), Wcab = Wat(c, a, b), Wcba = Wat(c, b, a);
      const float Vabc = Vat(a, b, c, Wabc), Vacb = Vat(a, c, b, Wacb), Vbac = Vat(b, a, c, Wbac);
      const float Vbca = Vat(b, c, a, Wbca), Vcab = Vat(c, a, b, Wcab), Vcba = Vat(c, b, a, Wcba);
      const float X = Wabc * Vabc + Wacb * Vacb + Wbac * Vbac + Wbca * Vbca + Wcab * Vcab + Wcba * Vcba;
      const float Y = Vabc + Vbca + Vcab;
      const float Z = Vacb + Vbac + Vcba;
      const float Ef = (Y - 2.0f * Z) * (Wabc + Wbca + Wcab) + (Z - 2.0f * Y) * (Wacb + Wbac + Wcba) + 3.0f * X;
      const double wgt = 1.0 + (a == b) + (b == c);
      acc += (double)Ef / ((Dab - fv[c]) * wgt);
    }
  }
  __shared__ double sm[EB / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < EB / 32; ++w) s += sm[w];
    part[(int64_t)k * gridDim.x + blockIdx.x] += (2.0 - (i == j) - (j == k)) * s;
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

// 3-level row spec helper for packing: rows (x, y, z) with strides, K with stride.
PackSpec pspec(int64_t d1, int64_t d2, int64_t d3, int64_t s1, int64_t s2, int64_t s3, int64_t K, int64_t ks) {
  PackSpec p;
  p.R = d1 * d2 * d3;
  p.K = K;
  p.Kp = packed_kp(K, SPLIT3.P);
  p.P = SPLIT3.P;
  p.code = SPLIT3.code_a;
  p.rd2 = d2; p.rd3 = d3; p.rs1 = s1; p.rs2 = s2; p.rs3 = s3;
  p.kd2 = 1; p.kd3 = K; p.ks1 = 0; p.ks2 = 0; p.ks3 = ks;
  return p;
}

// Epilogue map: m = (m1, m2, m3) and n = (n1, n2, n3) with output strides.
EpiMap emap(int64_t M, int64_t md2, int64_t md3, int64_t ms1, int64_t ms2, int64_t ms3, int64_t N, int64_t nd2,
            int64_t nd3, int64_t ns1, int64_t ns2, int64_t ns3, double alpha, double beta, float* C) {
  EpiMap e;
  e.M = M; e.md2 = md2; e.md3 = md3; e.ms1 = ms1; e.ms2 = ms2; e.ms3 = ms3;
  e.N = N; e.nd2 = nd2; e.nd3 = nd3; e.ns1 = ns1; e.ns2 = ns2; e.ns3 = ns3;
  e.alpha = alpha; e.beta = beta; e.C = C; e.mode = EPI_F32;
  e.work = 0.0;
  return e;
}

}  // namespace

double triples_mixed(fcc_ctx* c) {
  cudaStream_t s = c->stream;
  const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
  TView B = rm(c->B.p, {Q, n, n});
  TView Boo = slice(slice(B, 1, 0, o), 2, 0, o);
  TView Bov = slice(slice(B, 1, 0, o), 2, o, v);
  TView Bvv = slice(slice(B, 1, o, v), 2, o, v);
  // FP64 integrals, then their split-BF16 packed copies
  DBuf<double> ovvv, ooov;
  ovvv.alloc(o * v * v * v);
  ooov.alloc(o * o * o * v);
  einsum(1.0, "Qia,Qbd->iabd", Bov, Bvv, 0.0, rm(ovvv.p, {o, v, v, v}), s);
  einsum(1.0, "Qli,Qjb->lijb", Boo, Bov, 0.0, rm(ooov.p, {o, o, o, v}), s);
  const int64_t v2 = v * v, v3 = v2 * v;
  const int64_t Kv = packed_kp(v, SPLIT3.P), Ko = packed_kp(o, SPLIT3.P);
  auto packA = [&](const double* src, PackSpec ps, __nv_bfloat16* dst) { ps.code = SPLIT3.code_a; pack_split(src, ps, dst, s); };
  auto packB = [&](const double* src, PackSpec ps, __nv_bfloat16* dst) { ps.code = SPLIT3.code_b; pack_split(src, ps, dst, s); };
  DBuf<__nv_bfloat16> OVpA, OVpB, OVpTB, P1, P2A, P3, P3A, P3T, OOq, OOrB;
  PackSpec ps_ov = pspec(o, v, v, v3, v2, v, v, 1);            // OVp[x][y][z]  = (xy|zd)
  PackSpec ps_ovt = pspec(o, v, v, v3, v, v2, v, 1);           // OVpT[x][y][z] = (xz|yd)
  OVpA.alloc(ps_ov.R * Kv); OVpB.alloc(ps_ov.R * Kv); OVpTB.alloc(ps_ovt.R * Kv);
  packA(ovvv.p, ps_ov, OVpA.p);
  packB(ovvv.p, ps_ov, OVpB.p);
  packB(ovvv.p, ps_ovt, OVpTB.p);
  ovvv.release();
  const double* t2 = c->t2.p;   // t2[i][j][a][b]: strides o*v2, v2, v, 1
  PackSpec ps1 = pspec(o, o, v, v2, o * v2, v, v, 1);          // P1[x][k][c]  = t(k,x,c,:)
  PackSpec ps2 = pspec(o, o, v, o * v2, v2, v, v, 1);          // P2[x][k][b]  = t(x,k,b,:)
  PackSpec ps3 = pspec(o, v, v, o * v2, v, 1, o, v2);          // P3[x][c][a]  = t(x,l,c,a) over l
  PackSpec ps3t = pspec(o, v, v, o * v2, 1, v, o, v2);         // P3T[x][y][z] = t(x,l,z,y) over l
  P1.alloc(ps1.R * Kv); P2A.alloc(ps2.R * Kv); P3.alloc(ps3.R * Ko); P3A.alloc(ps3.R * Ko); P3T.alloc(ps3t.R * Ko);
  packB(t2, ps1, P1.p);
  packA(t2, ps2, P2A.p);
  packB(t2, ps3, P3.p);
  packA(t2, ps3, P3A.p);
  packB(t2, ps3t, P3T.p);
  // ooov[l][y][x][a] = (ly|xa): strides l o2v, y o v, x v, a 1
  PackSpec psq = pspec(o, o, v, v, o * v, 1, o, o * o * v);    // OOq[x][y][a]
  PackSpec psr = pspec(o, o, v, o * v, v, 1, o, o * o * v);    // OOr[y][x][a]
  OOq.alloc(psq.R * Ko); OOrB.alloc(psr.R * Ko);
  packA(ooov.p, psq, OOq.p);
  packB(ooov.p, psr, OOrB.p);
  ooov.release();

  DBuf<float> Wb, t1f, ovovf;
  Wb.alloc(std::max<int64_t>(1, std::min<int64_t>(o, (96ll << 20) / (v3 * 4))) * v3);
  t1f.alloc(o * v);
  ovovf.alloc(o * v * o * v);
  to_f32_kernel<<<152 * 4, 256, 0, s>>>(c->t1.p, t1f.p, o * v);
  FCC_CHECK_LAUNCH();
  to_f32_kernel<<<152 * 16, 256, 0, s>>>(c->ovov.p, ovovf.p, o * v * o * v);
  FCC_CHECK_LAUNCH();
  DBuf<double> part, out;
  part.alloc(o * EBLOCKS);
  out.alloc(1);
  part.zero(s);
  if (!c->dev_err.p) c->dev_err.alloc(1);
  FCC_CUDA(cudaMemsetAsync(c->dev_err.p, 0, sizeof(int), s));
  int* err = c->dev_err.p;
  const int64_t Rov = o * v2, Rp = o * o * v, Rp3 = o * v2;
  // k is processed in chunks whose W (FP32) fits comfortably in L2, so the
  // twelve read-modify-write epilogues and the energy pass hit L2
  const int64_t KC = std::max<int64_t>(1, std::min<int64_t>(o, (96ll << 20) / (v3 * 4)));
  float* W = Wb.p;
  for (int64_t i = 0; i < o; ++i)
    for (int64_t j = 0; j <= i; ++j)
      for (int64_t k0 = 0; k0 <= j; k0 += KC) {
        const int64_t nk = std::min<int64_t>(KC, j + 1 - k0);
        // W[k-k0][a][b][c]: strides v3, v2, v, 1.  Operands are oriented so the
        // GEMM's N index ends in c (stride 1): coalesced epilogue stores.
        // :109  (ia|bd) t(k,j,c,d)  -  (li|jb) t(k,l,c,a)
        gemm_bf16x3(OVpA.p, Rov, i * v2, P1.p, Rp, (j * o + k0) * v, Kv,
                    emap(v2, v, v, 0, v2, v, nk * v, nk, v, 0, v3, 1, 1.0, 0.0, W), err, s);
        gemm_bf16x3(OOq.p, Rp, (j * o + i) * v, P3T.p, Rp3, k0 * v2, Ko,
                    emap(v, 1, v, 0, 0, v, nk * v2, v, v, v3, v2, 1, -1.0, 1.0, W), err, s);
        // :110  (jb|ad) t(k,i,c,d)  -  (lj|ia) t(k,l,c,b)
        gemm_bf16x3(OVpA.p, Rov, j * v2, P1.p, Rp, (i * o + k0) * v, Kv,
                    emap(v2, v, v, 0, v, v2, nk * v, nk, v, 0, v3, 1, 1.0, 1.0, W), err, s);
        gemm_bf16x3(OOq.p, Rp, (i * o + j) * v, P3T.p, Rp3, k0 * v2, Ko,
                    emap(v, 1, v, 0, 0, v2, nk * v2, v, v, v3, v, 1, -1.0, 1.0, W), err, s);
        // :111  (kc|ad) t(j,i,b,d)  -  (lk|ia) t(j,l,b,c)
        gemm_bf16x3(P2A.p, Rp, (j * o + i) * v, OVpTB.p, Rov, k0 * v2, Kv,
                    emap(v, 1, v, 0, 0, v, nk * v2, v, v, v3, v2, 1, 1.0, 1.0, W), err, s);
        gemm_bf16x3(OOq.p, Rp, (i * o + k0) * v, P3.p, Rp3, j * v2, Ko,
                    emap(nk * v, nk, v, 0, v3, v2, v2, v, v, 0, v, 1, -1.0, 1.0, W), err, s);
        // :112  (kc|bd) t(j,i,d,a)  -  (lk|jb) t(i,l,a,c)
        gemm_bf16x3(P2A.p, Rp, (i * o + j) * v, OVpTB.p, Rov, k0 * v2, Kv,
                    emap(v, 1, v, 0, 0, v2, nk * v2, v, v, v3, v, 1, 1.0, 1.0, W), err, s);
        gemm_bf16x3(OOq.p, Rp, (j * o + k0) * v, P3.p, Rp3, i * v2, Ko,
                    emap(nk * v, nk, v, 0, v3, v, v2, v, v, 0, v2, 1, -1.0, 1.0, W), err, s);
        // :113  (ia|cd) t(k,j,d,b)  -  (li|kc) t(j,l,b,a)
        gemm_bf16x3(P2A.p, Rp, (j * o + k0) * v, OVpB.p, Rov, i * v2, Kv,
                    emap(nk * v, nk, v, 0, v3, v, v2, v, v, 0, v2, 1, 1.0, 1.0, W), err, s);
        gemm_bf16x3(P3A.p, Rp3, j * v2, OOrB.p, Rp, (i * o + k0) * v, Ko,
                    emap(v2, v, v, 0, v, v2, nk * v, nk, v, 0, v3, 1, -1.0, 1.0, W), err, s);
        // :114  (jb|cd) t(k,i,d,a)  -  (lj|kc) t(i,l,a,b)
        gemm_bf16x3(P2A.p, Rp, (i * o + k0) * v, OVpB.p, Rov, j * v2, Kv,
                    emap(nk * v, nk, v, 0, v3, v2, v2, v, v, 0, v, 1, 1.0, 1.0, W), err, s);
        gemm_bf16x3(P3A.p, Rp3, i * v2, OOrB.p, Rp, (j * o + k0) * v, Ko,
                    emap(v2, v, v, 0, v2, v, nk * v, nk, v, 0, v3, 1, -1.0, 1.0, W), err, s);
        dim3 g(EBLOCKS, (unsigned)nk);
        const int pe = prof_begin(s);
        triples_energy_batch_kernel<<<g, EB, 0, s>>>(W, t1f.p, ovovf.p, c->eps.p, (int)o, (int)v, (int)i, (int)j,
                                                     (int)k0, part.p);
        FCC_CHECK_LAUNCH();
        prof_end(s, pe, PROF_TRIPLES, (double)nk * (double)v * (v + 1) * (v + 2) / 6.0);
      }
  sum_parts_kernel<<<1, 1, 0, s>>>(part.p, o * EBLOCKS, out.p);
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
