// Exact-slice BF16 tensor-core contraction (the Ozaki scheme) for GB300.
//
// C = alpha * A.B^T + beta * C for FP64 operands, evaluated from signed 6-bit
// digit slices of A and B (see fcc_tc.cuh).  Every digit is an integer
// |d| <= 64, exact in BF16; every product of two digits is an integer of at
// most 2^12, so a run of 2048 products accumulated by tcgen05.mma in FP32
// stays an exact integer (|sum| <= 2^23).  The kernel therefore closes an
// accumulation chunk every 32 k-blocks (or at the end of a weight group), and
// the epilogue warps add the chunk, times its weight 2^(-6g) (exact), into a
// double-FP32 (hi + lo, ~2^-48 relative) running sum held in TMEM.  Two TMEM
// accumulators alternate, so the MMA thread fills one while the epilogue
// drains the other.  The final epilogue converts hi and lo to FP64 with the
// row and column scales applied by integer exponent arithmetic (the FP64 pipe
// is 1/64 rate) and stores or reduces (red.add) into C.
//
// TMEM columns (128 x 512 x 32-bit): [0,128) and [128,256) chunk
// accumulators, [256,384) hi and [384,512) lo words of the running sums.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "fcc_tc.cuh"
#include "fcc_tcgen05.cuh"

namespace fcc {

namespace {

using namespace tc5;

constexpr int OZ_BM = 128;
constexpr int OZ_BN = 128;
constexpr int OZ_BK = 64;
constexpr int OZ_STAGES = 6;
constexpr int OZ_THREADS = 192;      // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int OZ_BITS = 6;           // bits per digit slice
constexpr int OZ_CH = 32;            // k-blocks per exact FP32 chunk: 2048 products of at most 64*64, |sum| <= 2^23
constexpr int OZ_MAXPAIRS = 40;
constexpr int OZ_A_BYTES = OZ_BM * OZ_BK * 2;
constexpr int OZ_B_BYTES = OZ_BN * OZ_BK * 2;
constexpr int OZ_STAGE_BYTES = OZ_A_BYTES + OZ_B_BYTES;
// the final epilogue's 32 x 32 FP64 transpose tile per epilogue warp, beside
// the operand ring (a persistent CTA is already loading its next unit)
constexpr int OZ_TILE_BYTES = 4 * 32 * 33 * 8;
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE_BYTES + OZ_TILE_BYTES + 1024;
constexpr int OZ_COL_LO = 256, OZ_COL_HI = 384;

// Slice pairs in the order of the k loop: by weight group g = sa + sb + 2,
// then by sa; next[p] = first pair of the following group.
struct OzPairs {
  int n;
  int8_t sa[OZ_MAXPAIRS], sb[OZ_MAXPAIRS], g[OZ_MAXPAIRS];
  int16_t next[OZ_MAXPAIRS];
};

OzPairs make_pairs(int G) {
  OzPairs p;
  std::memset(&p, 0, sizeof(p));
  const int S = G - 1;
  for (int g = 2; g <= G; ++g) {
    const int first = p.n;
    for (int a = 1; a < g; ++a) {
      const int b = g - a;
      if (a > S || b > S) continue;
      p.sa[p.n] = (int8_t)(a - 1);
      p.sb[p.n] = (int8_t)(b - 1);
      p.g[p.n] = (int8_t)g;
      ++p.n;
    }
    for (int q = first; q < p.n; ++q) p.next[q] = (int16_t)p.n;
  }
  return p;
}

// end of the chunk that starts at step st (steps pair-major, nkb k-blocks per
// pair): at most OZ_CH steps, never across a weight group or the end st1
__device__ __forceinline__ int oz_chunk_end(const OzPairs& pr, int nkb, int st, int st1) {
  const int gend = (int)pr.next[st / nkb] * nkb;
  return min(min(st + OZ_CH, gend), st1);
}

// 2^e as a double (0 below the normal range)
__device__ __forceinline__ double oz_pow2(int e) {
  if (e < -1022) return 0.0;
  if (e > 1023) e = 1023;
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// frexp-style exponent of the row scale from the stored biased exponent
__device__ __forceinline__ int oz_row_exp(int be) { return be ? be - 1022 : 0; }

// hi + lo += v in double-FP32 (TwoSum, then renormalisation)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  const float l = __fadd_rn(lo, err);
  const float h = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(h, s));
  hi = h;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

// Work unit u of the persistent grid: output tile grouped_tile(u % tiles)
// over the K range u / tiles (k-blocks [kb0, kb0 + nku)), all slice pairs;
// the unit's steps are pair-major, st = p * nku + (kb - kb0).  Units running
// at the same time share one K range, so the operand panels they stream stay
// in L2 across the slice pairs that reuse them.
struct OzUnit {
  int64_t m0, n0;
  int kb0, nku;
};
__device__ __forceinline__ OzUnit oz_unit(int64_t u, int64_t tm, int64_t tn, int nkb, int kper) {
  const int64_t tiles = tm * tn;
  int64_t mt, nt;
  grouped_tile(u % tiles, tm, tn, mt, nt);
  const int z = (int)(u / tiles);
  OzUnit r;
  r.m0 = mt * OZ_BM;
  r.n0 = nt * OZ_BN;
  r.kb0 = z * kper;
  r.nku = min(nkb, r.kb0 + kper) - r.kb0;
  return r;
}

// Persistent: CTA b processes units b, b + gridDim.x, ...  The TMA ring and
// the two chunk accumulators run on across units, so the loads and the MMAs
// of a unit's first chunks overlap the previous unit's final epilogue (which
// reads the running sums; only the epilogue warps touch those, in order).
__global__ void __launch_bounds__(OZ_THREADS, 1)
    gemm_oz_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int nkb,
                   int kpad, const __grid_constant__ OzPairs pr, int kper, int64_t tm, int64_t tn,
                   int64_t units, const int* __restrict__ exA, const int* __restrict__ exB, int G, EpiMap ep,
                   int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[OZ_STAGES];
  __shared__ __align__(8) uint64_t empty_bar[OZ_STAGES];
  __shared__ __align__(8) uint64_t accf_bar[2];   // chunk accumulator b is complete
  __shared__ __align__(8) uint64_t acce_bar[2];   // chunk accumulator b is drained
  __shared__ __align__(8) uint64_t done_bar;      // every issued MMA has completed
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_flag;

  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + OZ_STAGES * OZ_A_BYTES;
  double* stile = reinterpret_cast<double*>(smem + OZ_STAGES * OZ_STAGE_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&accf_bar[b]), 1);
      mbar_init(smem_u32(&acce_bar[b]), 4);   // one arrival per epilogue warp
    }
    mbar_init(smem_u32(&done_bar), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_holder;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int it = 0;
    bool stop = false;
    for (int64_t u = blockIdx.x; u < units && !stop; u += gridDim.x) {
      const OzUnit un = oz_unit(u, tm, tn, nkb, kper);
      const int nst = pr.n * un.nku;
      for (int st = 0; st < nst; ++st, ++it) {
        const int s = it % OZ_STAGES;
        const uint32_t ph = (it / OZ_STAGES) & 1;
        if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1)) { atomicExch(&abort_flag, 1); stop = true; break; }
        if (*(volatile int*)&abort_flag) { stop = true; break; }
        const int p = st / un.nku, kb = un.kb0 + (st - p * un.nku);
        const uint32_t fb = smem_u32(&full_bar[s]);
        mbar_expect_tx(fb, OZ_STAGE_BYTES);
        tma_load_2d(smem_u32(sA + s * OZ_A_BYTES), &tmA, (int)pr.sa[p] * kpad + kb * OZ_BK, (int32_t)un.m0, fb);
        tma_load_2d(smem_u32(sB + s * OZ_B_BYTES), &tmB, (int)pr.sb[p] * kpad + kb * OZ_BK, (int32_t)un.n0, fb);
      }
    }
    // on an abort, wait (bounded) for the loads still in flight before the
    // shared memory can be released
    if (*(volatile int*)&abort_flag) {
      for (int j = max(0, it - OZ_STAGES); j < it; ++j)
        (void)mbar_wait(smem_u32(&full_bar[j % OZ_STAGES]), (j / OZ_STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = idesc_bf16(OZ_BM, OZ_BN);
    int it = 0, chunk = 0;
    bool ok = true;
    for (int64_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
      const OzUnit un = oz_unit(u, tm, tn, nkb, kper);
      const int nst = pr.n * un.nku;
      for (int st = 0; st < nst && ok;) {
        const int ce = oz_chunk_end(pr, un.nku, st, nst);
        const int b = chunk & 1;
        if (!mbar_wait(smem_u32(&acce_bar[b]), ((chunk >> 1) & 1) ^ 1)) { atomicExch(&abort_flag, 1); ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dcol = tmem + (uint32_t)(b * OZ_BN);
        for (int x = st; x < ce; ++x, ++it) {
          const int s = it % OZ_STAGES;
          const uint32_t ph = (it / OZ_STAGES) & 1;
          if (!mbar_wait(smem_u32(&full_bar[s]), ph)) { atomicExch(&abort_flag, 1); ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t ad = sw128_desc(smem_u32(sA + s * OZ_A_BYTES));
          const uint64_t bd = sw128_desc(smem_u32(sB + s * OZ_B_BYTES));
#pragma unroll
          for (int kk = 0; kk < OZ_BK / 16; ++kk) {
            const uint32_t acc = (x > st || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
                "l"(ad + (uint64_t)(2 * kk)), "l"(bd + (uint64_t)(2 * kk)), "r"(idesc), "r"(acc)
                : "memory");
          }
          tc_commit(smem_u32(&empty_bar[s]));
        }
        if (!ok) break;
        tc_commit(smem_u32(&accf_bar[b]));
        st = ce;
        ++chunk;
      }
    }
    tc_commit(smem_u32(&done_bar));
  } else if (warp >= 2) {
    // ---------------- epilogue warps: rows q*32 .. q*32+31 of each tile
    const int q = warp & 3;
    const uint32_t lanebase = tmem + ((uint32_t)(q * 32) << 16);
    double (*tile)[33] = reinterpret_cast<double (*)[33]>(stile + q * 32 * 33);
    bool ok = true;
    int chunk = 0;   // over all units: the accumulator and its barrier phase
    // alpha = +-2^ka folds into the exponent arithmetic; otherwise one FP64 multiply
    const unsigned long long ab = (unsigned long long)__double_as_longlong(ep.alpha);
    const bool apow2 = (ab & ((1ull << 52) - 1)) == 0 && ((ab >> 52) & 0x7FF) != 0;
    const int ka = apow2 ? (int)((ab >> 52) & 0x7FF) - 1023 : 0;
    const bool aneg = apow2 && (ab >> 63);
    for (int64_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
      const OzUnit un = oz_unit(u, tm, tn, nkb, kper);
      const int nst = pr.n * un.nku;
      int uchunk = 0;  // chunks of this unit: the first one starts the running sums
      for (int st = 0; st < nst;) {
        const int ce = oz_chunk_end(pr, un.nku, st, nst);
        const int g = pr.g[st / un.nku];
        const int b = chunk & 1;
        ok = mbar_wait(smem_u32(&accf_bar[b]), (chunk >> 1) & 1);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok || __any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) { atomicExch(&abort_flag, 1); ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // weight of the group, 2^(-6g), exact in FP32
        const float wg = __int_as_float((127 - OZ_BITS * g) << 23);
#pragma unroll 1
        for (int c0 = 0; c0 < OZ_BN; c0 += 32) {
          uint32_t acc[32], hi[32], lo[32];
          tmem_ld32(lanebase + (uint32_t)(b * OZ_BN + c0), acc);
          if (uchunk > 0) {
            tmem_ld32(lanebase + (uint32_t)(OZ_COL_HI + c0), hi);
            tmem_ld32(lanebase + (uint32_t)(OZ_COL_LO + c0), lo);
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            // the chunk sum is an exact integer below 2^22; times 2^(-6g) exact
            const float v = __fmul_rn(__uint_as_float(acc[jj]), wg);
            float h = uchunk > 0 ? __uint_as_float(hi[jj]) : 0.0f;
            float l = uchunk > 0 ? __uint_as_float(lo[jj]) : 0.0f;
            ff_add(h, l, v);
            hi[jj] = __float_as_uint(h);
            lo[jj] = __float_as_uint(l);
          }
          tmem_st32(lanebase + (uint32_t)(OZ_COL_HI + c0), hi);
          tmem_st32(lanebase + (uint32_t)(OZ_COL_LO + c0), lo);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&acce_bar[b]));
        st = ce;
        ++chunk;
        ++uchunk;
      }
      if (!ok || uchunk == 0) break;
      // ---- final epilogue of the unit: the running sums, scaled, to C (the
      // unit's last chunk barrier covered every MMA of the unit; the sums were
      // written by this warp, whose stores have completed)
      const int row = q * 32 + lane;
      const int64_t m = un.m0 + row;
      int64_t crow = 0;
      int erow = 0;
      if (m < ep.M) {
        int64_t m3 = m % ep.md3, r = m / ep.md3;
        int64_t m2 = r % ep.md2, m1 = r / ep.md2;
        crow = m1 * ep.ms1 + m2 * ep.ms2 + m3 * ep.ms3;
        erow = oz_row_exp(exA[m]);
      }
#pragma unroll 1
      for (int c0 = 0; c0 < OZ_BN; c0 += 32) {
        if (un.n0 + c0 >= ep.N) break;
        uint32_t hi[32], lo[32];
        tmem_ld32(lanebase + (uint32_t)(OZ_COL_HI + c0), hi);
        tmem_ld32(lanebase + (uint32_t)(OZ_COL_LO + c0), lo);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // this lane's column exponent, broadcast per column below
        const int64_t nl = un.n0 + c0 + lane;
        const int ecl = nl < ep.N ? oz_row_exp(exB[nl]) : 0;
        __syncwarp();
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const int e = erow + __shfl_sync(0xffffffffu, ecl, jj) + ka;
          tile[lane][jj] = f32_to_f64_scaled(__uint_as_float(hi[jj]), e, aneg) +
                           f32_to_f64_scaled(__uint_as_float(lo[jj]), e, aneg);
        }
        __syncwarp();
        const int64_t n = un.n0 + c0 + lane;
        const bool nok = n < ep.N;
        int64_t coff = 0;
        if (nok) {
          int64_t n3 = n % ep.nd3, rr = n / ep.nd3;
          int64_t n2 = rr % ep.nd2, n1 = rr / ep.nd2;
          coff = n1 * ep.ns1 + n2 * ep.ns2 + n3 * ep.ns3;
        }
#pragma unroll
        for (int jr = 0; jr < 32; ++jr) {
          const int64_t roff = __shfl_sync(0xffffffffu, crow, jr);
          const int64_t mm = un.m0 + q * 32 + jr;
          if (mm >= ep.M || !nok) continue;
          double val = tile[jr][lane];
          if (!apow2) val *= ep.alpha;
          double* dst = static_cast<double*>(ep.C) + roff + coff;
          if (ep.atomic) atomicAdd(dst, val);
          else *dst = val;
        }
        __syncwarp();
      }
    }
    // every MMA is complete before TMEM is freed
    bool dn = mbar_wait(smem_u32(&done_bar), 0);
    dn = __all_sync(0xffffffffu, dn);
    if (!dn) atomicExch(&abort_flag, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
}

// ---------------------------------------------------------------- packing

__device__ __forceinline__ int biased_exp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7FF); }

// ex[r] = max over the row of the biased exponent (ex zeroed before), for
// sources whose k index is the faster one: a warp per (row, k-slab), each
// lane reading 4 consecutive k at a time
__global__ void __launch_bounds__(256) oz_exp_rows_kernel(const double* __restrict__ src, PackSpec ps, int64_t kslab,
                                                          int* __restrict__ ex) {
  const int lane = threadIdx.x & 31;
  const int64_t nks = (ps.K + kslab - 1) / kslab;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool k1 = pack_k_single(ps);
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < ps.R * nks; w += nw) {
    const int64_t r = w / nks, ka = (w % nks) * kslab, kb = min(ps.K, ka + kslab);
    const int64_t ro = pack_row_off(ps, r);
    int m = 0;
    for (int64_t k0 = ka + 4 * lane; k0 < kb; k0 += 128) {
      double xv[4];
      pack_load4(src, ps, k1, ro, k0, (int)min((int64_t)4, kb - k0), xv);
#pragma unroll
      for (int q = 0; q < 4; ++q) m = max(m, biased_exp(xv[q]));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0 && m > 0) atomicMax(ex + r, m);
  }
}

// same for sources whose row index is the faster one: 32 rows x 8 k-lanes
// per block over one k-slab, the column offsets of each 32-column step in
// shared memory
__global__ void __launch_bounds__(256) oz_exp_tiles_kernel(const double* __restrict__ src, PackSpec ps, int64_t kslab,
                                                           int* __restrict__ ex) {
  __shared__ int red[8][32];
  __shared__ int64_t coff[32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t nrt = (ps.R + 31) / 32, nks = (ps.K + kslab - 1) / kslab;
  for (int64_t tb = blockIdx.x; tb < nrt * nks; tb += gridDim.x) {
    const int64_t r = (tb / nks) * 32 + tx;
    const int64_t ka = (tb % nks) * kslab, kb = min(ps.K, ka + kslab);
    const int64_t ro = r < ps.R ? pack_row_off(ps, r) : 0;
    int m = 0;
    for (int64_t kc = ka; kc < kb; kc += 32) {
      __syncthreads();   // the previous offsets are consumed
      if (ty == 0) coff[tx] = kc + tx < kb ? pack_col_off(ps, kc + tx) : 0;
      __syncthreads();
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int kk = ty + 8 * j;
        if (r < ps.R && kc + kk < kb) m = max(m, biased_exp(src[ro + coff[kk]]));
      }
    }
    red[ty][tx] = m;
    __syncthreads();
    if (ty == 0) {
      for (int j = 1; j < 8; ++j) m = max(m, red[j][tx]);
      if (r < ps.R && m > 0) atomicMax(ex + r, m);
    }
    __syncthreads();
  }
}

// bf16 bits of the integer d (|d| < 2^22; exact in bf16 for |d| <= 256): the
// float 1.5 * 2^23 + d, less the bias, is d exactly, and its top 16 bits are
// the bf16 of d
__device__ __forceinline__ uint32_t oz_int_bf16(int d) {
  return __float_as_uint(__int_as_float(0x4B400000 + d) - 12582912.0f) >> 16;
}

// The S balanced base-64 digits of y = x 2^-e (|x| < 2^e), as bf16 bits: the
// integer Z = round(|y| 64^S) is written as d_1 64^(S-1) + ... + d_S with
// d_S..d_2 in [-32, 32) and d_1 = the rest, 0..64, all signed like x.  The
// low digits are the plain base-64 digits of Z + 32 (64^(S-2) + ... + 1),
// less 32 (a digit of Z at or above 32 carries one into the next, as in the
// sequential cut).  Integer arithmetic only; |y - sum_s d_s 64^-s| <= 64^-S / 2.
template <int S>
__device__ __forceinline__ void oz_digits(double x, int e, uint32_t (&d)[S]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int be = (int)((bits >> 52) & 0x7FF);
  unsigned long long Z = 0;
  if (be != 0) {
    const unsigned long long m = (bits & ((1ull << 52) - 1)) | (1ull << 52);   // |x| = m 2^(be - 1075)
    const int sh = 1075 + e - 6 * S - be;                                      // Z = m 2^-sh, sh > 0
    if (sh <= 0) Z = m << (-sh);
    else if (sh < 64) Z = (m >> sh) + ((m >> (sh - 1)) & 1ull);
  }
  constexpr unsigned long long C = 32ull * (((1ull << (6 * (S - 1))) - 1) / 63);
  const unsigned long long Zc = Z + C;
  const int neg = (int)(bits >> 63);
#pragma unroll
  for (int s = 1; s < S; ++s) {
    const int dv = (int)((Zc >> (6 * (S - 1 - s))) & 63ull) - 32;
    d[s] = oz_int_bf16(neg ? -dv : dv);
  }
  const int top = (int)(Zc >> (6 * (S - 1)));
  d[0] = oz_int_bf16(neg ? -top : top);
}

constexpr int OZ_MAXS = 8;

// dst[r][s*Kpad + k]: row walk (k the faster source index), 2^lg threads per
// row, each cutting 4 consecutive k and writing one 8-byte word per slice
// (zeros over the padding [K, Kpad))
template <int S>
__global__ void __launch_bounds__(256) oz_pack_rows_kernel(const double* __restrict__ src, PackSpec ps, int64_t Kpad,
                                                           const int* __restrict__ ex, __nv_bfloat16* __restrict__ dst,
                                                           PackWalk pw) {
  const int tpr = 1 << pw.lg, lane = threadIdx.x & (tpr - 1), rpb = 256 >> pw.lg;
  const int64_t ng = Kpad >> 2;
  const bool k1 = pack_k_single(ps);
  const int64_t units = ps.R * pw.nseg;
  for (int64_t u = (int64_t)blockIdx.x * rpb + (threadIdx.x >> pw.lg); u < units; u += (int64_t)gridDim.x * rpb) {
    const int64_t r = pw.nseg == 1 ? u : u / pw.nseg;
    const int64_t g0 = (u - r * pw.nseg) * pw.gseg, g1 = min(ng, g0 + pw.gseg);
    const int e = oz_row_exp(ex[r]);
    const int64_t ro = pack_row_off(ps, r);
    __nv_bfloat16* drow = dst + r * (S * Kpad);
    for (int64_t g = g0 + lane; g < g1; g += tpr) {
      const int64_t k0 = g << 2;
      uint2 w[S];
      if (k0 < ps.K) {
        double xv[4];
        pack_load4(src, ps, k1, ro, k0, (int)min((int64_t)4, ps.K - k0), xv);
        uint32_t dg[4][S];
#pragma unroll
        for (int q = 0; q < 4; ++q) oz_digits<S>(xv[q], e, dg[q]);
#pragma unroll
        for (int s = 0; s < S; ++s) w[s] = make_uint2(dg[0][s] | (dg[1][s] << 16), dg[2][s] | (dg[3][s] << 16));
      } else {
#pragma unroll
        for (int s = 0; s < S; ++s) w[s] = make_uint2(0u, 0u);
      }
#pragma unroll
      for (int s = 0; s < S; ++s) *reinterpret_cast<uint2*>(drow + s * Kpad + k0) = w[s];
    }
  }
}

// transposing walk through 32 x 32 tiles (row index faster in the source):
// source offsets of the tile's rows and columns in shared memory, coalesced
// reads along rows, and each thread cuts two consecutive k of one row and
// writes one 4-byte word per slice (the tiles cover [0, Kpad), zeros past K)
template <int S>
__global__ void __launch_bounds__(256) oz_pack_tiles_kernel(const double* __restrict__ src, PackSpec ps, int64_t Kpad,
                                                            const int* __restrict__ ex,
                                                            __nv_bfloat16* __restrict__ dst) {
  __shared__ double tile[32][33];
  __shared__ int64_t roff[32], coff[32];
  const int64_t ntr = (ps.R + 31) / 32, ntk = Kpad / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int kp = threadIdx.x & 15, rw = threadIdx.x >> 4;   // write phase: k pair, row
  for (int64_t tb = blockIdx.x; tb < ntr * ntk; tb += gridDim.x) {
    const int64_t r0 = (tb / ntk) * 32, k0 = (tb % ntk) * 32;
    __syncthreads();   // the previous tile is consumed
    if (ty == 0) roff[tx] = r0 + tx < ps.R ? pack_row_off(ps, r0 + tx) : 0;
    else if (ty == 1) coff[tx] = k0 + tx < ps.K ? pack_col_off(ps, k0 + tx) : 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kk = ty + 8 * j;
      tile[kk][tx] = (r0 + tx < ps.R && k0 + kk < ps.K) ? src[roff[tx] + coff[kk]] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int rr = rw + 16 * j;
      const int64_t r = r0 + rr;
      if (r >= ps.R) continue;
      const int e = oz_row_exp(ex[r]);
      uint32_t da[S], db[S];
      oz_digits<S>(tile[2 * kp][rr], e, da);
      oz_digits<S>(tile[2 * kp + 1][rr], e, db);
      uint32_t* d = reinterpret_cast<uint32_t*>(dst + r * (S * Kpad) + k0 + 2 * kp);
#pragma unroll
      for (int s = 0; s < S; ++s) d[(s * Kpad) >> 1] = da[s] | (db[s] << 16);
    }
  }
}

std::once_flag g_oz_attr;

}  // namespace

int64_t oz_kpad(int64_t K) { return ((K + OZ_BK - 1) / OZ_BK) * OZ_BK; }

void pack_oz(const double* src, const PackSpec& ps, int S, __nv_bfloat16* dst, int* ex, cudaStream_t s) {
  if (ps.R <= 0 || ps.K <= 0) return;
  if (S < 1 || S > OZ_MAXS) fail(FCC_ERR_BAD_ARG, "bad slice count");
  if (ps.R >= (int64_t(1) << 31) || ps.K >= (int64_t(1) << 31)) fail(FCC_ERR_BAD_ARG, "pack extent too large");
  const int64_t Kpad = oz_kpad(ps.K);
  const int pidx = prof_begin(s);
  struct End { cudaStream_t s; int i; double b; ~End() { prof_end(s, i, PROF_PACK, b); } } pend{s, pidx,
      2.0 * (double)ps.R * (double)ps.K * 8.0 + (double)ps.R * (double)(S * Kpad) * 2.0};
  FCC_CUDA(cudaMemsetAsync(ex, 0, sizeof(int) * ps.R, s));
  const int64_t kfast = std::llabs(ps.kd3 > 1 ? ps.ks3 : (ps.kd2 > 1 ? ps.ks2 : ps.ks1));
  const int64_t rfast = std::llabs(ps.rd3 > 1 ? ps.rs3 : (ps.rd2 > 1 ? ps.rs2 : ps.rs1));
  const bool tiles = rfast < kfast && ps.R >= 32;
  // k-slabs so that the exponent pass has enough independent work
  const int64_t want = 152 * 64;
  const int64_t units = tiles ? (ps.R + 31) / 32 : ps.R;
  int64_t kslab = ps.K;
  if (units < want) kslab = std::max<int64_t>(256, (ps.K * units + want - 1) / want);
  const int64_t nks = (ps.K + kslab - 1) / kslab;
  const PackWalk pw = pack_walk(ps.R, Kpad / 4);
  const unsigned rgrid = pack_walk_grid(pw, ps.R);
  const unsigned tgrid = (unsigned)std::min<int64_t>(((ps.R + 31) / 32) * (Kpad / 32), 152 * 16);
#define FCC_OZ_PACK(SS)                                                                       \
  case SS:                                                                                    \
    if (tiles) oz_pack_tiles_kernel<SS><<<tgrid, 256, 0, s>>>(src, ps, Kpad, ex, dst);         \
    else oz_pack_rows_kernel<SS><<<rgrid, 256, 0, s>>>(src, ps, Kpad, ex, dst, pw);            \
    break;
  if (tiles) {
    oz_exp_tiles_kernel<<<(unsigned)std::min<int64_t>(units * nks, 152 * 32), 256, 0, s>>>(src, ps, kslab, ex);
  } else {
    const int64_t warps = units * nks;
    oz_exp_rows_kernel<<<(unsigned)std::min<int64_t>((warps + 7) / 8, 152 * 32), 256, 0, s>>>(src, ps, kslab, ex);
  }
  FCC_CHECK_LAUNCH();
  switch (S) {
    FCC_OZ_PACK(1)
    FCC_OZ_PACK(2)
    FCC_OZ_PACK(3)
    FCC_OZ_PACK(4)
    FCC_OZ_PACK(5)
    FCC_OZ_PACK(6)
    FCC_OZ_PACK(7)
    FCC_OZ_PACK(8)
    default: fail(FCC_ERR_BAD_ARG, "bad slice count");
  }
#undef FCC_OZ_PACK
  FCC_CHECK_LAUNCH();
}

void gemm_oz(const __nv_bfloat16* A, int64_t a_rows, const int* exA, const __nv_bfloat16* B, int64_t b_rows,
             const int* exB, int64_t Kpad, int G, const EpiMap& ep, int* err, cudaStream_t s) {
  if (ep.M <= 0 || ep.N <= 0) return;
  if (ep.mode != EPI_F64) fail(FCC_ERR_BAD_ARG, "exact-slice products write FP64 only");
  if (G < 2 || G > OZ_MAXS + 1) fail(FCC_ERR_BAD_ARG, "bad exact-slice group count");
  if (Kpad <= 0 || Kpad % OZ_BK) fail(FCC_ERR_BAD_ARG, "bad padded K");
  if (a_rows < ep.M || b_rows < ep.N) fail(FCC_ERR_BAD_ARG, "packed operands smaller than the output");
  const int S = G - 1;
  const int nkb = (int)(Kpad / OZ_BK);
  std::call_once(g_oz_attr, []() {
    cudaFuncSetAttribute(gemm_oz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
  });
  const OzPairs pr = make_pairs(G);
  CUtensorMap ta = tma_map_bf16(A, a_rows, S * Kpad, OZ_BM);
  CUtensorMap tb = tma_map_bf16(B, b_rows, S * Kpad, OZ_BN);
  const int64_t tm = (ep.M + OZ_BM - 1) / OZ_BM, tn = (ep.N + OZ_BN - 1) / OZ_BN;
  const int64_t tiles = tm * tn;
  // K ranges per tile.  (1) The units that run at the same time (one per SM,
  // about 8 tile rows x 19 tile columns in the grouped order) share one K
  // range; their operand panels (all S slices of a 128-row block over the
  // range) must fit in L2 together, or every slice is fetched again from HBM
  // for each slice pair that uses it (a full-K ring launch at (H2O)8 read
  // 17 GB for 0.76 GB of packed operands).  (2) More ranges also fill the GPU
  // when the output has few tiles; a unit pays a fixed cost (its final
  // epilogue and the reduction into C) of about 48 k-block steps.
  const double panel = (double)OZ_BM * S * (double)Kpad * 2.0;
  const int64_t conc = std::min<int64_t>(tiles, 152);
  const int64_t rblk = std::min<int64_t>(tm, 8);
  const int64_t cblk = std::min<int64_t>(tn, (conc + rblk - 1) / rblk);
  constexpr double L2_BUDGET = 48.0 * (1 << 20);
  int zl2 = (int)std::ceil((double)(rblk + cblk) * panel / L2_BUDGET);
  const int total = pr.n * nkb;
  int zw = 1;
  double best = 1e300;
  constexpr double CTA_FIXED_STEPS = 48.0;
  for (int sp = 1; sp <= 64 && sp * OZ_CH <= total; ++sp) {
    const double waves = std::ceil((double)(tiles * sp) / 152.0);
    const double t = waves * ((double)total / sp + CTA_FIXED_STEPS);
    if (t < best * 0.97) { best = t; zw = sp; }
  }
  int splits = std::max(zl2, zw);
  splits = std::max(1, std::min({splits, 64, std::max(1, nkb / 4)}));
  const int kper = (nkb + splits - 1) / splits;
  splits = (nkb + kper - 1) / kper;
  // no loads of C in the kernel: beta = 0 and one K range store, otherwise C
  // is scaled by beta first (not for beta = 1) and the kernel reduces into it
  EpiMap e2 = ep;
  e2.atomic = (splits > 1 || ep.beta != 0.0) ? 1 : 0;
  if (e2.atomic && ep.beta != 1.0) scale_output(ep, ep.beta, s);
  const int64_t units = tiles * splits;
  const int64_t grid = std::min<int64_t>(units, 152);   // one persistent CTA per SM
  const int pidx = prof_begin(s);
  gemm_oz_kernel<<<(unsigned)grid, OZ_THREADS, OZ_SMEM, s>>>(ta, tb, nkb, (int)Kpad, pr, kper, tm, tn, units, exA,
                                                             exB, G, e2, err);
  FCC_CHECK_LAUNCH();
  prof_end(s, pidx, PROF_OZ, ep.work > 0 ? ep.work : 2.0 * (double)ep.M * (double)ep.N * (double)(Kpad * pr.n));
}

}  // namespace fcc
