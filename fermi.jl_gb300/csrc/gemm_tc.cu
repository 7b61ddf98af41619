// Split-BF16 tensor-core contraction for GB300 (sm_103a): tcgen05.mma with the
// accumulator in TMEM, operands staged by TMA (cp.async.bulk.tensor) into
// 128-byte-swizzled shared memory, an mbarrier pipeline between one producer
// thread, one MMA-issuing thread and four epilogue warps.
//
// A FP64 contraction C = alpha * A.B + beta * C is evaluated as one BF16 GEMM
// over a K-concatenated operand pair (three products, FP32 accumulation):
//   A' = [hi(A) | hi(A) | lo(A)],  B' = [hi(B) | lo(B) | hi(B)]
//   A'.B'^T = hi(A) hi(B) + hi(A) lo(B) + lo(A) hi(B)
// with hi(x) = bf16(x) and lo(x) = bf16(x - hi(x)).  The pack kernel gathers
// the operand from any strided tensor view (the index permutation of the
// contraction is folded into it) and the epilogue scatters into any strided
// output view, so no separate transpose pass exists.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "fcc_tc.cuh"
#include "fcc_tcgen05.cuh"

namespace fcc {

namespace {

using namespace tc5;

constexpr int BM = 128;
constexpr int BK = 64;                       // one 128-byte swizzle atom of bf16 per row
constexpr int TC_THREADS = 192;              // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

template <int BN>
struct TcCfg {
  static constexpr int STAGES = (BN == 256) ? 4 : 6;
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;  // + alignment slack
};

// bf16 bits of (-1)^sgn * m * 2^e for 0 <= m <= 256; zero below the bf16
// normal range (|value| < 2^-126), infinity above it.
__device__ __forceinline__ uint16_t bf16_bits(uint32_t sgn, uint32_t m, int e) {
  if (m == 0) return 0;
  const int lz = __clz(m) - 24;              // m in [1, 255]: shift up to [128, 255]
  if (lz >= 0) { m <<= lz; e -= lz; }
  else { m >>= 1; e += 1; }                  // m == 256
  const int b = e + 7 + 127;                 // m * 2^e = (m / 128) * 2^(e + 7)
  if (b <= 0) return 0;
  if (b >= 255) return (uint16_t)((sgn << 15) | 0x7F80u);
  return (uint16_t)((sgn << 15) | ((uint32_t)b << 7) | (m & 0x7Fu));
}

// a (0 < a < 2^62) rounded to nearest-even at 8 significant bits: returns m
// in [1, 256] with a ~ m * 2^sh
__device__ __forceinline__ uint32_t round8(uint64_t a, int& sh) {
  const int n = 64 - __clzll((long long)a);
  if (n <= 8) { sh = 0; return (uint32_t)a; }
  sh = n - 8;
  const uint64_t q = a >> sh, rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  return (uint32_t)(q + ((rem > half || (rem == half && (q & 1))) ? 1u : 0u));
}

// hi, mid, lo bf16 pieces of x, each the nearest (ties to even) 8-bit value to
// what the previous pieces leave, so |x - hi - mid - lo| <= 2^-24 |x|
// (typically ~2^-27; pieces below the bf16 range become zero).  Integer arithmetic on the
// FP64 bit pattern: the remainders are exact and no FP64 instruction (a slow
// pipe on this part) is issued.
__device__ __noinline__ void split3_int(double x, __nv_bfloat16 (&lv)[3]) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((u >> 52) & 0x7FF);
  uint16_t h = 0, m = 0, l = 0;
  if (ex == 0x7FF) {                         // inf keeps its sign, nan becomes the canonical bf16 nan
    const bool nan = (u & ((1ull << 52) - 1)) != 0;
    lv[0] = __ushort_as_bfloat16(nan ? (unsigned short)0x7FFF : (unsigned short)(((u >> 48) & 0x8000u) | 0x7F80u));
    lv[1] = lv[2] = __ushort_as_bfloat16((unsigned short)0);
    return;
  }
  if (ex != 0) {                             // zero and FP64 subnormals give zeros
    const uint64_t M = (u & ((1ull << 52) - 1)) | (1ull << 52);   // |x| = M 2^e0
    const int e0 = ex - 1075;
    uint32_t sg = (uint32_t)(u >> 63);
    int sh;
    uint32_t q = round8(M, sh);
    h = bf16_bits(sg, q, e0 + sh);
    int64_t r = (int64_t)M - ((int64_t)q << sh);
    if (r != 0) {
      if (r < 0) { sg ^= 1u; r = -r; }
      q = round8((uint64_t)r, sh);
      m = bf16_bits(sg, q, e0 + sh);
      r -= (int64_t)q << sh;
      if (r != 0) {
        if (r < 0) { sg ^= 1u; r = -r; }
        q = round8((uint64_t)r, sh);
        l = bf16_bits(sg, q, e0 + sh);
      }
    }
  }
  lv[0] = __ushort_as_bfloat16(h);
  lv[1] = __ushort_as_bfloat16(m);
  lv[2] = __ushort_as_bfloat16(l);
}

// float of an integer v < 2^23, exactly
__device__ __forceinline__ float small_uint_float(uint32_t v) { return __uint_as_float(0x4B000000u | v) - 8388608.0f; }

// bf16 bits of the nearest (ties to even) 8-bit value to a * scale, for an
// integer 0 < a < 2^46 and a power of two scale with a * scale in the normal
// float range.  a is cut at 24 significant bits with the last one set when
// anything below is nonzero (rounding to odd, Boldo & Melquiond, IEEE Trans.
// Comput. 57 (2008)), so that the float-to-bf16 rounding of that float equals
// the rounding of a itself: a = X + Y with X = (a >> 23) 2^23 and Y < 2^23,
// both exact floats; s = X + Y rounded toward zero is a cut at 24 bits, and
// s - X is exact (Sterbenz), so s - X != Y tells whether the cut lost bits.
__device__ __forceinline__ uint32_t rne8_bits(uint64_t a, float scale) {
  const float X = small_uint_float((uint32_t)(a >> 23)) * 8388608.0f;
  const float Y = small_uint_float((uint32_t)a & 0x7FFFFFu);
  const float sr = __fadd_rz(X, Y);
  const uint32_t odd = __fsub_rn(sr, X) != Y ? 1u : 0u;
  const float f = __fmul_rn(__uint_as_float(__float_as_uint(sr) | odd), scale);
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(f));
}

// integer value of the positive bf16 piece pb in units of 2^e0
__device__ __forceinline__ uint64_t piece_units(uint32_t pb, int e0) {
  const uint64_t m8 = 0x80u | (pb & 0x7Fu);
  const int sh = (int)((pb >> 7) & 0xFFu) - 134 - e0;
  return sh >= 0 ? m8 << sh : m8 >> (-sh);
}

// The same three pieces as split3_int, computed with single-precision
// arithmetic where every piece is a normal float (2^-74 <= |x| < 2^127, so
// all pieces, multiples of the FP64 ulp of x, are at least 2^-126): the
// remainders stay exact 64-bit integers in units of that ulp, and each
// rounding to 8 bits goes through rne8_bits; other x take split3_int (not
// inlined, so the common path carries none of its instructions).
__device__ __forceinline__ void split3(double x, __nv_bfloat16 (&lv)[3]) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex < 949 || ex > 1149) {
    split3_int(x, lv);
    return;
  }
  const uint32_t sg = (uint32_t)(u >> 63);
  const int e0 = ex - 1075;                                       // |x| = M 2^e0
  const uint64_t M = (u & ((1ull << 52) - 1)) | (1ull << 52);
  // hi: the top 24 bits of M rounded to odd, as a float of the scale of x
  const uint32_t A = (uint32_t)(M >> 29) | ((M & ((1ull << 29) - 1)) != 0 ? 1u : 0u);
  const uint32_t hb =
      (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(__uint_as_float(((uint32_t)(ex - 896) << 23) | (A & 0x7FFFFFu))));
  const int64_t r1 = (int64_t)M - (int64_t)piece_units(hb, e0);
  uint32_t m = 0, l = 0;
  if (r1 != 0) {
    const float scale = __uint_as_float((uint32_t)(e0 + 127) << 23);   // 2^e0
    const uint32_t sg1 = sg ^ (r1 < 0 ? 1u : 0u);
    const uint64_t a1 = (uint64_t)(r1 < 0 ? -r1 : r1);
    const uint32_t mb = rne8_bits(a1, scale);
    m = (sg1 << 15) | mb;
    const int64_t r2 = (int64_t)a1 - (int64_t)piece_units(mb, e0);
    if (r2 != 0) {
      const uint32_t sg2 = sg1 ^ (r2 < 0 ? 1u : 0u);
      l = (sg2 << 15) | rne8_bits((uint64_t)(r2 < 0 ? -r2 : r2), scale);
    }
  }
  lv[0] = __ushort_as_bfloat16((unsigned short)((sg << 15) | hb));
  lv[1] = __ushort_as_bfloat16((unsigned short)m);
  lv[2] = __ushort_as_bfloat16((unsigned short)l);
}

// piece `lev` (0 hi, 1 mid, 2 lo) without a dynamically indexed local array
__device__ __forceinline__ __nv_bfloat16 piece(const __nv_bfloat16 (&lv)[3], int lev) {
  return lev == 0 ? lv[0] : (lev == 1 ? lv[1] : lv[2]);
}

template <int BN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_bf16_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int64_t a_row0,
                        int64_t b_row0, int num_k, int k_chunk, EpiMap ep, int* err) {
  using Cfg = TcCfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[Cfg::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[Cfg::STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_flag;
  __shared__ float epi_tile[4][32][33];   // per epilogue warp: 32 x 32 transpose

  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + Cfg::STAGES * Cfg::A_BYTES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&acc_bar), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_holder;
  int64_t mt, nt;
  grouped_tile(blockIdx.x, (ep.M + BM - 1) / BM, (ep.N + BN - 1) / BN, mt, nt);
  const int64_t m0 = mt * BM;
  const int64_t n0 = nt * BN;
  // split-K: this CTA reduces k-tiles [kb, ke); partial sums are added atomically
  const int kb = (int)blockIdx.z * k_chunk;
  const int ke = min(num_k, kb + k_chunk);
  const int nkt = max(0, ke - kb);

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer (none at all under the no_loads test hook:
    // nothing is then in flight, and the MMA thread's bounded wait gives up)
    for (int kt = 0; kt < (ep.no_loads ? 0 : nkt); ++kt) {
      const int s = kt % Cfg::STAGES;
      const uint32_t ph = (kt / Cfg::STAGES) & 1;
      if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1)) { atomicExch(&abort_flag, 1); break; }
      if (*(volatile int*)&abort_flag) break;
      const uint32_t fb = smem_u32(&full_bar[s]);
      mbar_expect_tx(fb, Cfg::STAGE_BYTES);
      tma_load_2d(smem_u32(sA + s * Cfg::A_BYTES), &tmA, (kb + kt) * BK, (int32_t)(a_row0 + m0), fb);
      tma_load_2d(smem_u32(sB + s * Cfg::B_BYTES), &tmB, (kb + kt) * BK, (int32_t)(b_row0 + n0), fb);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer (single thread)
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    bool ok = true;
    for (int kt = 0; kt < nkt; ++kt) {
      const int s = kt % Cfg::STAGES;
      const uint32_t ph = (kt / Cfg::STAGES) & 1;
      if (!mbar_wait(smem_u32(&full_bar[s]), ph)) { atomicExch(&abort_flag, 1); ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ad = sw128_desc(smem_u32(sA + s * Cfg::A_BYTES));
      const uint64_t bd = sw128_desc(smem_u32(sB + s * Cfg::B_BYTES));
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad + (uint64_t)(2 * kk)), "l"(bd + (uint64_t)(2 * kk)), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&empty_bar[s]))
                   : "memory");
    }
    // signals the epilogue once every issued MMA has completed (also on abort)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&acc_bar))
                 : "memory");
    (void)ok;
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> strided global stores
    bool ok = mbar_wait(smem_u32(&acc_bar), 0);
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) atomicExch(&abort_flag, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int q = warp & 3;              // TMEM lane quadrant this warp may access
    const int row = q * 32 + lane;
    const int64_t m = m0 + row;
    const bool abort_now = __any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0);
    if (ok && !abort_now && nkt > 0) {
      // this lane's row offset; rows are broadcast to the warp below
      int64_t crow = 0;
      if (m < ep.M) {
        int64_t m3 = m % ep.md3, r = m / ep.md3;
        int64_t m2 = r % ep.md2, m1 = r / ep.md2;
        crow = m1 * ep.ms1 + m2 * ep.ms2 + m3 * ep.ms3;
      }
      float (*tile)[33] = epi_tile[q];
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        if (n0 + c0 >= ep.N) break;
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // transpose the warp's 32 x 32 block through shared memory so each
        // store instruction writes 32 consecutive columns of one row
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j) tile[lane][j] = __uint_as_float(r[j]);
        __syncwarp();
        const int64_t n = n0 + c0 + lane;
        const bool nok = n < ep.N;
        int64_t coff = 0;
        if (nok) {
          int64_t n3 = n % ep.nd3, rr = n / ep.nd3;
          int64_t n2 = rr % ep.nd2, n1 = rr / ep.nd2;
          coff = n1 * ep.ns1 + n2 * ep.ns2 + n3 * ep.ns3;
        }
        // all loads of the block first (independent, so they overlap), then
        // the stores
        // FP64 outputs with beta = 1 are reduced into C (red.add, no load);
        // only other betas read C
        const bool rmw = ep.beta != 0.0 && !ep.atomic && ep.mode != EPI_SPLIT &&
                         !(ep.mode == EPI_F64 && ep.beta == 1.0);
        double prev[32];
        float prevf[32];
        if (rmw) {
#pragma unroll
          for (int jr = 0; jr < 32; ++jr) {
            const int64_t roff = __shfl_sync(0xffffffffu, crow, jr);
            const bool ok2 = nok && (m0 + q * 32 + jr) < ep.M;
            prev[jr] = 0.0;
            prevf[jr] = 0.0f;
            if (ok2) {
              if (ep.mode == EPI_F32) prevf[jr] = static_cast<const float*>(ep.C)[roff + coff];
              else prev[jr] = static_cast<const double*>(ep.C)[roff + coff];
            }
          }
        }
#pragma unroll
        for (int jr = 0; jr < 32; ++jr) {
          const int64_t roff = __shfl_sync(0xffffffffu, crow, jr);
          const int64_t mm = m0 + q * 32 + jr;
          if (mm >= ep.M || !nok) continue;
          const int64_t off = roff + coff;
          if (ep.mode == EPI_F32) {
            // FP32 output: FP32 arithmetic (the FP64 pipe is 1/64 rate on GB300)
            float* dst = static_cast<float*>(ep.C) + off;
            float fv = (float)ep.alpha * tile[jr][lane];
            if (rmw) fv += (float)ep.beta * prevf[jr];
            if (ep.atomic) atomicAdd(dst, fv);
            else *dst = fv;
            continue;
          }
          if (ep.mode == EPI_F64) {
            // FP32 product, converted to FP64 by integer arithmetic (the FP64
            // pipe, which F2F conversions use, is 1/64 rate on GB300)
            double val = f32_to_f64_scaled((float)ep.alpha * tile[jr][lane], 0, false);
            double* dst = static_cast<double*>(ep.C) + off;
            if (ep.atomic || ep.beta == 1.0) atomicAdd(dst, val);
            else if (rmw) *dst = val + ep.beta * prev[jr];
            else *dst = val;
            continue;
          }
          double val = (double)((float)ep.alpha * tile[jr][lane]);
          if (rmw) val = (ep.beta == 1.0) ? prev[jr] + val : val + ep.beta * prev[jr];
          if (ep.mode == EPI_SPLIT) {
            __nv_bfloat16* dst = static_cast<__nv_bfloat16*>(ep.C) + off;
            __nv_bfloat16 lv[3];
            split3(val, lv);
            for (int p = 0; p < ep.P; ++p) dst[p * ep.piece] = piece(lv, (ep.code >> (2 * p)) & 3);
          } else if (ep.mode == EPI_F32) {
            float* dst = static_cast<float*>(ep.C) + off;
            if (ep.atomic) atomicAdd(dst, (float)val);
            else *dst = (float)val;
          } else {
            double* dst = static_cast<double*>(ep.C) + off;
            if (ep.atomic) atomicAdd(dst, val);
            else *dst = val;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
}

// ---------------------------------------------------------------- packing

// Scale modes of the split packing: the source times 1, times -1 (a sign flip
// of the bit pattern) or times a general factor (one FP64 multiply).
enum { PK_ONE = 0, PK_NEG = 1, PK_ANY = 2 };
template <int SM>
__device__ __forceinline__ double pk_scaled(double v, double scale) {
  if (SM == PK_ONE) return v;
  if (SM == PK_NEG) return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
  return v * scale;
}

// dst[r][k'] (row pitch Kp) from src: piece p of k' = p*K + k holds hi, mid or
// lo of src(r, k) per `code`; columns >= P*K are zero.  Row walk (k the
// faster source index): 2^lg threads per row, each splitting 4 consecutive k
// once and writing all P pieces, or zeroing 4 of the pad columns.
template <int SM>
__global__ void __launch_bounds__(256) pack_rows_kernel(const double* __restrict__ src, PackSpec ps,
                                                        __nv_bfloat16* __restrict__ dst, PackWalk pw) {
  const int tpr = 1 << pw.lg, lane = threadIdx.x & (tpr - 1), rpb = 256 >> pw.lg;
  const int64_t kq = (ps.K + 3) >> 2, pk = ps.P * ps.K;
  const int64_t ng = kq + ((ps.Kp - pk + 3) >> 2);
  const bool k1 = pack_k_single(ps);
  const bool vec = (ps.K & 3) == 0 && (ps.Kp & 3) == 0 && (reinterpret_cast<uintptr_t>(dst) & 7) == 0;
  const int64_t units = ps.R * pw.nseg;
  for (int64_t u = (int64_t)blockIdx.x * rpb + (threadIdx.x >> pw.lg); u < units; u += (int64_t)gridDim.x * rpb) {
    const int64_t r = pw.nseg == 1 ? u : u / pw.nseg;
    const int64_t g0 = (u - r * pw.nseg) * pw.gseg, g1 = min(ng, g0 + pw.gseg);
    const int64_t ro = pack_row_off(ps, r);
    __nv_bfloat16* drow = dst + r * ps.Kp;
    for (int64_t g = g0 + lane; g < g1; g += tpr) {
      if (g < kq) {
        const int64_t k0 = g << 2;
        const int cnt = (int)min((int64_t)4, ps.K - k0);
        double xv[4];
        pack_load4(src, ps, k1, ro, k0, cnt, xv);
        __nv_bfloat16 lv[4][3];
#pragma unroll
        for (int q = 0; q < 4; ++q) split3(pk_scaled<SM>(xv[q], ps.scale), lv[q]);
        for (int p = 0; p < ps.P; ++p) {
          const int lev = (ps.code >> (2 * p)) & 3;
          __nv_bfloat16* d = drow + p * ps.K + k0;
          if (vec && cnt == 4) {
            __nv_bfloat162 v0 = __halves2bfloat162(piece(lv[0], lev), piece(lv[1], lev));
            __nv_bfloat162 v1 = __halves2bfloat162(piece(lv[2], lev), piece(lv[3], lev));
            uint2 u;
            u.x = *reinterpret_cast<uint32_t*>(&v0);
            u.y = *reinterpret_cast<uint32_t*>(&v1);
            *reinterpret_cast<uint2*>(d) = u;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (q < cnt) d[q] = piece(lv[q], lev);
          }
        }
      } else {
        const int64_t c0 = pk + ((g - kq) << 2);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (c0 + q < ps.Kp) drow[c0 + q] = __ushort_as_bfloat16((unsigned short)0);
      }
    }
  }
}

// Transposing walk through 32 x 32 tiles, for sources whose row index is the
// faster one in memory: the tile's row and column source offsets are
// computed once into shared memory, reads coalesce along rows, and each
// thread splits two consecutive k of one row and writes them as one 4-byte
// store per piece.
template <int SM>
__global__ void __launch_bounds__(256) pack_tiles_kernel(const double* __restrict__ src, PackSpec ps,
                                                         __nv_bfloat16* __restrict__ dst) {
  __shared__ double tile[32][33];
  __shared__ int64_t roff[32], coff[32];
  const int64_t ntr = (ps.R + 31) / 32, ntk = (ps.K + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int kp = threadIdx.x & 15, rw = threadIdx.x >> 4;   // write phase: k pair, row
  const bool pair = (ps.K & 1) == 0 && (ps.Kp & 1) == 0 && (reinterpret_cast<uintptr_t>(dst) & 3) == 0;
  for (int64_t tb = blockIdx.x; tb < ntr * ntk; tb += gridDim.x) {
    const int64_t r0 = (tb / ntk) * 32, k0 = (tb % ntk) * 32;
    __syncthreads();   // the previous tile is consumed
    if (ty == 0) roff[tx] = r0 + tx < ps.R ? pack_row_off(ps, r0 + tx) : 0;
    else if (ty == 1) coff[tx] = k0 + tx < ps.K ? pack_col_off(ps, k0 + tx) : 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kk = ty + 8 * j;
      tile[kk][tx] =
          (r0 + tx < ps.R && k0 + kk < ps.K) ? pk_scaled<SM>(src[roff[tx] + coff[kk]], ps.scale) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int rr = rw + 16 * j;
      const int64_t r = r0 + rr, k = k0 + 2 * kp;
      if (r >= ps.R || k >= ps.K) continue;
      const bool two = k + 1 < ps.K;
      __nv_bfloat16 a[3], b[3];
      split3(tile[2 * kp][rr], a);
      split3(two ? tile[2 * kp + 1][rr] : 0.0, b);
      __nv_bfloat16* d = dst + r * ps.Kp + k;
      for (int p = 0; p < ps.P; ++p) {
        const int lev = (ps.code >> (2 * p)) & 3;
        if (two && pair) {
          *reinterpret_cast<__nv_bfloat162*>(d + p * ps.K) = __halves2bfloat162(piece(a, lev), piece(b, lev));
        } else {
          d[p * ps.K] = piece(a, lev);
          if (two) d[p * ps.K + 1] = piece(b, lev);
        }
      }
    }
  }
}

// zero columns [P*K, Kp) of every row
__global__ void pack_pad_kernel(PackSpec ps, __nv_bfloat16* __restrict__ dst) {
  const int64_t w = ps.Kp - ps.P * ps.K;
  const int64_t total = ps.R * w;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / w, c = t - r * w;
    dst[r * ps.Kp + ps.P * ps.K + c] = __float2bfloat16_rn(0.0f);
  }
}

// C = beta * C over an epilogue map (before split-K atomics).
__global__ void scale_out_kernel(EpiMap ep, double beta) {
  const int64_t total = ep.M * ep.N;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / ep.N, n = t - m * ep.N;
    const int64_t m3 = m % ep.md3, qm = m / ep.md3, n3 = n % ep.nd3, qn = n / ep.nd3;
    const int64_t off = (qm / ep.md2) * ep.ms1 + (qm % ep.md2) * ep.ms2 + m3 * ep.ms3 + (qn / ep.nd2) * ep.ns1 +
                        (qn % ep.nd2) * ep.ns2 + n3 * ep.ns3;
    if (ep.mode == EPI_F32) {
      float* d = static_cast<float*>(ep.C) + off;
      *d = beta == 0.0 ? 0.0f : (float)(beta * *d);
    } else {
      double* d = static_cast<double*>(ep.C) + off;
      *d = beta == 0.0 ? 0.0 : beta * *d;
    }
  }
}

// -------------------------------------------------------- tensor maps
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

void get_encoder() {
  std::call_once(g_encode_once, []() {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_encode) fail(FCC_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
}

CUtensorMap make_map(const __nv_bfloat16* base, int64_t rows, int64_t Kp, int box_rows) {
  get_encoder();
  if (Kp % BK != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0)
    fail(FCC_ERR_BAD_ARG, "packed operand misaligned for TMA");
  CUtensorMap tm;
  std::memset(&tm, 0, sizeof(tm));
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(FCC_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return tm;
}

template <int BN>
void launch_tc(const __nv_bfloat16* A, int64_t a_rows, int64_t a_row0, const __nv_bfloat16* B, int64_t b_rows,
               int64_t b_row0, int64_t Kp, const EpiMap& ep, int* err, cudaStream_t s) {
  using Cfg = TcCfg<BN>;
  static std::once_flag attr_once;
  std::call_once(attr_once, []() {
    cudaFuncSetAttribute(gemm_bf16_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  });
  CUtensorMap ta = make_map(A, a_rows, Kp, BM);
  CUtensorMap tb = make_map(B, b_rows, Kp, BN);
  const int64_t tm = (ep.M + BM - 1) / BM, tn = (ep.N + BN - 1) / BN;
  const int num_k = (int)(Kp / BK);
  // split K across CTAs when the output has too few tiles to fill the GPU
  int splits = 1;
  if (ep.mode != EPI_SPLIT && tm * tn < 152 && num_k >= 16)
    splits = (int)std::min<int64_t>((152 + tm * tn - 1) / (tm * tn), num_k / 8);
  splits = std::max(1, std::min(splits, 64));
  const int chunk = (num_k + splits - 1) / splits;
  splits = (num_k + chunk - 1) / chunk;
  EpiMap e2 = ep;
  if (splits > 1) {
    if (ep.beta != 1.0) {   // C = beta * C before the partial sums are added
      const int64_t tot = ep.M * ep.N;
      scale_out_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 152 * 16), 256, 0, s>>>(ep, ep.beta);
      FCC_CHECK_LAUNCH();
    }
    e2.atomic = 1;
  }
  if (tm * tn > 2147483647ll) fail(FCC_ERR_BAD_ARG, "tensor-core grid too large");
  dim3 grid((unsigned)(tm * tn), 1u, (unsigned)splits);
  const int pidx = prof_begin(s);
  gemm_bf16_tc_kernel<BN><<<grid, TC_THREADS, Cfg::SMEM, s>>>(ta, tb, a_row0, b_row0, num_k, chunk, e2, err);
  FCC_CHECK_LAUNCH();
  // executed BF16 flops (padded K included)
  prof_end(s, pidx, PROF_TC, ep.work > 0 ? ep.work : 2.0 * (double)ep.M * (double)ep.N * (double)Kp);
}

}  // namespace

int64_t packed_kp(int64_t K, int P) { return ((P * K + BK - 1) / BK) * BK; }

CUtensorMap tma_map_bf16(const __nv_bfloat16* base, int64_t rows, int64_t cols, int box_rows) {
  return make_map(base, rows, cols, box_rows);
}

void scale_output(const EpiMap& ep, double beta, cudaStream_t s) {
  const int64_t tot = ep.M * ep.N;
  if (tot <= 0) return;
  scale_out_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 152 * 16), 256, 0, s>>>(ep, beta);
  FCC_CHECK_LAUNCH();
}

void pack_split(const double* src, const PackSpec& ps, __nv_bfloat16* dst, cudaStream_t s) {
  if (ps.R <= 0 || ps.K <= 0) return;
  const int pidx = prof_begin(s);
  struct End { cudaStream_t s; int i; double b; ~End() { prof_end(s, i, PROF_PACK, b); } } pend{s, pidx,
      (double)ps.R * (double)ps.K * 8.0 + (double)ps.R * (double)ps.Kp * 2.0};
  if (ps.P < 1 || ps.P > 8 || ps.Kp < ps.P * ps.K) fail(FCC_ERR_BAD_ARG, "bad pack spec");
  if (ps.R >= (int64_t(1) << 31) || ps.K >= (int64_t(1) << 31)) fail(FCC_ERR_BAD_ARG, "pack extent too large");
  const int64_t kfast = std::llabs(ps.kd3 > 1 ? ps.ks3 : (ps.kd2 > 1 ? ps.ks2 : ps.ks1));
  const int64_t rfast = std::llabs(ps.rd3 > 1 ? ps.rs3 : (ps.rd2 > 1 ? ps.rs2 : ps.rs1));
  const int sm = ps.scale == 1.0 ? PK_ONE : (ps.scale == -1.0 ? PK_NEG : PK_ANY);
  if (rfast < kfast && ps.R >= 32) {
    const int64_t tiles = ((ps.R + 31) / 32) * ((ps.K + 31) / 32);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 152 * 16);
    if (sm == PK_ONE) pack_tiles_kernel<PK_ONE><<<grid, 256, 0, s>>>(src, ps, dst);
    else if (sm == PK_NEG) pack_tiles_kernel<PK_NEG><<<grid, 256, 0, s>>>(src, ps, dst);
    else pack_tiles_kernel<PK_ANY><<<grid, 256, 0, s>>>(src, ps, dst);
    FCC_CHECK_LAUNCH();
    if (ps.Kp > ps.P * ps.K) {
      const int64_t tot = ps.R * (ps.Kp - ps.P * ps.K);
      pack_pad_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 152 * 16), 256, 0, s>>>(ps, dst);
      FCC_CHECK_LAUNCH();
    }
  } else {
    const PackWalk pw = pack_walk(ps.R, (ps.K + 3) / 4 + (ps.Kp - ps.P * ps.K + 3) / 4);
    const unsigned grid = pack_walk_grid(pw, ps.R);
    if (sm == PK_ONE) pack_rows_kernel<PK_ONE><<<grid, 256, 0, s>>>(src, ps, dst, pw);
    else if (sm == PK_NEG) pack_rows_kernel<PK_NEG><<<grid, 256, 0, s>>>(src, ps, dst, pw);
    else pack_rows_kernel<PK_ANY><<<grid, 256, 0, s>>>(src, ps, dst, pw);
    FCC_CHECK_LAUNCH();
  }
}

void gemm_bf16x3(const __nv_bfloat16* A, int64_t a_rows, int64_t a_row0, const __nv_bfloat16* B, int64_t b_rows,
                 int64_t b_row0, int64_t Kp, const EpiMap& ep, int* err, cudaStream_t s) {
  if (ep.M <= 0 || ep.N <= 0) return;
  if (Kp <= 0 || Kp % BK) fail(FCC_ERR_BAD_ARG, "bad packed K");
  if (ep.N >= 256) launch_tc<256>(A, a_rows, a_row0, B, b_rows, b_row0, Kp, ep, err, s);
  else launch_tc<128>(A, a_rows, a_row0, B, b_rows, b_row0, Kp, ep, err, s);
}

}  // namespace fcc
