// Grouped, K-segmented split-BF16 tensor-core GEMM for the (T) intermediates.
//
// For one pair (i, j) and a run of k, W_ijk[a][b][c] is the sum of twelve
// contractions (PerturbativeTriples/ijk.jl:109-114).  Each term carries one
// virtual index alone on one operand (c, b or a) and the other two together
// on the other operand; grouping the terms by that lone index gives three
// groups of four terms with the same (pair, lone) orientation:
//   group 0: rows (a,b), columns c    group 1: rows (a,c), columns b
//   group 2: rows (b,c), columns a
// so each group is ONE product whose K is the concatenation of the four
// terms' K ranges (two over d, two over l; the l terms' signs are folded
// into their packed operands).  One launch computes all groups for all k of
// the run: CTA (m-tile, group, k), four K segments, each read by TMA from
// its own packed operand.  The FP32 results are stored once, G_g[k][pair][lone]
// (no read-modify-write); the energy kernel adds the three groups.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "fcc_t3.cuh"
#include "fcc_tcgen05.cuh"

namespace fcc {

namespace {

using namespace tc5;

constexpr int T3_BM = 128;
constexpr int T3_BK = 64;
constexpr int T3_THREADS = 192;   // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
template <int BN>
struct T3Cfg {
  static constexpr int STAGES = BN > 192 ? 4 : 5;
  static constexpr int A_BYTES = T3_BM * T3_BK * 2;
  static constexpr int B_BYTES = BN * T3_BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
  static constexpr int TMEM_COLS = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;   // per accumulator (two)
};

__device__ __forceinline__ int t3_sel(int code, int i, int j, int k) { return code == 0 ? i : (code == 1 ? j : k); }

// tile t -> (m-tile, n-tile, group, k - k0), m-tile fastest.  Group 0 comes
// first for every k of the run (its A operands belong to i and j only, so
// they stay in L2 across the k sweep); then groups 1 and 2 alternate per k
// (they share the A operands of k, and each keeps its i- or j-operands).
// With the group outermost of all, group 0's A panels were evicted between
// consecutive k and read again from HBM for every k.
struct T3Tile {
  int mt, nt, g, kq;
};
__device__ __forceinline__ T3Tile t3_tile(int t, int tm, int tn, int nk) {
  T3Tile r;
  const int per = tm * tn;
  const int q = t / per, rem = t - q * per;
  r.mt = rem % tm;
  r.nt = rem / tm;
  if (q < nk) {
    r.g = 0;
    r.kq = q;
  } else {
    const int q2 = q - nk;
    r.kq = q2 >> 1;
    r.g = 1 + (q2 & 1);
  }
  return r;
}

// Persistent: each CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...;
// the TMA thread streams the K segments of its tiles through a shared-memory
// ring, the MMA thread alternates two TMEM accumulators, and the epilogue
// warps store tile t while the MMAs of tile t+1 run.
template <int BN>
__global__ void __launch_bounds__(T3_THREADS, 1) gemm_t3_kernel(const __grid_constant__ T3Params P, int tm,
                                                                 int tn, int ntiles) {
  using Cfg = T3Cfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[Cfg::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[Cfg::STAGES];
  __shared__ __align__(8) uint64_t accf_bar[2];   // accumulator b holds a finished tile
  __shared__ __align__(8) uint64_t acce_bar[2];   // accumulator b has been read out
  __shared__ __align__(8) uint64_t done_bar;      // every issued MMA has completed
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_flag;
  __shared__ float epi_tile[4][32][33];

  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + Cfg::STAGES * Cfg::A_BYTES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t v = P.v, o = P.o;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::STAGES; ++s) {
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
                 "r"(2 * Cfg::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_holder;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer over the tiles' K segments
    int it = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
      const T3Tile tl = t3_tile(t, tm, tn, P.nk);
      const int kk = P.k0 + tl.kq;
      const int64_t m0 = (int64_t)tl.mt * T3_BM;
      for (int s = 0; s < T3_NSEG && !stop; ++s) {
        const T3Seg sg = P.seg[tl.g][s];
        const int32_t arow = (int32_t)(t3_sel(sg.asel, P.i, P.j, kk) * v * v + m0);
        const int32_t brow =
            (int32_t)((t3_sel(sg.bsel1, P.i, P.j, kk) * o + t3_sel(sg.bsel2, P.i, P.j, kk)) * v + (int64_t)tl.nt * BN);
        for (int kb = 0; kb < sg.nkb; ++kb, ++it) {
          const int st = it % Cfg::STAGES;
          const uint32_t ph = (it / Cfg::STAGES) & 1;
          if (!mbar_wait(smem_u32(&empty_bar[st]), ph ^ 1)) { atomicExch(&abort_flag, 1); stop = true; break; }
          if (*(volatile int*)&abort_flag) { stop = true; break; }
          const uint32_t fb = smem_u32(&full_bar[st]);
          mbar_expect_tx(fb, Cfg::STAGE_BYTES);
          tma_load_2d(smem_u32(sA + st * Cfg::A_BYTES), &P.maps[sg.amap], kb * T3_BK, arow, fb);
          tma_load_2d(smem_u32(sB + st * Cfg::B_BYTES), &P.maps[sg.bmap], kb * T3_BK, brow, fb);
        }
      }
    }
    if (stop) {
      // wait (bounded) for loads still in flight before shared memory is released
      for (int q = max(0, it - Cfg::STAGES); q < it; ++q)
        (void)mbar_wait(smem_u32(&full_bar[q % Cfg::STAGES]), (q / Cfg::STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = idesc_bf16(T3_BM, BN);
    int it = 0, lt = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
      const int g = t3_tile(t, tm, tn, P.nk).g;
      int total = 0;
      for (int s = 0; s < T3_NSEG; ++s) total += P.seg[g][s].nkb;
      const int b = lt & 1;
      if (!mbar_wait(smem_u32(&acce_bar[b]), ((lt >> 1) & 1) ^ 1)) { atomicExch(&abort_flag, 1); break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t dcol = tmem + (uint32_t)(b * Cfg::TMEM_COLS);
      for (int x = 0; x < total; ++x, ++it) {
        const int st = it % Cfg::STAGES;
        const uint32_t ph = (it / Cfg::STAGES) & 1;
        if (!mbar_wait(smem_u32(&full_bar[st]), ph)) { atomicExch(&abort_flag, 1); ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint64_t ad = sw128_desc(smem_u32(sA + st * Cfg::A_BYTES));
        const uint64_t bd = sw128_desc(smem_u32(sB + st * Cfg::B_BYTES));
#pragma unroll
        for (int q = 0; q < T3_BK / 16; ++q) {
          const uint32_t acc = (x > 0 || q > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
              "l"(ad + (uint64_t)(2 * q)), "l"(bd + (uint64_t)(2 * q)), "r"(idesc), "r"(acc)
              : "memory");
        }
        tc_commit(smem_u32(&empty_bar[st]));
      }
      if (!ok) break;
      tc_commit(smem_u32(&accf_bar[b]));
    }
    // TMEM is freed only after every issued MMA has completed (also on an abort)
    tc_commit(smem_u32(&done_bar));
    if (!mbar_wait(smem_u32(&done_bar), 0)) atomicExch(&abort_flag, 1);
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> transposed 32 x 32 blocks -> plain FP32 stores
    const int q = warp & 3;
    const int64_t v2 = v * v;
    float (*tile)[33] = epi_tile[q];
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const T3Tile tl = t3_tile(t, tm, tn, P.nk);
      const int b = lt & 1;
      bool ok = mbar_wait(smem_u32(&accf_bar[b]), (lt >> 1) & 1);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok || __any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) { atomicExch(&abort_flag, 1); break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int64_t m0 = (int64_t)tl.mt * T3_BM;
      const int64_t nbk = t3_nb(v);
      float* out = P.G + ((int64_t)tl.g * P.nk + tl.kq) * t3_slab(v);
      const int64_t nb0 = (int64_t)tl.nt * BN;
      // this lane's row (pair (x, y)) offset in the blocked layout; rows are
      // broadcast to the warp below
      int64_t myroff = 0;
      {
        const int64_t mr = m0 + q * 32 + lane;
        if (mr < v2) {
          const int x = (int)(mr / v), y = (int)(mr - (int64_t)x * v);
          myroff = t3_blk(x, y, 0, nbk);
        }
      }
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        if (nb0 + c0 >= v) break;
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * Cfg::TMEM_COLS + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        __syncwarp();
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) tile[lane][jj] = __uint_as_float(r[jj]);
        __syncwarp();
        const int64_t n = nb0 + c0 + lane;
        const int64_t coff = ((n >> 3) << 9) + (n & 7);   // lone index z = n within the (X, Y) block row
#pragma unroll 4
        for (int jr = 0; jr < 32; ++jr) {
          const int64_t roff = __shfl_sync(0xffffffffu, myroff, jr);
          const int64_t m = m0 + q * 32 + jr;
          if (m < v2 && n < v) out[roff + coff] = tile[jr][lane];
        }
      }
      // the accumulator is free for the tile after next
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&acce_bar[b]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * Cfg::TMEM_COLS)
                 : "memory");
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(P.err, 1);
}

template <int BN>
void launch_t3(const T3Params& P, cudaStream_t s) {
  using Cfg = T3Cfg<BN>;
  static std::once_flag once;
  std::call_once(once, []() {
    cudaFuncSetAttribute(gemm_t3_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
  });
  const int64_t tm = ((int64_t)P.v * P.v + T3_BM - 1) / T3_BM;
  const int64_t tn = (P.v + BN - 1) / BN;
  const int64_t ntiles = tm * tn * 3 * P.nk;
  if (ntiles > (int64_t)1 << 30) fail(FCC_ERR_BAD_ARG, "too many (T) tiles in one launch");
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, 152);
  gemm_t3_kernel<BN><<<grid, T3_THREADS, Cfg::SMEM, s>>>(P, (int)tm, (int)tn, (int)ntiles);
  FCC_CHECK_LAUNCH();
}

}  // namespace

int t3_bn(int v) {
  if (v <= 128) return 128;
  if (v <= 160) return 160;
  if (v <= 192) return 192;
  return 256;   // v > 256: several column tiles
}

void gemm_t3(const T3Params& P, cudaStream_t s) {
  if (P.nk <= 0) return;
  if (P.nk > 65535) fail(FCC_ERR_BAD_ARG, "too many k in one (T) launch");
  const double flops = 2.0 * 3.0 * (double)P.nk * (double)P.v * P.v * P.v *
                       (double)(P.seg[0][0].nkb + P.seg[0][1].nkb + P.seg[0][2].nkb + P.seg[0][3].nkb) * T3_BK;
  const int pidx = prof_begin(s);
  switch (P.bn) {
    case 128: launch_t3<128>(P, s); break;
    case 160: launch_t3<160>(P, s); break;
    case 192: launch_t3<192>(P, s); break;
    case 256: launch_t3<256>(P, s); break;
    default: fail(FCC_ERR_BAD_ARG, "no (T) tile width for this v");
  }
  prof_end(s, pidx, PROF_TC, flops);
}

}  // namespace fcc
