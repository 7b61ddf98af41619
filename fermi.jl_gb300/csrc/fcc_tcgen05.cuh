// Device helpers shared by the tcgen05 GEMM kernels: shared-memory
// addresses, bounded mbarrier waits, TMA 2-D tile loads, shared-memory matrix
// descriptors (128-byte swizzle) and the kind::f16 instruction descriptor.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

namespace fcc {
namespace tc5 {

constexpr uint64_t WAIT_NS = 2000000000ull;  // every mbarrier wait gives up after 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase; false after WAIT_NS.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (it == 0) t0 = globaltimer();
    else if ((it & 63) == 0 && globaltimer() - t0 > WAIT_NS) return false;
  }
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* tm, int32_t x, int32_t y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row groups 1024 bytes apart (SBO), fixed version bits 46-48 = 0b001.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}


__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// (double)f * 2^e (negated if neg) by integer exponent arithmetic; FP32
// subnormals and results below the FP64 normal range give 0
__device__ __forceinline__ double f32_to_f64_scaled(float f, int e, bool neg) {
  const uint32_t b = __float_as_uint(f);
  const int ex = (int)((b >> 23) & 0xFF);
  if (ex == 0) return 0.0;
  int ne = ex - 127 + 1023 + e;
  if (ne <= 0) return 0.0;
  if (ne > 2046) ne = 2047;
  const unsigned long long sign = (unsigned long long)((b >> 31) ^ (neg ? 1u : 0u)) << 63;
  const unsigned long long bits = sign | ((unsigned long long)ne << 52) | ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

// Output tile of linear block index lin on a tm x tn tile grid, walked in
// groups of 8 tile rows (row fastest inside a group) so that the CTAs resident
// at the same time share A and B panels in L2.
__device__ __forceinline__ void grouped_tile(int64_t lin, int64_t tm, int64_t tn, int64_t& mt, int64_t& nt) {
  constexpr int64_t GM = 8;
  const int64_t per_group = GM * tn;
  const int64_t g = lin / per_group;
  const int64_t first = g * GM;
  const int64_t gm = tm - first < GM ? tm - first : GM;
  const int64_t r = lin - g * per_group;
  mt = first + r % gm;
  nt = r / gm;
}

}  // namespace tc5
}  // namespace fcc
