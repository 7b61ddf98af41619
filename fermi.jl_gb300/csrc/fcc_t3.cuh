// The (T) tensor-core GEMM: three orientation groups of four K segments each
// (see gemm_t3.cu), one launch per pair (i, j) and run of k.
#pragma once
#include <cuda.h>

#include "fcc_common.cuh"

namespace fcc {

constexpr int T3_NSEG = 4;

// One K segment: A rows sel(asel)*v*v + m (packed operand maps[amap]),
// B rows (sel(bsel1)*o + sel(bsel2))*v + n (maps[bmap]), nkb 64-column
// blocks; sel codes 0 = i, 1 = j, 2 = k.
struct T3Seg {
  int8_t amap, asel, bmap, bsel1, bsel2;
  int16_t nkb;
};

struct T3Params {
  CUtensorMap maps[7];
  T3Seg seg[3][T3_NSEG];
  int i, j, k0, nk, o, v;
  int bn;      // B tile width: 128, 160, 192 or 256 (t3_bn(v) unless set for a test)
  float* G;    // G[g][k - k0] FP32 in 8 x 8 x 8 sub-cube blocks (t3_blk)
  int* err;    // set to 1 if a bounded wait gave up
};

// Layout of one G_g[k] slab over (pair first index x, pair second index y,
// lone index z): 8 x 8 x 8 sub-cubes, each 512 contiguous floats, blocks
// ordered (X, Y, Z) with nb = ceil(v / 8) per index; the energy kernel reads
// whole sub-cubes with 2 KB loads.
__host__ __device__ constexpr int64_t t3_nb(int64_t v) { return (v + 7) / 8; }
__host__ __device__ constexpr int64_t t3_slab(int64_t v) { return t3_nb(v) * t3_nb(v) * t3_nb(v) * 512; }
__device__ __forceinline__ int64_t t3_blk(int x, int y, int z, int64_t nb) {
  return ((((int64_t)(x >> 3) * nb + (y >> 3)) * nb + (z >> 3)) << 9) + ((x & 7) << 6) + ((y & 7) << 3) + (z & 7);
}

// the B tile width used for v virtuals (256 with several column tiles above 256)
int t3_bn(int v);
void gemm_t3(const T3Params& P, cudaStream_t s);

}  // namespace fcc
