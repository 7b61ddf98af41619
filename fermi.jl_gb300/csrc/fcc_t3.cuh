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
  float* G;    // G[g][k - k0][v*v][v], FP32
  int* err;    // set to 1 if a bounded wait gave up
};

// the B tile width used for v virtuals (256 with several column tiles above 256)
int t3_bn(int v);
void gemm_t3(const T3Params& P, cudaStream_t s);

}  // namespace fcc
