// Opt-in per-kernel-class timing with CUDA events on the launching stream
// (measurement support for the bench; off by default, no effect on results).
#include <mutex>

#include "fcc_common.cuh"

namespace fcc {

namespace {

struct Rec {
  cudaEvent_t a, b;
  int cls;
  double work;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

}  // namespace

bool prof_on() { return g_on; }

int prof_begin(cudaStream_t s) {
  if (!g_on) return -1;
  std::lock_guard<std::mutex> lk(g_mu);
  Rec r{take(), take(), 0, 0.0};
  if (!r.a || !r.b) return -1;
  cudaEventRecord(r.a, s);
  g_recs.push_back(r);
  return (int)g_recs.size() - 1;
}

void prof_end(cudaStream_t s, int idx, int cls, double work) {
  if (idx < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx >= (int)g_recs.size()) return;
  g_recs[idx].cls = cls;
  g_recs[idx].work = work;
  cudaEventRecord(g_recs[idx].b, s);
}

}  // namespace fcc

extern "C" {

int fcc_prof_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(fcc::g_mu);
  fcc::g_on = on != 0;
  return FCC_OK;
}

// out[4*c + 0] = launches, [1] = milliseconds, [2] = work units (flop or
// bytes), [3] = max single launch ms, for classes c < ncls; resets the log.
int fcc_prof_read(double* out, int32_t ncls) {
  if (!out || ncls < 1) return FCC_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(fcc::g_mu);
  for (int k = 0; k < 4 * ncls; ++k) out[k] = 0.0;
  for (auto& r : fcc::g_recs) {
    float ms = 0.0f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess &&
        r.cls >= 0 && r.cls < ncls) {
      out[4 * r.cls + 0] += 1.0;
      out[4 * r.cls + 1] += ms;
      out[4 * r.cls + 2] += r.work;
      if (ms > out[4 * r.cls + 3]) out[4 * r.cls + 3] = ms;
    }
    fcc::g_pool.push_back(r.a);
    fcc::g_pool.push_back(r.b);
  }
  fcc::g_recs.clear();
  return FCC_OK;
}

}  // extern "C"
