// Test hooks (include/fermicc_testing.h): one contraction on the device.
#include <cstring>

#include "../../include/fermicc_testing.h"
#include "fcc_ctx.cuh"

static cudaStream_t fcc_stream_of(const fcc_ctx* c) { return c->stream; }

namespace {

fcc::TView view_of(double* p, const int64_t* dims, int rank) {
  fcc::TView t;
  t.p = p;
  t.rank = rank;
  int64_t s = 1;
  for (int k = rank - 1; k >= 0; --k) { t.dim[k] = dims[k]; t.str[k] = s; s *= dims[k]; }
  return t;
}

int64_t count(const int64_t* dims, int rank) {
  int64_t n = 1;
  for (int k = 0; k < rank; ++k) n *= dims[k];
  return n;
}

}  // namespace

namespace fcc { int64_t launch_count(); }

extern "C" int64_t fcc_stat_launches(void) { return fcc::launch_count(); }

extern "C" void* fcc_stream(const fcc_ctx* c) { return c ? (void*)fcc_stream_of(c) : nullptr; }

extern "C" int fcc_test_set_t3_bn(fcc_ctx* c, int32_t bn) {
  if (!c || !(bn == 0 || bn == 128 || bn == 160 || bn == 192 || bn == 256)) return FCC_ERR_BAD_ARG;
  c->t3_bn_override = bn;
  return FCC_OK;
}

extern "C" int fcc_test_set_t3_kc(fcc_ctx* c, int32_t kc) {
  if (!c || kc < 0 || kc > 64) return FCC_ERR_BAD_ARG;
  c->t3_kc_override = kc;
  return FCC_OK;
}

extern "C" int fcc_test_inject(fcc_ctx* c, int32_t kind) {
  if (!c || !(kind == 0 || kind == FCC_TEST_FAULT_NO_LOADS || kind == FCC_TEST_FAULT_NAN)) return FCC_ERR_BAD_ARG;
  c->test_fault = kind;
  return FCC_OK;
}

extern "C" int fcc_test_triples_subset(fcc_ctx* c, const int32_t* ijk, int32_t n, double* e_each) {
  if (!c || !ijk || !e_each || n < 1) return FCC_ERR_BAD_ARG;
  try {
    FCC_CUDA(cudaSetDevice(c->device));
    if (!c->have_ccsd) return FCC_ERR_STATE;
    std::vector<int3> sub;
    for (int32_t q = 0; q < n; ++q) {
      const int i = ijk[3 * q], j = ijk[3 * q + 1], k = ijk[3 * q + 2];
      if (!(0 <= k && k <= j && j <= i && i < c->o)) return FCC_ERR_BAD_ARG;
      sub.push_back(make_int3(i, j, k));
    }
    std::vector<double> each;
    fcc::WorkspaceScope ws(&c->f64ws);
    fcc::TcScope fp64(nullptr);
    fcc::triples_fp64(c, &sub, &each);
    for (int32_t q = 0; q < n; ++q) e_each[q] = each[q];
    return FCC_OK;
  } catch (const fcc::Error& e) {
    c->last_error = e.what;
    return e.code;
  } catch (...) {
    return FCC_ERR_CUDA;
  }
}

extern "C" int fcc_test_contract(int32_t precision, const char* spec, const double* A, const int64_t* adims,
                                 int32_t arank, const double* B, const int64_t* bdims, int32_t brank, double* C,
                                 const int64_t* cdims, int32_t crank, double alpha, double beta) {
  try {
    if (!spec || !A || !B || !C || !adims || !bdims || !cdims || arank < 1 || arank > 4 || brank < 1 || brank > 4 ||
        crank < 1 || crank > 4)
      return FCC_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return FCC_ERR_NO_DEVICE;
    FCC_CUDA(cudaSetDevice(0));
    cudaStream_t s;
    FCC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SDel { cudaStream_t s; ~SDel() { cudaStreamDestroy(s); } } sdel{s};
    const int64_t na = count(adims, arank), nb = count(bdims, brank), nc = count(cdims, crank);
    fcc::DBuf<double> dA, dB, dC;
    dA.alloc(na); dB.alloc(nb); dC.alloc(nc);
    fcc::DBuf<int> err;
    err.alloc(1);
    FCC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    FCC_CUDA(cudaMemcpyAsync(dA.p, A, na * 8, cudaMemcpyHostToDevice, s));
    FCC_CUDA(cudaMemcpyAsync(dB.p, B, nb * 8, cudaMemcpyHostToDevice, s));
    FCC_CUDA(cudaMemcpyAsync(dC.p, C, nc * 8, cudaMemcpyHostToDevice, s));
    fcc::TcEngine eng;
    eng.enabled = precision != FCC_PREC_FP64;
    if (precision == 2) eng.scheme = fcc::SPLIT6;
    if (precision == 3 || (precision >= 12 && precision <= 19)) {
      eng.exact = true;
      eng.oz_groups = precision == 3 ? fcc::OZ_G_DEFAULT : precision - 10;
    } else if (precision < 0 || precision > 3) {
      return FCC_ERR_BAD_ARG;
    }
    eng.min_flops = 0.0;
    eng.min_dim = 1;
    eng.err = err.p;
    {
      fcc::TcScope scope(&eng);
      fcc::einsum(alpha, spec, view_of(dA.p, adims, arank), view_of(dB.p, bdims, brank), beta,
                  view_of(dC.p, cdims, crank), s);
    }
    if (precision != FCC_PREC_FP64 && eng.tc_calls != 1) return FCC_ERR_BAD_ARG;
    int herr = 0;
    FCC_CUDA(cudaMemcpyAsync(C, dC.p, nc * 8, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    return herr ? FCC_ERR_TIMEOUT : FCC_OK;
  } catch (const fcc::Error& e) {
    return e.code;
  } catch (...) {
    return FCC_ERR_CUDA;
  }
}

extern "C" int fcc_test_split3(const double* x, int64_t R, int64_t K, int32_t row_fastest, double scale,
                               uint16_t* out) {
  try {
    if (!x || !out || R < 1 || K < 1) return FCC_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return FCC_ERR_NO_DEVICE;
    FCC_CUDA(cudaSetDevice(0));
    cudaStream_t s;
    FCC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SDel { cudaStream_t s; ~SDel() { cudaStreamDestroy(s); } } sdel{s};
    // source R x K, row-major (k fastest) or column-major (r fastest); three
    // planes hi | mid | lo per packed row
    fcc::PackSpec ps;
    ps.R = R;
    ps.K = K;
    ps.P = 3;
    ps.Kp = 3 * K;
    ps.code = 0u | (1u << 2) | (2u << 4);
    ps.scale = scale;
    ps.rd2 = 1; ps.rd3 = R; ps.rs1 = 0; ps.rs2 = 0; ps.rs3 = row_fastest ? 1 : K;
    ps.kd2 = 1; ps.kd3 = K; ps.ks1 = 0; ps.ks2 = 0; ps.ks3 = row_fastest ? R : 1;
    fcc::DBuf<double> dx;
    fcc::DBuf<__nv_bfloat16> dy;
    dx.alloc(R * K);
    dy.alloc(R * 3 * K);
    FCC_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * R * K, cudaMemcpyHostToDevice, s));
    fcc::pack_split(dx.p, ps, dy.p, s);
    FCC_CUDA(cudaMemcpyAsync(out, dy.p, sizeof(uint16_t) * R * 3 * K, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    return FCC_OK;
  } catch (const fcc::Error& e) {
    return e.code;
  } catch (...) {
    return FCC_ERR_CUDA;
  }
}

extern "C" int fcc_test_pack_oz(const double* x, int64_t R, int64_t K, int32_t row_fastest, int32_t S, uint16_t* out,
                                int32_t* ex) {
  try {
    if (!x || !out || !ex || R < 1 || K < 1 || S < 1 || S > 8) return FCC_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return FCC_ERR_NO_DEVICE;
    FCC_CUDA(cudaSetDevice(0));
    cudaStream_t s;
    FCC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SDel { cudaStream_t s; ~SDel() { cudaStreamDestroy(s); } } sdel{s};
    fcc::PackSpec ps;
    ps.R = R;
    ps.K = K;
    ps.Kp = fcc::oz_kpad(K);
    ps.rd2 = 1; ps.rd3 = R; ps.rs1 = 0; ps.rs2 = 0; ps.rs3 = row_fastest ? 1 : K;
    ps.kd2 = 1; ps.kd3 = K; ps.ks1 = 0; ps.ks2 = 0; ps.ks3 = row_fastest ? R : 1;
    const int64_t n = R * S * ps.Kp;
    fcc::DBuf<double> dx;
    fcc::DBuf<__nv_bfloat16> dy;
    fcc::DBuf<int> dex;
    dx.alloc(R * K);
    dy.alloc(n);
    dex.alloc(R);
    FCC_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * R * K, cudaMemcpyHostToDevice, s));
    fcc::pack_oz(dx.p, ps, S, dy.p, dex.p, s);
    FCC_CUDA(cudaMemcpyAsync(out, dy.p, sizeof(uint16_t) * n, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaMemcpyAsync(ex, dex.p, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, s));
    FCC_CUDA(cudaStreamSynchronize(s));
    return FCC_OK;
  } catch (const fcc::Error& e) {
    return e.code;
  } catch (...) {
    return FCC_ERR_CUDA;
  }
}
