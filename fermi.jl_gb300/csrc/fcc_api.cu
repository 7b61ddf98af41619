// C ABI of libfermicc (declared in include/fermicc.h).  Every entry point
// converts internal failures into status codes; nothing aborts the caller.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "fcc_ctx.cuh"

using fcc::TView;
using fcc::cm;
using fcc::rm;
using fcc::slice;

namespace {

template <class F>
int guarded(fcc_ctx* c, F&& f) {
  try {
    if (c) {
      c->last_error.clear();
      cudaError_t e = cudaSetDevice(c->device);
      if (e != cudaSuccess) { c->last_error = cudaGetErrorString(e); return FCC_ERR_CUDA; }
    }
    fcc::WorkspaceScope ws(c ? &c->f64ws : nullptr);
    return f();
  } catch (const fcc::Error& e) {
    if (c) c->last_error = e.what;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (c) c->last_error = "host allocation failed";
    return FCC_ERR_OOM;
  } catch (...) {
    if (c) c->last_error = "unexpected internal error";
    return FCC_ERR_CUDA;
  }
}

// Host -> device copy of a column-major tensor into a strided device view.
void upload_view(fcc_ctx* c, const double* host, size_t count, const TView& src_shape, const TView& dst) {
  fcc::DBuf<double> tmp;
  tmp.alloc(count);
  FCC_CUDA(cudaMemcpyAsync(tmp.p, host, count * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  TView s = src_shape;
  s.p = tmp.p;
  std::string idx = "abcd";
  std::string spec = idx.substr(0, s.rank) + "->" + idx.substr(0, s.rank);
  fcc::einsum1(1.0, spec.c_str(), s, 0.0, dst, c->stream);
  FCC_CUDA(cudaStreamSynchronize(c->stream));
}

void download_view(fcc_ctx* c, const TView& src, const TView& dst_shape, double* host, size_t count) {
  fcc::DBuf<double> tmp;
  tmp.alloc(count);
  TView d = dst_shape;
  d.p = tmp.p;
  std::string idx = "abcd";
  std::string spec = idx.substr(0, d.rank) + "->" + idx.substr(0, d.rank);
  fcc::einsum1(1.0, spec.c_str(), src, 0.0, d, c->stream);
  FCC_CUDA(cudaMemcpyAsync(host, tmp.p, count * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  FCC_CUDA(cudaStreamSynchronize(c->stream));
}

bool finite_all(const double* p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

void common_tail(fcc_ctx* c, const double* eps_o, const double* eps_v, double e_ref) {
  const int64_t o = c->o, v = c->v;
  c->eps_h.assign(eps_o, eps_o + o);
  c->eps_h.insert(c->eps_h.end(), eps_v, eps_v + v);
  for (int64_t i = 0; i < o; ++i)
    for (int64_t a = 0; a < v; ++a)
      if (!(eps_o[i] < eps_v[a])) fcc::fail(FCC_ERR_BAD_ARG, "orbital energies: an occupied level is not below a virtual one");
  c->eps.alloc(o + v);
  FCC_CUDA(cudaMemcpyAsync(c->eps.p, c->eps_h.data(), sizeof(double) * (o + v), cudaMemcpyHostToDevice, c->stream));
  c->e_ref = e_ref;
  fcc::setup_integrals(c);
  fcc::make_mp2_guess(c);
  FCC_CUDA(cudaStreamSynchronize(c->stream));
  c->have_ints = true;
  c->have_guess = false;
  c->have_ccsd = false;
}

// b[Q,mu,nu] (device, column-major) -> c->B over the active MO range, then the
// common setup; Bmn (and t) are freed on return
int upload_ao_common(fcc_ctx* c, fcc::DBuf<double>& dB, const double* C, int32_t nbf, int32_t nmo, int32_t core,
                     int32_t ndocc, const double* eps, double e_ref) {
  const int64_t Q = c->Q, n = c->n;
  const int64_t nb = nbf;
  fcc::DBuf<double> dC, t;
  dC.alloc(nb * nmo);
  FCC_CUDA(cudaMemcpyAsync(dC.p, C, sizeof(double) * nb * nmo, cudaMemcpyHostToDevice, c->stream));
  // column-major views: b[Q, mu, nu] (Q fastest), C[mu, p] (mu fastest); active p in [core, core + n)
  TView b = cm(dB.p, {Q, nb, nb});
  TView Ca = slice(cm(dC.p, {nb, (int64_t)nmo}), 1, core, n);
  t.alloc(Q * nb * n);
  TView tv = rm(t.p, {Q, nb, n});
  fcc::einsum(1.0, "Qmn,nq->Qmq", b, Ca, 0.0, tv, c->stream);
  c->B.alloc(Q * n * n);
  fcc::einsum(1.0, "mp,Qmq->Qpq", Ca, tv, 0.0, rm(c->B.p, {Q, n, n}), c->stream);
  FCC_CUDA(cudaStreamSynchronize(c->stream));
  common_tail(c, eps + core, eps + ndocc, e_ref);
  return FCC_OK;
}

void check_ao_ranges(fcc_ctx* c, const void* a, const void* C, const double* eps, int32_t nbf, int32_t nmo, int32_t core,
                     int32_t ndocc, double e_ref) {
  if (!a || !C || !eps) fcc::fail(FCC_ERR_BAD_ARG, "null input");
  if (c->Q <= 0) fcc::fail(FCC_ERR_STATE, "context created with naux = 0 (conventional); use fcc_upload_conv");
  if (nbf <= 0 || nmo <= 0 || nmo > nbf || core < 0 || ndocc - core != c->o || ndocc + c->v > nmo)
    fcc::fail(FCC_ERR_BAD_ARG, "orbital ranges do not match the context (ndocc - core = o, ndocc + v <= nmo)");
  if (!finite_all(eps, nmo) || !std::isfinite(e_ref)) fcc::fail(FCC_ERR_BAD_ARG, "non-finite orbital or reference energy");
}


}  // namespace

extern "C" {

void fcc_default_opts(fcc_opts* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->max_iter = 50;
  p->diis = 1;
  p->ndiis = 3;
  p->diis_start = 3;
  p->diis_relax = 3;
  p->diis_prec = 32;
  p->precision = FCC_PREC_FP64;
  p->e_conv = 1e-10;
  p->max_rms = 1e-10;
  p->damp = 0.0;
  p->mixed_switch_rms = 1e-5;
}

const char* fcc_strerror(int code) {
  switch (code) {
    case FCC_OK: return "success";
    case FCC_ERR_BAD_ARG: return "invalid argument";
    case FCC_ERR_OOM: return "out of device memory";
    case FCC_ERR_CUDA: return "CUDA error";
    case FCC_NO_CONVERGE: return "CC equations did not converge";
    case FCC_ERR_NAN: return "non-finite amplitudes or energy";
    case FCC_ERR_TIMEOUT: return "a bounded device wait timed out";
    case FCC_ERR_STATE: return "call out of order";
    case FCC_ERR_NO_DEVICE: return "no usable sm_103 (GB300) device";
    default: return "unknown status";
  }
}

const char* fcc_last_error(const fcc_ctx* c) { return c ? c->last_error.c_str() : ""; }

int fcc_create(fcc_ctx** out, int32_t o, int32_t v, int32_t naux, int32_t device) {
  if (!out) return FCC_ERR_BAD_ARG;
  *out = nullptr;
  if (o <= 0 || v <= 0 || naux < 0) return FCC_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return FCC_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FCC_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) return FCC_ERR_NO_DEVICE;
  fcc_ctx* c = new (std::nothrow) fcc_ctx();
  if (!c) return FCC_ERR_OOM;
  c->device = device;
  c->o = o;
  c->v = v;
  c->Q = naux;
  c->n = (int64_t)o + v;
  int rc = guarded(c, [&]() {
    FCC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    return FCC_OK;
  });
  if (rc != FCC_OK) { delete c; return rc; }
  *out = c;
  return FCC_OK;
}

void fcc_destroy(fcc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  // DBuf members free themselves
  cudaStream_t s = c->stream;
  delete c;
  if (s) cudaStreamDestroy(s);
}

int fcc_upload_df(fcc_ctx* c, const double* Boo, const double* Bov, const double* Bvv, const double* eps_o,
                  const double* eps_v, double e_ref) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!Boo || !Bov || !Bvv || !eps_o || !eps_v) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    if (c->Q <= 0) fcc::fail(FCC_ERR_STATE, "context created with naux = 0 (conventional); use fcc_upload_conv");
    const int64_t o = c->o, v = c->v, Q = c->Q, n = c->n;
    if (!finite_all(eps_o, o) || !finite_all(eps_v, v) || !std::isfinite(e_ref))
      fcc::fail(FCC_ERR_BAD_ARG, "non-finite orbital or reference energy");
    c->B.alloc(Q * n * n);
    TView B = rm(c->B.p, {Q, n, n});
    auto blk = [&](int64_t r0, int64_t nr, int64_t c0, int64_t nc) { return slice(slice(B, 1, r0, nr), 2, c0, nc); };
    upload_view(c, Boo, Q * o * o, cm(nullptr, {Q, o, o}), blk(0, o, 0, o));
    upload_view(c, Bov, Q * o * v, cm(nullptr, {Q, o, v}), blk(0, o, o, v));
    upload_view(c, Bvv, Q * v * v, cm(nullptr, {Q, v, v}), blk(o, v, o, v));
    fcc::einsum1(1.0, "Qia->Qai", blk(0, o, o, v), 0.0, blk(o, v, 0, o), c->stream);
    common_tail(c, eps_o, eps_v, e_ref);
    return FCC_OK;
  });
}

// AO three-index factors and MO coefficients: the MO transform of
// DFERI.jl:15-69 (BOO, BOV, BVV from aoints["ERI"] and the orbitals) runs on
// the device as two FP64 contractions over the active orbital range,
//   t[Q,mu,q] = sum_nu b[Q,mu,nu] C[nu,q],   B[Q,p,q] = sum_mu C[mu,p] t[Q,mu,q],
// which yields the full factor (OO, OV, VO, VV blocks) at once.
// AO three-index integrals (pq|P) and the fitting metric J^-1/2: the fit of
// AtomicIntegrals.jl:37-38, b[Q,p,q] = sum_P (pq|P) [J^-1/2]_PQ, on the device,
// then the MO transform below.
int fcc_upload_ao3_df(fcc_ctx* c, const double* Pqp, const double* Jh, const double* C, int32_t nbf, int32_t nmo,
                      int32_t core, int32_t ndocc, const double* eps, double e_ref) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    check_ao_ranges(c, Pqp, C, eps, nbf, nmo, core, ndocc, e_ref);
    if (!Jh) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    const int64_t Q = c->Q, nb = nbf;
    fcc::DBuf<double> dB;
    {
      fcc::DBuf<double> dP, dJ;
      dP.alloc(nb * nb * Q);
      dJ.alloc(Q * Q);
      FCC_CUDA(cudaMemcpyAsync(dP.p, Pqp, sizeof(double) * nb * nb * Q, cudaMemcpyHostToDevice, c->stream));
      FCC_CUDA(cudaMemcpyAsync(dJ.p, Jh, sizeof(double) * Q * Q, cudaMemcpyHostToDevice, c->stream));
      dB.alloc(Q * nb * nb);
      // Pqp[p, q, P] and Jh[P, Q] column-major; b written column-major [Q, p, q]
      fcc::einsum(1.0, "pqP,PQ->Qpq", cm(dP.p, {nb, nb, Q}), cm(dJ.p, {Q, Q}), 0.0, cm(dB.p, {Q, nb, nb}), c->stream);
      FCC_CUDA(cudaStreamSynchronize(c->stream));
    }
    return upload_ao_common(c, dB, C, nbf, nmo, core, ndocc, eps, e_ref);
  });
}

int fcc_upload_ao_df(fcc_ctx* c, const double* Bmn, const double* C, int32_t nbf, int32_t nmo, int32_t core,
                     int32_t ndocc, const double* eps, double e_ref) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    check_ao_ranges(c, Bmn, C, eps, nbf, nmo, core, ndocc, e_ref);
    const int64_t Q = c->Q, nb = nbf;
    fcc::DBuf<double> dB;
    dB.alloc(Q * nb * nb);
    FCC_CUDA(cudaMemcpyAsync(dB.p, Bmn, sizeof(double) * Q * nb * nb, cudaMemcpyHostToDevice, c->stream));
    return upload_ao_common(c, dB, C, nbf, nmo, core, ndocc, eps, e_ref);
  });
}

// Conventional integrals: the full (pq|rs) over the active MOs is rebuilt
// from the six blocks and factorised exactly by a pivoted Cholesky
// decomposition (tolerance 1e-13 on the residual diagonal), which yields
// three-index factors B[Q,p,q] with (pq|rs) = sum_Q B[Q,p,q] B[Q,r,s]; the
// rest of the path is then the same as with density fitting.
int fcc_upload_conv(fcc_ctx* c, const double* OOOO, const double* OOOV, const double* OOVV, const double* OVOV,
                    const double* OVVV, const double* VVVV, const double* eps_o, const double* eps_v, double e_ref) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!OOOO || !OOOV || !OOVV || !OVOV || !OVVV || !VVVV || !eps_o || !eps_v) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    const int64_t o = c->o, v = c->v, n = c->n;
    if (n > 64) fcc::fail(FCC_ERR_BAD_ARG, "conventional path supports at most 64 active orbitals");
    const int64_t n2 = n * n;
    std::vector<double> g(n2 * n2, 0.0);
    auto G = [&](int64_t p, int64_t q, int64_t r, int64_t s) -> double& { return g[((p * n + q) * n + r) * n + s]; };
    struct Blk { const double* a; char k[4]; };
    Blk blks[6] = {{OOOO, {'o', 'o', 'o', 'o'}}, {OOOV, {'o', 'o', 'o', 'v'}}, {OOVV, {'o', 'o', 'v', 'v'}},
                   {OVOV, {'o', 'v', 'o', 'v'}}, {OVVV, {'o', 'v', 'v', 'v'}}, {VVVV, {'v', 'v', 'v', 'v'}}};
    for (auto& b : blks) {
      int64_t d[4], off[4];
      for (int k = 0; k < 4; ++k) { d[k] = b.k[k] == 'o' ? o : v; off[k] = b.k[k] == 'o' ? 0 : o; }
      for (int64_t x3 = 0; x3 < d[3]; ++x3)
        for (int64_t x2 = 0; x2 < d[2]; ++x2)
          for (int64_t x1 = 0; x1 < d[1]; ++x1)
            for (int64_t x0 = 0; x0 < d[0]; ++x0) {
              double val = b.a[((x3 * d[2] + x2) * d[1] + x1) * d[0] + x0];   // column-major
              int64_t p = x0 + off[0], q = x1 + off[1], r = x2 + off[2], s = x3 + off[3];
              G(p, q, r, s) = val; G(q, p, r, s) = val; G(p, q, s, r) = val; G(q, p, s, r) = val;
              G(r, s, p, q) = val; G(s, r, p, q) = val; G(r, s, q, p) = val; G(s, r, q, p) = val;
            }
    }
    if (!finite_all(g.data(), g.size())) fcc::fail(FCC_ERR_BAD_ARG, "non-finite integrals");
    // pivoted Cholesky of the n^2 x n^2 matrix V[(pq),(rs)]
    std::vector<double> diag(n2);
    for (int64_t x = 0; x < n2; ++x) diag[x] = g[x * n2 + x];
    std::vector<std::vector<double>> L;
    const double tol = 1e-13;
    while ((int64_t)L.size() < n2) {
      int64_t piv = std::max_element(diag.begin(), diag.end()) - diag.begin();
      double dmax = diag[piv];
      if (dmax < tol) break;
      std::vector<double> col(n2);
      for (int64_t x = 0; x < n2; ++x) {
        double s = g[x * n2 + piv];
        for (auto& l : L) s -= l[x] * l[piv];
        col[x] = s / std::sqrt(dmax);
      }
      for (int64_t x = 0; x < n2; ++x) diag[x] -= col[x] * col[x];
      diag[piv] = 0.0;
      L.push_back(std::move(col));
    }
    const int64_t Q = (int64_t)L.size();
    if (Q == 0) fcc::fail(FCC_ERR_BAD_ARG, "integrals are numerically zero");
    std::vector<double> Bh(Q * n2);
    for (int64_t q = 0; q < Q; ++q) std::memcpy(&Bh[q * n2], L[q].data(), sizeof(double) * n2);
    c->Q = Q;
    c->B.alloc(Q * n2);
    FCC_CUDA(cudaMemcpyAsync(c->B.p, Bh.data(), sizeof(double) * Q * n2, cudaMemcpyHostToDevice, c->stream));
    FCC_CUDA(cudaStreamSynchronize(c->stream));
    common_tail(c, eps_o, eps_v, e_ref);
    return FCC_OK;
  });
}

int fcc_set_guess(fcc_ctx* c, const double* T1, const double* T2) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "upload integrals first");
    if (!T1 && !T2) {  // back to the MP2 guess, built on the device
      fcc::make_mp2_guess(c);
      FCC_CUDA(cudaStreamSynchronize(c->stream));
      c->have_guess = false;
      c->have_ccsd = false;
      return FCC_OK;
    }
    if (!T1 || !T2) fcc::fail(FCC_ERR_BAD_ARG, "give both amplitudes or neither");
    const int64_t o = c->o, v = c->v;
    if (!finite_all(T1, o * v) || !finite_all(T2, o * o * v * v)) fcc::fail(FCC_ERR_NAN, "non-finite guess amplitudes");
    upload_view(c, T1, o * v, cm(nullptr, {o, v}), rm(c->t1.p, {o, v}));
    upload_view(c, T2, o * o * v * v, cm(nullptr, {o, o, v, v}), rm(c->t2.p, {o, o, v, v}));
    c->have_guess = true;
    c->have_ccsd = false;
    return FCC_OK;
  });
}

int fcc_ccsd_run(fcc_ctx* c, const fcc_opts* opts, fcc_iter_stats* log, int32_t log_cap, fcc_ccsd_result* out) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "upload integrals first");
    if (log_cap < 0 || (log_cap > 0 && !log)) fcc::fail(FCC_ERR_BAD_ARG, "bad log buffer");
    fcc_opts def;
    fcc_default_opts(&def);
    return fcc::ccsd_run(c, opts ? opts : &def, log, log_cap, out);
  });
}

int fcc_get_amps(fcc_ctx* c, double* T1, double* T2) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "no amplitudes yet");
    const int64_t o = c->o, v = c->v;
    if (T1) download_view(c, rm(c->t1.p, {o, v}), cm(nullptr, {o, v}), T1, o * v);
    if (T2) download_view(c, rm(c->t2.p, {o, o, v, v}), cm(nullptr, {o, o, v, v}), T2, o * o * v * v);
    return FCC_OK;
  });
}

int fcc_mp2_energy(fcc_ctx* c, double* e_corr) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!e_corr) fcc::fail(FCC_ERR_BAD_ARG, "null output");
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "upload integrals first");
    *e_corr = fcc::mp2_energy(c);
    return std::isfinite(*e_corr) ? FCC_OK : FCC_ERR_NAN;
  });
}

int fcc_triples(fcc_ctx* c, int32_t precision, double* et_out) {
  if (!c) return FCC_ERR_BAD_ARG;
  return guarded(c, [&]() {
    if (!et_out) fcc::fail(FCC_ERR_BAD_ARG, "null output");
    if (!c->have_ccsd) fcc::fail(FCC_ERR_STATE, "run CCSD before (T)");
    if (precision != FCC_PREC_FP64 && precision != FCC_PREC_MIXED)
      fcc::fail(FCC_ERR_BAD_ARG, "(T) precision must be FCC_PREC_FP64 or FCC_PREC_MIXED");
    *et_out = precision == FCC_PREC_FP64 ? fcc::triples_fp64(c) : fcc::triples_mixed(c);
    return std::isfinite(*et_out) ? FCC_OK : FCC_ERR_NAN;
  });
}

}  // extern "C"
