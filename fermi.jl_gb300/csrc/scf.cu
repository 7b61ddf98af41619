// DF-RHF Fock build on the device: the density-fitted build_fock! of Fermi
// (src/Methods/HartreeFock/RHF/RHFHelper.jl:88-93)
//   F[m,n] = H[m,n] + 2 sum_rs D[r,s] b[Q,m,n] b[Q,r,s] - sum_rs D[r,s] b[Q,m,r] b[Q,n,s]
// and the RHF electronic energy sum(D .* (H .+ F)) (RHFHelper.jl:65-67), with
// b[Q,mu,nu] = aoints["ERI"] resident in HBM for the whole SCF.
//
// Layout: b is kept exactly as Julia holds it, column-major [Q, mu, nu] (Q
// fastest), so row r = mu + nbf*nu of the flattened pair index is a contiguous
// run of naux values.
//   gamma[Q] = sum_r b[Q,r] D[r]        gamma_part/gamma_sum kernels below:
//                                        threads along Q read b coalesced, D[r]
//                                        is a broadcast; partial sums per row
//                                        chunk, summed in a fixed order.
//   J = 2 b^T gamma                     warp-per-row FP64 GEMV (rows contiguous).
//   Y[Q,m,s] = sum_r b[Q,m,r] D[r,s]    FP64 DMMA contraction, M = (Q,m) fused.
//   K[m,n] = sum_{Q,s} Y[Q,m,s] b[Q,n,s] FP64 DMMA contraction, split over K.
// The occupied-orbital form (D = Co Co^T, as every RHF iteration has) factors
// K through X[Q,m,i] = sum_r b[Q,m,r] Co[r,i], K = X X^T: 4 naux nbf^2 nocc
// flops instead of 4 naux nbf^3.
#include <algorithm>
#include <cmath>
#include <new>

#include "fcc_common.cuh"
#include "fcc_tc.cuh"

using fcc::cm;

struct fcc_scf {
  int device = 0;
  int64_t n = 0, Q = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  bool have_b = false;
  fcc::DBuf<double> b;                // b[Q, mu, nu], column-major
  fcc::DBuf<double> H, D, F, C, Y;    // nbf^2 matrices, occupied orbitals, K intermediate
  fcc::DBuf<double> gam, gpart, red;
  fcc::DBuf<double> f64ws;            // split-K partial sums of the FP64 contractions
};

namespace {

constexpr int GAMMA_THREADS = 128;

__global__ void gamma_part_kernel(const double* __restrict__ b, const double* __restrict__ D, int64_t Q, int64_t R,
                                  int64_t rows_per, double* __restrict__ part) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Q) return;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per, r1 = min(R, r0 + rows_per);
  double s0 = 0.0, s1 = 0.0;
  int64_t r = r0;
  for (; r + 1 < r1; r += 2) {
    s0 += b[r * Q + q] * D[r];
    s1 += b[(r + 1) * Q + q] * D[r + 1];
  }
  if (r < r1) s0 += b[r * Q + q] * D[r];
  part[(int64_t)blockIdx.y * Q + q] = s0 + s1;
}

__global__ void gamma_sum_kernel(const double* __restrict__ part, int64_t Q, int nchunks, double* __restrict__ gam) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Q) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += part[(int64_t)c * Q + q];
  gam[q] = s;
}

// sum(D .* (H .+ F)) over R elements: one block, fixed reduction order.
__global__ void rhf_energy_kernel(const double* __restrict__ D, const double* __restrict__ H,
                                  const double* __restrict__ F, int64_t R, double* __restrict__ out) {
  __shared__ double sh[1024];
  double s = 0.0;
  for (int64_t r = threadIdx.x; r < R; r += blockDim.x) s += D[r] * (H[r] + F[r]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

template <class Fn>
int guarded(fcc_scf* s, Fn&& f) {
  try {
    if (s) {
      s->last_error.clear();
      cudaError_t e = cudaSetDevice(s->device);
      if (e != cudaSuccess) { s->last_error = cudaGetErrorString(e); return FCC_ERR_CUDA; }
    }
    fcc::TcScope fp64_only(nullptr);   // every contraction here runs in FP64
    fcc::WorkspaceScope ws(s ? &s->f64ws : nullptr);
    return f();
  } catch (const fcc::Error& e) {
    if (s) s->last_error = e.what;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (s) s->last_error = "host allocation failed";
    return FCC_ERR_OOM;
  } catch (...) {
    if (s) s->last_error = "unexpected internal error";
    return FCC_ERR_CUDA;
  }
}

void check_finite(const double* p, int64_t n, const char* what) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) fcc::fail(FCC_ERR_BAD_ARG, std::string("non-finite ") + what);
}

// F = H + 2 J[D] (device H, D already in place); leaves F on the device.
void coulomb(fcc_scf* s) {
  const int64_t n = s->n, Q = s->Q, R = n * n;
  const int64_t qblocks = (Q + GAMMA_THREADS - 1) / GAMMA_THREADS;
  int64_t nchunks = std::max<int64_t>(1, std::min<int64_t>(R, (152 * 8 + qblocks - 1) / qblocks));
  const int64_t rows_per = (R + nchunks - 1) / nchunks;
  nchunks = (R + rows_per - 1) / rows_per;
  if (s->gpart.n < (size_t)(nchunks * Q)) s->gpart.alloc(nchunks * Q);
  gamma_part_kernel<<<dim3((unsigned)qblocks, (unsigned)nchunks), GAMMA_THREADS, 0, s->stream>>>(
      s->b.p, s->D.p, Q, R, rows_per, s->gpart.p);
  FCC_CHECK_LAUNCH();
  gamma_sum_kernel<<<(unsigned)qblocks, GAMMA_THREADS, 0, s->stream>>>(s->gpart.p, Q, (int)nchunks, s->gam.p);
  FCC_CHECK_LAUNCH();
  FCC_CUDA(cudaMemcpyAsync(s->F.p, s->H.p, sizeof(double) * R, cudaMemcpyDeviceToDevice, s->stream));
  fcc::einsum(2.0, "Qr,Q->r", cm(s->b.p, {Q, R}), cm(s->gam.p, {Q}), 1.0, cm(s->F.p, {R}), s->stream);
}

void finish(fcc_scf* s, double* F, double* eelec) {
  const int64_t R = s->n * s->n;
  if (eelec) {
    rhf_energy_kernel<<<1, 1024, 0, s->stream>>>(s->D.p, s->H.p, s->F.p, R, s->red.p);
    FCC_CHECK_LAUNCH();
    FCC_CUDA(cudaMemcpyAsync(eelec, s->red.p, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  }
  FCC_CUDA(cudaMemcpyAsync(F, s->F.p, sizeof(double) * R, cudaMemcpyDeviceToHost, s->stream));
  FCC_CUDA(cudaStreamSynchronize(s->stream));
}

}  // namespace

extern "C" {

const char* fcc_scf_last_error(const fcc_scf* s) { return s ? s->last_error.c_str() : ""; }

int fcc_scf_create(fcc_scf** out, int32_t nbf, int32_t naux, int32_t device) {
  if (!out) return FCC_ERR_BAD_ARG;
  *out = nullptr;
  if (nbf <= 0 || naux <= 0) return FCC_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return FCC_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FCC_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) return FCC_ERR_NO_DEVICE;
  fcc_scf* s = new (std::nothrow) fcc_scf();
  if (!s) return FCC_ERR_OOM;
  s->device = device;
  s->n = nbf;
  s->Q = naux;
  int rc = guarded(s, [&]() {
    FCC_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    const int64_t R = s->n * s->n;
    s->b.alloc(s->Q * R);
    s->H.alloc(R);
    s->D.alloc(R);
    s->F.alloc(R);
    s->gam.alloc(s->Q);
    s->red.alloc(1);
    return FCC_OK;
  });
  if (rc != FCC_OK) {
    cudaStream_t st = s->stream;
    delete s;
    if (st) cudaStreamDestroy(st);
    return rc;
  }
  *out = s;
  return FCC_OK;
}

void fcc_scf_destroy(fcc_scf* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaStream_t st = s->stream;
  delete s;
  if (st) cudaStreamDestroy(st);
}

int fcc_scf_upload_b(fcc_scf* s, const double* Bmn) {
  if (!s) return FCC_ERR_BAD_ARG;
  return guarded(s, [&]() {
    if (!Bmn) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    const int64_t count = s->Q * s->n * s->n;
    check_finite(Bmn, count, "three-index factor");
    FCC_CUDA(cudaMemcpyAsync(s->b.p, Bmn, sizeof(double) * count, cudaMemcpyHostToDevice, s->stream));
    FCC_CUDA(cudaStreamSynchronize(s->stream));
    s->have_b = true;
    return FCC_OK;
  });
}

int fcc_scf_fit(fcc_scf* s, const double* Pqp, const double* Jh) {
  if (!s) return FCC_ERR_BAD_ARG;
  return guarded(s, [&]() {
    if (!Pqp || !Jh) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    const int64_t n = s->n, Q = s->Q;
    check_finite(Jh, Q * Q, "fitting metric");
    fcc::DBuf<double> dP, dJ;
    dP.alloc(n * n * Q);
    dJ.alloc(Q * Q);
    FCC_CUDA(cudaMemcpyAsync(dP.p, Pqp, sizeof(double) * n * n * Q, cudaMemcpyHostToDevice, s->stream));
    FCC_CUDA(cudaMemcpyAsync(dJ.p, Jh, sizeof(double) * Q * Q, cudaMemcpyHostToDevice, s->stream));
    // AtomicIntegrals.jl:37-38: b[Q,p,q] = sum_P Pqp[p,q,P] Jh[P,Q]
    fcc::einsum(1.0, "pqP,PQ->Qpq", cm(dP.p, {n, n, Q}), cm(dJ.p, {Q, Q}), 0.0, cm(s->b.p, {Q, n, n}), s->stream);
    FCC_CUDA(cudaStreamSynchronize(s->stream));
    s->have_b = true;
    return FCC_OK;
  });
}

int fcc_scf_build_fock(fcc_scf* s, const double* H, const double* D, double* F, double* eelec) {
  if (!s) return FCC_ERR_BAD_ARG;
  return guarded(s, [&]() {
    if (!H || !D || !F) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    if (!s->have_b) fcc::fail(FCC_ERR_STATE, "no three-index factors: call fcc_scf_upload_b or fcc_scf_fit first");
    const int64_t n = s->n, Q = s->Q, R = n * n;
    check_finite(H, R, "core Hamiltonian");
    check_finite(D, R, "density");
    FCC_CUDA(cudaMemcpyAsync(s->H.p, H, sizeof(double) * R, cudaMemcpyHostToDevice, s->stream));
    FCC_CUDA(cudaMemcpyAsync(s->D.p, D, sizeof(double) * R, cudaMemcpyHostToDevice, s->stream));
    coulomb(s);
    if (s->Y.n < (size_t)(Q * R)) s->Y.alloc(Q * R);
    fcc::einsum(1.0, "Qmr,rs->Qms", cm(s->b.p, {Q, n, n}), cm(s->D.p, {n, n}), 0.0, cm(s->Y.p, {Q, n, n}),
                s->stream);
    fcc::einsum(-1.0, "Qms,Qns->mn", cm(s->Y.p, {Q, n, n}), cm(s->b.p, {Q, n, n}), 1.0, cm(s->F.p, {n, n}),
                s->stream);
    finish(s, F, eelec);
    return FCC_OK;
  });
}

int fcc_scf_build_fock_occ(fcc_scf* s, const double* H, const double* Co, int32_t nocc, double* F, double* eelec) {
  if (!s) return FCC_ERR_BAD_ARG;
  return guarded(s, [&]() {
    if (!H || !Co || !F) fcc::fail(FCC_ERR_BAD_ARG, "null input");
    if (nocc <= 0 || nocc > s->n) fcc::fail(FCC_ERR_BAD_ARG, "nocc out of range");
    if (!s->have_b) fcc::fail(FCC_ERR_STATE, "no three-index factors: call fcc_scf_upload_b or fcc_scf_fit first");
    const int64_t n = s->n, Q = s->Q, R = n * n, o = nocc;
    check_finite(H, R, "core Hamiltonian");
    check_finite(Co, n * o, "occupied orbitals");
    if (s->C.n < (size_t)(n * o)) s->C.alloc(n * o);
    FCC_CUDA(cudaMemcpyAsync(s->H.p, H, sizeof(double) * R, cudaMemcpyHostToDevice, s->stream));
    FCC_CUDA(cudaMemcpyAsync(s->C.p, Co, sizeof(double) * n * o, cudaMemcpyHostToDevice, s->stream));
    // D[u,v] = Co[u,m] Co[v,m] (RHFa.jl:119, :147)
    fcc::einsum(1.0, "ui,vi->uv", cm(s->C.p, {n, o}), cm(s->C.p, {n, o}), 0.0, cm(s->D.p, {n, n}), s->stream);
    coulomb(s);
    if (s->Y.n < (size_t)(Q * n * o)) s->Y.alloc(Q * n * o);
    fcc::einsum(1.0, "Qmr,ri->Qmi", cm(s->b.p, {Q, n, n}), cm(s->C.p, {n, o}), 0.0, cm(s->Y.p, {Q, n, o}),
                s->stream);
    fcc::einsum(-1.0, "Qmi,Qni->mn", cm(s->Y.p, {Q, n, o}), cm(s->Y.p, {Q, n, o}), 1.0, cm(s->F.p, {n, n}),
                s->stream);
    finish(s, F, eelec);
    return FCC_OK;
  });
}

}  // extern "C"
