// Checkpoint files of the CC amplitudes: resume a long run, or keep converged
// amplitudes as training data or as the guess of a nearby geometry.
//
// Layout (little-endian): a 64-byte header
//   char   magic[8] = "FCCCKPT1"
//   int32  version = 1, o, v, naux
//   double correlation energy of the stored amplitudes, reference energy
//   int32  iterations done, converged (0/1), 4 x reserved (0)
// then T1 (o x v) and T2 (o x o x v x v), FP64, column-major (the Julia layout
// fcc_get_amps returns and fcc_set_guess takes).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "fcc_ctx.cuh"

namespace fcc {

namespace {

struct CkptHeader {
  char magic[8];
  int32_t version, o, v, naux;
  double ecc, e_ref;
  int32_t iterations, converged;
  int32_t reserved[4];
};
static_assert(sizeof(CkptHeader) == 64, "checkpoint header must be 64 bytes");

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) std::fclose(f);
  }
};

// row-major device tensor -> column-major host array
void to_host_colmajor(fcc_ctx* c, const double* dev, std::initializer_list<int64_t> dims, std::vector<double>& out) {
  int64_t n = 1;
  for (int64_t d : dims) n *= d;
  DBuf<double> tmp;
  tmp.alloc(n);
  TView src = rm(const_cast<double*>(dev), dims);
  TView dst = cm(tmp.p, dims);
  const char* spec = src.rank == 2 ? "ab->ab" : "abcd->abcd";
  einsum1(1.0, spec, src, 0.0, dst, c->stream);
  out.resize(n);
  FCC_CUDA(cudaMemcpyAsync(out.data(), tmp.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  FCC_CUDA(cudaStreamSynchronize(c->stream));
}

// column-major host array -> row-major device tensor
void from_host_colmajor(fcc_ctx* c, const std::vector<double>& in, std::initializer_list<int64_t> dims, double* dev) {
  DBuf<double> tmp;
  tmp.alloc(in.size());
  FCC_CUDA(cudaMemcpyAsync(tmp.p, in.data(), sizeof(double) * in.size(), cudaMemcpyHostToDevice, c->stream));
  TView src = cm(tmp.p, dims);
  TView dst = rm(dev, dims);
  const char* spec = src.rank == 2 ? "ab->ab" : "abcd->abcd";
  einsum1(1.0, spec, src, 0.0, dst, c->stream);
  FCC_CUDA(cudaStreamSynchronize(c->stream));
}

}  // namespace

void checkpoint_write(fcc_ctx* c, const std::string& path, const double* t1, const double* t2, double ecc,
                      int32_t iterations, int32_t converged) {
  const int64_t o = c->o, v = c->v;
  std::vector<double> h1, h2;
  to_host_colmajor(c, t1, {o, v}, h1);
  to_host_colmajor(c, t2, {o, o, v, v}, h2);
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, "FCCCKPT1", 8);
  h.version = 1;
  h.o = (int32_t)o;
  h.v = (int32_t)v;
  h.naux = (int32_t)c->Q;
  h.ecc = ecc;
  h.e_ref = c->e_ref;
  h.iterations = iterations;
  h.converged = converged;
  // write to a temporary name, then rename: a crash mid-write keeps the old file
  const std::string tmp = path + ".tmp";
  {
    std::unique_ptr<FILE, FileCloser> f(std::fopen(tmp.c_str(), "wb"));
    if (!f) fail(FCC_ERR_BAD_ARG, "cannot open checkpoint file for writing: " + tmp);
    if (std::fwrite(&h, sizeof(h), 1, f.get()) != 1 || std::fwrite(h1.data(), sizeof(double), h1.size(), f.get()) != h1.size() ||
        std::fwrite(h2.data(), sizeof(double), h2.size(), f.get()) != h2.size())
      fail(FCC_ERR_BAD_ARG, "cannot write checkpoint file: " + tmp);
    if (std::fflush(f.get()) != 0) fail(FCC_ERR_BAD_ARG, "cannot write checkpoint file: " + tmp);
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) fail(FCC_ERR_BAD_ARG, "cannot rename checkpoint file to " + path);
}

}  // namespace fcc

namespace {

template <class F>
int ckpt_guard(fcc_ctx* c, F&& f) {
  try {
    c->last_error.clear();
    return f();
  } catch (const fcc::Error& e) {
    c->last_error = e.what;
    return e.code;
  } catch (const std::bad_alloc&) {
    c->last_error = "host allocation failed";
    return FCC_ERR_OOM;
  } catch (...) {
    c->last_error = "unexpected failure";
    return FCC_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

int fcc_checkpoint_save(fcc_ctx* c, const char* path) {
  if (!c || !path || !*path) return FCC_ERR_BAD_ARG;
  return ckpt_guard(c, [&]() {
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "no amplitudes yet");
    FCC_CUDA(cudaSetDevice(c->device));
    fcc::checkpoint_write(c, path, c->t1.p, c->t2.p, c->last_ecc, c->last_iters, c->last_converged);
    return FCC_OK;
  });
}

int fcc_checkpoint_load(fcc_ctx* c, const char* path) {
  if (!c || !path || !*path) return FCC_ERR_BAD_ARG;
  return ckpt_guard(c, [&]() {
    if (!c->have_ints) fcc::fail(FCC_ERR_STATE, "upload integrals first");
    FCC_CUDA(cudaSetDevice(c->device));
    std::unique_ptr<FILE, fcc::FileCloser> f(std::fopen(path, "rb"));
    if (!f) fcc::fail(FCC_ERR_BAD_ARG, std::string("cannot open checkpoint file: ") + path);
    fcc::CkptHeader h;
    if (std::fread(&h, sizeof(h), 1, f.get()) != 1 || std::memcmp(h.magic, "FCCCKPT1", 8) != 0 || h.version != 1)
      fcc::fail(FCC_ERR_BAD_ARG, std::string("not a checkpoint file: ") + path);
    if (h.o != c->o || h.v != c->v)
      fcc::fail(FCC_ERR_BAD_ARG, "checkpoint dimensions (o, v) differ from this context");
    const int64_t o = c->o, v = c->v;
    std::vector<double> h1(o * v), h2(o * o * v * v);
    if (std::fread(h1.data(), sizeof(double), h1.size(), f.get()) != h1.size() ||
        std::fread(h2.data(), sizeof(double), h2.size(), f.get()) != h2.size())
      fcc::fail(FCC_ERR_BAD_ARG, std::string("truncated checkpoint file: ") + path);
    for (double x : h1)
      if (!std::isfinite(x)) fcc::fail(FCC_ERR_NAN, "non-finite amplitudes in the checkpoint");
    for (double x : h2)
      if (!std::isfinite(x)) fcc::fail(FCC_ERR_NAN, "non-finite amplitudes in the checkpoint");
    fcc::from_host_colmajor(c, h1, {o, v}, c->t1.p);
    fcc::from_host_colmajor(c, h2, {o, o, v, v}, c->t2.p);
    c->have_guess = true;
    c->have_ccsd = false;
    return FCC_OK;
  });
}

int fcc_set_checkpoint(fcc_ctx* c, const char* path, int32_t every) {
  if (!c || every < 0 || (every > 0 && (!path || !*path))) return FCC_ERR_BAD_ARG;
  c->ckpt_path = every > 0 ? path : "";
  c->ckpt_every = every;
  return FCC_OK;
}

}  // extern "C"
