// Context of one coupled-cluster problem on one GPU: device tensors, stream,
// options and the iteration state.
#pragma once
#include "fcc_common.cuh"
#include "fcc_tc.cuh"

struct fcc_ctx {
  int device = 0;
  int64_t o = 0, v = 0, Q = 0, n = 0;
  double e_ref = 0.0;
  bool have_ints = false, have_guess = false, have_ccsd = false;
  cudaStream_t stream = nullptr;
  std::string last_error;
  std::vector<double> eps_h;  // o + v orbital energies (host copy)

  // three-index factors, full MO range (active occupied + virtual):
  //   B[Q][p][q] row-major (q fastest), undressed and T1-dressed
  fcc::DBuf<double> B, Bt;
  fcc::DBuf<double> eps;      // o + v
  fcc::DBuf<double> h;        // n x n: diag(eps) - G(B), the frozen-core-including one-body part
  fcc::DBuf<double> F;        // n x n dressed Fock
  fcc::DBuf<double> Xm, Ym, tmpnn;
  fcc::DBuf<double> ones;     // length max(o, Q)
  fcc::DBuf<double> gam;      // Q
  // constant integrals
  fcc::DBuf<double> ovov;     // (kc|ld)      [o][v][o][v]
  fcc::DBuf<double> Lldkc;    // 2(ld|kc)-(lc|kd)  [o][v][o][v]
  fcc::DBuf<double> Lt;       // 2(kc|ld)-(kd|lc)  [o][o][v][v] (energy)
  fcc::DBuf<double> V2;       // (kc|ld)           [k][l][c][d]
  // amplitudes and residuals
  fcc::DBuf<double> t1, t2;   // current amplitudes [o][v], [o][o][v][v]
  fcc::DBuf<double> r1, r2;   // residuals
  fcc::DBuf<double> u, P, Cint, Dint, Fring, Xo, Wslab, Xq, Yq, Fvv, Foo;
  // symmetric / antisymmetric pp-ladder: pair tables (int2), channels
  fcc::DBuf<int2> pairP_v, pairM_v, pairP_o, pairM_o;   // (x<=y) and (x<y) pairs, row-major
  fcc::DBuf<double> Tp, Tm, Wp, Wm, LXp, LXm;
  // the dressed factors Bt[Q][x][y] (x, y virtual) packed once per residual
  // for every block's (ac|bd) product (rows (x, y), K = Q): digit slices and
  // row exponents, or the split pieces in the A and in the B order
  fcc::DBuf<__nv_bfloat16> bvvA, bvvB;
  fcc::DBuf<int> bvvEx;
  // reductions
  fcc::DBuf<double> red;      // device scratch for scalar reductions
  fcc::DBuf<double> f64ws;    // split-K partial sums of the FP64 contractions
  int64_t ladder_block = 0;

  // DIIS storage (slots of vec + err for T1 and T2)
  fcc::DBuf<double> dvec1, dvec2;
  fcc::DBuf<float> derr1s, derr2s;
  fcc::DBuf<double> derr1d, derr2d;

  // split-BF16 tensor-core engine (mixed form) and its device error flag
  fcc::TcEngine tc;
  fcc::DBuf<int> dev_err;
  // the last run
  double last_ecc = 0.0;      // correlation energy of the current amplitudes
  int32_t last_iters = 0, last_converged = 0;
  // periodic checkpoint of fcc_ccsd_run (empty path: off)
  std::string ckpt_path;
  int32_t ckpt_every = 0;
  int t3_bn_override = 0;     // test hook: B tile width of the mixed (T) GEMM (0: by v)
  int t3_kc_override = 0;     // test hook: k values per mixed (T) launch (0: the default run length)
  // test hook, one shot: FCC_TEST_FAULT_NO_LOADS makes the next tensor-core
  // GEMM of a CCSD run issue no TMA loads (its bounded waits run out);
  // FCC_TEST_FAULT_NAN writes a NaN into the next doubles residual
  int test_fault = 0;

  // (T) scratch
  fcc::DBuf<double> ovvv, ooov, Wt;
};

namespace fcc {
void setup_integrals(fcc_ctx* c);
void make_mp2_guess(fcc_ctx* c);
double cc_energy(fcc_ctx* c, const double* t1, const double* t2);
double mp2_energy(fcc_ctx* c);
void residual(fcc_ctx* c);
int ccsd_run(fcc_ctx* c, const fcc_opts* opts, fcc_iter_stats* log, int32_t log_cap, fcc_ccsd_result* out);
// E(T) in FP64; with `subset`, the energies of those triplets (i >= j >= k)
// one by one into `each` instead (returns 0)
double triples_fp64(fcc_ctx* c, const std::vector<int3>* subset = nullptr, std::vector<double>* each = nullptr);
double triples_mixed(fcc_ctx* c);
// write amplitudes (device, row-major) to a checkpoint file (checkpoint.cu)
void checkpoint_write(fcc_ctx* c, const std::string& path, const double* t1, const double* t2, double ecc,
                      int32_t iterations, int32_t converged);
}  // namespace fcc
