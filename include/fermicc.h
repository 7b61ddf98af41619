/*
 * fermicc.h -- C ABI of the GB300 coupled-cluster backend (libfermicc.so).
 *
 * This is the drop-in boundary for Fermi.jl's RCCSD / DF-RCCSD amplitude
 * iteration and RCCSD(T) correction.  Every entry point takes plain pointers
 * and sizes, returns an int status (0 = success, negative = error) and never
 * aborts the caller.  Arrays are COLUMN-MAJOR (Julia layout): the first index
 * is the fastest.  The library copies every input to the device during the
 * call and keeps no host pointer afterwards.
 *
 * Reference interfaces replaced (paths inside FermiQC/Fermi.jl v0.5.0):
 *   fcc_create / fcc_upload_df     RCCSD(moints, aoints, ::RCCSDa), DF overload,
 *                                  src/Methods/CoupledCluster/RCCSD/RCCSDa.jl:37-44
 *                                  (moints["BOO"], ["BOV"], ["BVV"], ["Fd"])
 *   fcc_upload_conv                the conventional overload, RCCSDa.jl:25-35
 *                                  (moints["OOOO"] .. ["VVVV"])
 *   fcc_set_guess                  RCCSD(moints, T1guess, T2guess, alg), RCCSDa.jl:92
 *                                  (without it: the MP2 guess of RCCSDa.jl:46-89)
 *   fcc_ccsd_run                   the iteration loop, RCCSDa.jl:92-244, with the
 *                                  equations of RCCSDHelper.jl:8-349 and DIIS.jl
 *   fcc_get_amps                   the T1 / T2 fields of struct RCCSD, RCCSD.jl:61-69
 *   fcc_triples                    RCCSDpT(ccsd, moints, ::ijk),
 *                                  src/Methods/CoupledCluster/PerturbativeTriples/ijk.jl:20-149
 *   fcc_strerror                   FermiException messages, src/Core/Options.jl:196-199
 *   fcc_upload_ao_df / _ao3_df     the DF fit and MO transform, AtomicIntegrals.jl:31-40,
 *                                  src/Core/Integrals/ROIntegrals/DFERI.jl:15-69
 *   fcc_mp2_energy                 RMP2_energy, src/Methods/MollerPlesset/RMP2/RMP2a.jl:91-140
 *   fcc_scf_build_fock(_occ)       build_fock! (DF), src/Methods/HartreeFock/RHF/RHFHelper.jl:88-93,
 *                                  and RHFEnergy, RHFHelper.jl:65-67
 */
#ifndef FERMICC_H
#define FERMICC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FCC_OK 0
#define FCC_ERR_BAD_ARG (-1)   /* invalid size, null pointer, bad option        */
#define FCC_ERR_OOM (-2)       /* device allocation failed                       */
#define FCC_ERR_CUDA (-3)      /* CUDA runtime error                             */
#define FCC_NO_CONVERGE (-4)   /* soft: max_iter reached, results still valid    */
#define FCC_ERR_NAN (-5)       /* non-finite amplitudes or energy detected       */
#define FCC_ERR_TIMEOUT (-6)   /* a bounded device wait gave up                  */
#define FCC_ERR_STATE (-7)     /* call out of order (e.g. triples before ccsd)   */
#define FCC_ERR_NO_DEVICE (-8) /* no usable sm_103 device                        */

/* arithmetic of the contractions */
#define FCC_PREC_FP64 0  /* FP64 throughout (the correctness form)                  */
#define FCC_PREC_MIXED 1 /* split-BF16 tensor-core contractions (3 products, FP32  */
                         /* accumulate) until rms < mixed_switch_rms, then exact-  */
                         /* slice BF16 products (Ozaki scheme, exact integer       */
                         /* accumulation) until the criteria hold, then the finish */
                         /* (mixed_finish): the run ends on an FP64-accurate       */
                         /* residual that meets e_conv / max_rms (the FP64 fixed   */
                         /* point); denominators, update, DIIS and energies are    */
                         /* FP64 throughout                                        */
#define FCC_PREC_EXACT 2 /* every residual from exact-slice products at 9 weight   */
                         /* groups (FP64-accurate contractions on the tensor cores)*/

/* finish of the mixed form (fcc_opts.mixed_finish) */
#define FCC_FINISH_EXACT 0 /* exact-slice products at 9 weight groups (default)   */
#define FCC_FINISH_FP64 1  /* FP64 (DMMA) contractions                             */

typedef struct fcc_ctx fcc_ctx;

/* Fermi's CC options (src/Core/Options.jl:40-104) plus the precision switch. */
typedef struct {
  int32_t max_iter;        /* cc_max_iter    (50)                              */
  int32_t diis;            /* cc_diis        (1)                               */
  int32_t ndiis;           /* cc_ndiis       (3)                               */
  int32_t diis_start;      /* diis_start     (3)                               */
  int32_t diis_relax;      /* cc_diis_relax  (3)                               */
  int32_t diis_prec;       /* diis_prec: 32 = "single" (default), 64 = "double" */
  int32_t precision;       /* FCC_PREC_FP64 (default), _MIXED or _EXACT        */
  int32_t mixed_finish;    /* FCC_FINISH_EXACT (default) or FCC_FINISH_FP64    */
  double e_conv;           /* cc_e_conv      (1e-10)                           */
  double max_rms;          /* cc_max_rms     (1e-10)                           */
  double damp;             /* cc_damp_ratio  (0.0)                             */
  double mixed_switch_rms; /* mixed form: leave 3-product BF16 at rms < this (1e-5) */
} fcc_opts;

/* One line of Fermi's iteration table (RCCSDa.jl:223). */
typedef struct {
  int32_t ite;
  int32_t diis;      /* 1 if this iteration extrapolated                */
  int32_t precision; /* residual of this iteration: 0 FP64, 1 split-BF16, */
                     /* 2 exact-slice BF16 (Ozaki scheme, 6-7 groups),   */
                     /* 3 exact-slice at 9 groups (FP64-accurate)        */
  int32_t pad;
  double energy;     /* correlation energy after the iteration          */
  double dE;
  double rms;        /* max(rms(dT1), rms(dT2))                         */
  double seconds;    /* device time of the iteration                    */
} fcc_iter_stats;

/* Fields of struct RCCSD (RCCSD.jl:61-69) except the amplitudes. */
typedef struct {
  double guessenergy; /* Eguess = E_cc(guess) + E_ref                   */
  double correlation; /* E_cc                                           */
  double energy;      /* E_cc + E_ref                                   */
  double e_conv;      /* last dE                                        */
  double t_conv;      /* last rms                                       */
  int32_t iterations;
  int32_t converged;
} fcc_ccsd_result;

void fcc_default_opts(fcc_opts* opts);

/* o active occupied, v active virtual, naux fitting functions (0 selects the
 * conventional path, which then needs fcc_upload_conv).  device = CUDA
 * ordinal; the device must be sm_103 (GB300). */
int fcc_create(fcc_ctx** out, int32_t o, int32_t v, int32_t naux, int32_t device);

/* Boo[Q,i,j] (naux x o x o), Bov[Q,i,a] (naux x o x v), Bvv[Q,a,b]
 * (naux x v x v), all column-major with Q fastest, frozen core already
 * removed; eps_o (o), eps_v (v) RHF orbital energies; e_ref the SCF energy. */
int fcc_upload_df(fcc_ctx* ctx, const double* Boo, const double* Bov, const double* Bvv,
                  const double* eps_o, const double* eps_v, double e_ref);

/* The MO transform on the device instead (DFERI.jl:15-69 replaced): Bmn is
 * Fermi's aoints["ERI"], b[Q,mu,nu] = sum_P (mu nu|P) [J^-1/2]_PQ
 * (AtomicIntegrals.jl:31-40), naux x nbf x nbf column-major; C the RHF
 * coefficients (nbf x nmo, column-major); the active occupied orbitals are
 * [core, ndocc) (core = drop_occ) and the virtuals [ndocc, ndocc + v); eps
 * the nmo orbital energies. */
int fcc_upload_ao_df(fcc_ctx* ctx, const double* Bmn, const double* C, int32_t nbf, int32_t nmo, int32_t core,
                     int32_t ndocc, const double* eps, double e_ref);

/* Both DF steps on the device: Pqp the AO three-index integrals (pq|P),
 * nbf x nbf x naux column-major, and Jh = J^-1/2 of the fitting metric
 * (naux x naux), from which b[Q,p,q] = sum_P (pq|P) Jh[P,Q]
 * (AtomicIntegrals.jl:37-38); then as fcc_upload_ao_df. */
int fcc_upload_ao3_df(fcc_ctx* ctx, const double* Pqp, const double* Jh, const double* C, int32_t nbf, int32_t nmo,
                      int32_t core, int32_t ndocc, const double* eps, double e_ref);

/* Conventional MO blocks in chemist's notation, column-major:
 * OOOO[i,j,k,l] = (ij|kl), OOOV[i,j,k,a], OOVV[i,j,a,b], OVOV[i,a,j,b],
 * OVVV[i,a,b,c], VVVV[a,b,c,d].  Intended for small molecules. */
int fcc_upload_conv(fcc_ctx* ctx, const double* OOOO, const double* OOOV, const double* OOVV,
                    const double* OVOV, const double* OVVV, const double* VVVV,
                    const double* eps_o, const double* eps_v, double e_ref);

/* Starting amplitudes T1[i,a] (o x v) and T2[i,j,a,b] (o x o x v x v).
 * Without this call the run starts from the MP2 guess; passing NULL for both
 * restores the MP2 guess (built on the device). */
int fcc_set_guess(fcc_ctx* ctx, const double* T1, const double* T2);

/* Run the CCSD iterations.  log may be NULL; otherwise up to log_cap lines are
 * written (one per iteration).  Returns FCC_NO_CONVERGE (with valid results)
 * when max_iter is reached. */
int fcc_ccsd_run(fcc_ctx* ctx, const fcc_opts* opts, fcc_iter_stats* log, int32_t log_cap,
                 fcc_ccsd_result* out);

/* Copy the current amplitudes to the host (either pointer may be NULL). */
int fcc_get_amps(fcc_ctx* ctx, double* T1, double* T2);

/* (T) correction from the converged amplitudes (FCC_PREC_FP64 or
 * FCC_PREC_MIXED); et_out receives E(T). */
int fcc_triples(fcc_ctx* ctx, int32_t precision, double* et_out);

/* DF-MP2 (or conventional MP2) correlation energy of the uploaded integrals:
 * sum_ijab (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_i + e_j - e_a - e_b), the
 * quantity RMP2_energy returns (MollerPlesset/RMP2/RMP2a.jl:91-140);
 * RMP2.energy = e_corr + the reference energy. */
int fcc_mp2_energy(fcc_ctx* ctx, double* e_corr);

/* ---- checkpoints ----------------------------------------------------------
 * Not in Fermi.jl, which restarts only through the guess arguments of
 * RCCSD(moints, T1guess, T2guess, alg) (RCCSDa.jl:92).  A checkpoint file is
 * a 64-byte header ("FCCCKPT1", version 1, o, v, naux as int32; correlation
 * and reference energy as double; iterations done and converged as int32;
 * 16 reserved bytes) followed by T1 (o x v) and T2 (o x o x v x v) in FP64,
 * column-major, little-endian.  Writes go to path + ".tmp" and are renamed
 * into place. */
/* write the current amplitudes */
int fcc_checkpoint_save(fcc_ctx* ctx, const char* path);
/* read a checkpoint of the same (o, v) as the starting amplitudes of the
 * next fcc_ccsd_run (as fcc_set_guess) */
int fcc_checkpoint_load(fcc_ctx* ctx, const char* path);
/* fcc_ccsd_run writes a checkpoint every `every` iterations and at its end
 * (every = 0: off) */
int fcc_set_checkpoint(fcc_ctx* ctx, const char* path, int32_t every);

/* ---- learned T2 initialiser ---------------------------------------------
 * A 16 -> 128 -> 128 -> 1 GELU MLP predicting the CCSD correction to each
 * MP2 doubles amplitude from per-element features; BF16 weights with FP32
 * master copies, trained by Adam on this GPU.  It only seeds the iteration
 * (the guess argument of RCCSD(moints, T1guess, T2guess, alg), RCCSDa.jl:92);
 * these entry points have no other counterpart in Fermi.jl. */
typedef struct fcc_mlp fcc_mlp;
int64_t fcc_mlp_num_params(void);
int fcc_mlp_create(fcc_mlp** out, int32_t device);
void fcc_mlp_destroy(fcc_mlp* m);
/* parameters: W1[128][16] b1[128] W2[128][128] b2[128] w3[128] b3 mu[16] sd[16] (FP32) */
int fcc_mlp_get_params(const fcc_mlp* m, float* params, int64_t n);
int fcc_mlp_set_params(fcc_mlp* m, const float* params, int64_t n);
/* append training samples (every stride-th element) from a converged CCSD on ctx */
int fcc_mlp_collect(fcc_mlp* m, fcc_ctx* ctx, int32_t stride);
/* the same restricted to the elements the guess corrects, |t_MP2| >= thresh
 * (kept in element order, so the sample set and its order are reproducible) */
int fcc_mlp_collect_ex(fcc_mlp* m, fcc_ctx* ctx, int32_t stride, double thresh);
/* number of samples collected so far */
int64_t fcc_mlp_num_samples(const fcc_mlp* m);
/* Adam steps on the collected samples (batches drawn with `seed`); loss_log
 * (may be NULL) receives one mean-squared error per step */
int fcc_mlp_train(fcc_mlp* m, int32_t steps, int32_t batch, double lr, uint64_t seed, double* loss_log);
/* gradient of the mean squared error for n host samples (n x 16 raw
 * features, targets); grad receives the trained parameters' gradients */
int fcc_mlp_grad(fcc_mlp* m, const float* X, const float* y, int32_t n, float* grad, double* loss);
/* T1 = 0 and T2 = MP2 + learned correction as the starting amplitudes of ctx
 * (the correction is applied where |t_MP2| >= 3e-4; the result is made
 * symmetric under (i,a) <-> (j,b)) */
int fcc_mlp_guess(fcc_ctx* ctx, const fcc_mlp* m);
/* same with the correction scaled by lam and applied where |t_MP2| >= thresh */
int fcc_mlp_guess_ex(fcc_ctx* ctx, const fcc_mlp* m, double lam, double thresh);

/* C = alpha * A.B + beta * C in FP64 on the DMMA pipe, split over K, for
 * callers that cannot allocate device memory (a framework that owns all
 * device memory through its own pool, or a path where cudaMalloc's implicit
 * device synchronisation is not acceptable).  This entry point has no
 * counterpart in Fermi.jl.  A (M x K, leading dimension lda), B (K x N, ldb)
 * and C (M x N, ldc) are ROW-MAJOR DEVICE arrays owned by the caller on the
 * current device; the work is queued on `stream` (a cudaStream_t of the
 * current device, NULL = legacy default stream; a stream of another device
 * gives FCC_ERR_BAD_ARG) and the call returns without synchronising.  It
 * allocates nothing: partial sums go to a fixed 16 MiB device array that
 * every GPU loading the library keeps until exit, so M * N must not exceed
 * 2^20 (FCC_ERR_BAD_ARG otherwise).  The first call on each device looks up
 * that array's device address and should be made before any stream capture.
 * Calls share the array: calls that overlap on the GPU race and must be
 * ordered by the caller. */
int fcc_gemm_f64_noalloc(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* stream);

/* ---- DF-RHF Fock build ----------------------------------------------------
 * Replaces build_fock!(F, H, D, ints::IntegralHelper{Float64,<:AbstractDFERI,
 * AtomicOrbitals}) (HartreeFock/RHF/RHFHelper.jl:88-93), called from the RHF
 * iterations (RHFa.jl:125, :150), and RHFEnergy (RHFHelper.jl:65-67).  The
 * handle keeps b[Q,mu,nu] (aoints["ERI"]) resident on the device for the
 * whole SCF; it is independent of an fcc_ctx. */
typedef struct fcc_scf fcc_scf;
int fcc_scf_create(fcc_scf** out, int32_t nbf, int32_t naux, int32_t device);
void fcc_scf_destroy(fcc_scf* s);
const char* fcc_scf_last_error(const fcc_scf* s);
/* b[Q,mu,nu], naux x nbf x nbf column-major (Fermi's aoints["ERI"] in DF mode) */
int fcc_scf_upload_b(fcc_scf* s, const double* Bmn);
/* the fit of AtomicIntegrals.jl:37-38 on the device instead: Pqp (pq|P)
 * nbf x nbf x naux and Jh = J^-1/2 naux x naux, both column-major */
int fcc_scf_fit(fcc_scf* s, const double* Pqp, const double* Jh);
/* F = H + 2 J[D] - K[D] for a density D (nbf x nbf, column-major, any
 * matrix); eelec (may be NULL) receives sum(D .* (H .+ F)) */
int fcc_scf_build_fock(fcc_scf* s, const double* H, const double* D, double* F, double* eelec);
/* the same for D = Co Co^T (Co: nbf x nocc occupied coefficients,
 * RHFa.jl:146-147), with K factored through Co: 4 naux nbf^2 nocc flops
 * instead of 4 naux nbf^3 */
int fcc_scf_build_fock_occ(fcc_scf* s, const double* H, const double* Co, int32_t nocc, double* F, double* eelec);

void fcc_destroy(fcc_ctx* ctx);
const char* fcc_strerror(int code);
/* Message of the last failing call on this context ("" if none). */
const char* fcc_last_error(const fcc_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* FERMICC_H */
