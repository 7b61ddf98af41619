"""ctypes binding of libfermicc.so (the C ABI declared in include/fermicc.h).

The library is looked up next to the package (built in-tree by build.py).  A
missing library is an error: there is no CPU fallback for the
coupled-cluster path.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "libfermicc.so")

FCC_OK = 0
FCC_ERR_BAD_ARG = -1
FCC_ERR_OOM = -2
FCC_ERR_CUDA = -3
FCC_NO_CONVERGE = -4
FCC_ERR_NAN = -5
FCC_ERR_TIMEOUT = -6
FCC_ERR_STATE = -7
FCC_ERR_NO_DEVICE = -8
FCC_PREC_FP64 = 0
FCC_PREC_MIXED = 1
FCC_PREC_EXACT = 2
FCC_FINISH_EXACT = 0
FCC_FINISH_FP64 = 1
FCC_TEST_FAULT_NO_LOADS = 1
FCC_TEST_FAULT_NAN = 2

# every symbol include/fermicc.h declares, and the test hooks of include/fermicc_testing.h
EXPORTS = ("fcc_default_opts", "fcc_create", "fcc_upload_df", "fcc_upload_conv", "fcc_set_guess",
           "fcc_ccsd_run", "fcc_get_amps", "fcc_triples", "fcc_destroy", "fcc_strerror", "fcc_last_error",
           "fcc_gemm_f64_noalloc", "fcc_mlp_num_params", "fcc_mlp_create", "fcc_mlp_destroy", "fcc_mlp_get_params",
           "fcc_mlp_set_params", "fcc_mlp_collect", "fcc_mlp_collect_ex", "fcc_mlp_num_samples", "fcc_mlp_train",
           "fcc_mlp_grad", "fcc_mlp_guess",
           "fcc_mlp_guess_ex", "fcc_checkpoint_save", "fcc_checkpoint_load", "fcc_set_checkpoint",
           "fcc_mp2_energy", "fcc_upload_ao_df", "fcc_upload_ao3_df", "fcc_scf_create", "fcc_scf_destroy",
           "fcc_scf_last_error", "fcc_scf_upload_b", "fcc_scf_fit", "fcc_scf_build_fock", "fcc_scf_build_fock_occ")
TEST_EXPORTS = ("fcc_test_contract", "fcc_stat_launches", "fcc_stream", "fcc_prof_enable", "fcc_prof_read",
                "fcc_test_set_t3_bn", "fcc_test_split3", "fcc_test_pack_oz", "fcc_test_inject",
                "fcc_test_triples_subset", "fcc_test_set_t3_kc")


class FccOpts(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int32), ("diis", ctypes.c_int32), ("ndiis", ctypes.c_int32),
                ("diis_start", ctypes.c_int32), ("diis_relax", ctypes.c_int32), ("diis_prec", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("mixed_finish", ctypes.c_int32), ("e_conv", ctypes.c_double),
                ("max_rms", ctypes.c_double), ("damp", ctypes.c_double), ("mixed_switch_rms", ctypes.c_double)]


class FccIterStats(ctypes.Structure):
    _fields_ = [("ite", ctypes.c_int32), ("diis", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("energy", ctypes.c_double), ("dE", ctypes.c_double),
                ("rms", ctypes.c_double), ("seconds", ctypes.c_double)]


class FccCCSDResult(ctypes.Structure):
    _fields_ = [("guessenergy", ctypes.c_double), ("correlation", ctypes.c_double), ("energy", ctypes.c_double),
                ("e_conv", ctypes.c_double), ("t_conv", ctypes.c_double), ("iterations", ctypes.c_int32),
                ("converged", ctypes.c_int32)]


_lib = None


def load():
    """Load libfermicc.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libfermicc.so not found at {LIB_PATH}: run __graft_entry__.build() "
                           "(the coupled-cluster path has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    i32 = ctypes.c_int32
    lib.fcc_default_opts.argtypes = [ctypes.POINTER(FccOpts)]
    lib.fcc_default_opts.restype = None
    lib.fcc_create.argtypes = [ctypes.POINTER(vp), i32, i32, i32, i32]
    lib.fcc_upload_df.argtypes = [vp, dp, dp, dp, dp, dp, ctypes.c_double]
    lib.fcc_upload_conv.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_double]
    lib.fcc_set_guess.argtypes = [vp, dp, dp]
    lib.fcc_ccsd_run.argtypes = [vp, ctypes.POINTER(FccOpts), ctypes.POINTER(FccIterStats), i32,
                                 ctypes.POINTER(FccCCSDResult)]
    lib.fcc_get_amps.argtypes = [vp, dp, dp]
    lib.fcc_triples.argtypes = [vp, i32, dp]
    lib.fcc_destroy.argtypes = [vp]
    lib.fcc_destroy.restype = None
    lib.fcc_strerror.argtypes = [ctypes.c_int]
    lib.fcc_strerror.restype = ctypes.c_char_p
    lib.fcc_last_error.argtypes = [vp]
    lib.fcc_last_error.restype = ctypes.c_char_p
    i64p = ctypes.POINTER(ctypes.c_int64)
    lib.fcc_test_contract.argtypes = [i32, ctypes.c_char_p, dp, i64p, i32, dp, i64p, i32, dp, i64p, i32,
                                      ctypes.c_double, ctypes.c_double]
    lib.fcc_test_contract.restype = ctypes.c_int
    lib.fcc_stat_launches.argtypes = []
    lib.fcc_stat_launches.restype = ctypes.c_int64
    i64 = ctypes.c_int64
    lib.fcc_gemm_f64_noalloc.argtypes = [i64, i64, i64, ctypes.c_double, vp, i64, vp, i64, ctypes.c_double, vp, i64, vp]
    lib.fcc_gemm_f64_noalloc.restype = ctypes.c_int
    fp = ctypes.POINTER(ctypes.c_float)
    lib.fcc_mlp_num_params.argtypes = []
    lib.fcc_mlp_num_params.restype = i64
    lib.fcc_mlp_create.argtypes = [ctypes.POINTER(vp), i32]
    lib.fcc_mlp_destroy.argtypes = [vp]
    lib.fcc_mlp_destroy.restype = None
    lib.fcc_mlp_get_params.argtypes = [vp, fp, i64]
    lib.fcc_mlp_set_params.argtypes = [vp, fp, i64]
    lib.fcc_mlp_collect.argtypes = [vp, vp, i32]
    lib.fcc_mlp_collect_ex.argtypes = [vp, vp, i32, ctypes.c_double]
    lib.fcc_mlp_collect_ex.restype = ctypes.c_int
    lib.fcc_mlp_num_samples.argtypes = [vp]
    lib.fcc_mlp_num_samples.restype = i64
    lib.fcc_mlp_train.argtypes = [vp, i32, i32, ctypes.c_double, ctypes.c_uint64, dp]
    lib.fcc_mlp_grad.argtypes = [vp, fp, fp, i32, fp, dp]
    lib.fcc_mlp_guess.argtypes = [vp, vp]
    lib.fcc_mlp_guess_ex.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double]
    lib.fcc_mlp_guess_ex.restype = ctypes.c_int
    for name in ("fcc_mlp_create", "fcc_mlp_get_params", "fcc_mlp_set_params", "fcc_mlp_collect", "fcc_mlp_train",
                 "fcc_mlp_grad", "fcc_mlp_guess"):
        getattr(lib, name).restype = ctypes.c_int
    lib.fcc_prof_enable.argtypes = [i32]
    lib.fcc_prof_enable.restype = ctypes.c_int
    lib.fcc_prof_read.argtypes = [dp, i32]
    lib.fcc_prof_read.restype = ctypes.c_int
    lib.fcc_test_set_t3_bn.argtypes = [vp, i32]
    lib.fcc_test_set_t3_bn.restype = ctypes.c_int
    lib.fcc_test_split3.argtypes = [dp, i64, i64, i32, ctypes.c_double, ctypes.POINTER(ctypes.c_uint16)]
    lib.fcc_test_split3.restype = ctypes.c_int
    lib.fcc_test_pack_oz.argtypes = [dp, i64, i64, i32, i32, ctypes.POINTER(ctypes.c_uint16),
                                     ctypes.POINTER(ctypes.c_int32)]
    lib.fcc_test_pack_oz.restype = ctypes.c_int
    lib.fcc_test_set_t3_kc.argtypes = [vp, i32]
    lib.fcc_test_set_t3_kc.restype = ctypes.c_int
    lib.fcc_test_inject.argtypes = [vp, i32]
    lib.fcc_test_inject.restype = ctypes.c_int
    lib.fcc_test_triples_subset.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), i32, dp]
    lib.fcc_test_triples_subset.restype = ctypes.c_int
    lib.fcc_stream.argtypes = [vp]
    lib.fcc_stream.restype = ctypes.c_void_p
    lib.fcc_mp2_energy.argtypes = [vp, dp]
    lib.fcc_upload_ao_df.argtypes = [vp, dp, dp, i32, i32, i32, i32, dp, ctypes.c_double]
    lib.fcc_upload_ao3_df.argtypes = [vp, dp, dp, dp, i32, i32, i32, i32, dp, ctypes.c_double]
    lib.fcc_checkpoint_save.argtypes = [vp, ctypes.c_char_p]
    lib.fcc_checkpoint_load.argtypes = [vp, ctypes.c_char_p]
    lib.fcc_set_checkpoint.argtypes = [vp, ctypes.c_char_p, i32]
    lib.fcc_scf_create.argtypes = [ctypes.POINTER(vp), i32, i32, i32]
    lib.fcc_scf_destroy.argtypes = [vp]
    lib.fcc_scf_destroy.restype = None
    lib.fcc_scf_last_error.argtypes = [vp]
    lib.fcc_scf_last_error.restype = ctypes.c_char_p
    lib.fcc_scf_upload_b.argtypes = [vp, dp]
    lib.fcc_scf_fit.argtypes = [vp, dp, dp]
    lib.fcc_scf_build_fock.argtypes = [vp, dp, dp, dp, dp]
    lib.fcc_scf_build_fock_occ.argtypes = [vp, dp, dp, i32, dp, dp]
    for name in ("fcc_scf_create", "fcc_scf_upload_b", "fcc_scf_fit", "fcc_scf_build_fock", "fcc_scf_build_fock_occ"):
        getattr(lib, name).restype = ctypes.c_int
    for name in ("fcc_create", "fcc_upload_df", "fcc_upload_conv", "fcc_set_guess", "fcc_ccsd_run",
                 "fcc_get_amps", "fcc_triples", "fcc_checkpoint_save", "fcc_checkpoint_load", "fcc_set_checkpoint", "fcc_mp2_energy",
                 "fcc_upload_ao_df", "fcc_upload_ao3_df"):
        getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib
