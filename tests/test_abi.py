"""The C ABI library: builds, loads, exports every declared symbol (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from fermicc import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return _lib.load()


def declared_functions(header="fermicc.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"\b(fcc_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions() + declared_functions("fermicc_testing.h")
    assert "fcc_ccsd_run" in names and "fcc_triples" in names
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from fermicc import _lib
    assert sorted(_lib.EXPORTS) == declared_functions()
    assert sorted(_lib.TEST_EXPORTS) == declared_functions("fermicc_testing.h")


def test_default_options_are_fermis(lib):
    from fermicc import _lib
    o = _lib.FccOpts()
    lib.fcc_default_opts(ctypes.byref(o))
    # src/Core/Options.jl:40-104
    assert (o.max_iter, o.diis, o.ndiis, o.diis_start, o.diis_relax) == (50, 1, 3, 3, 3)
    assert o.e_conv == 1e-10 and o.max_rms == 1e-10 and o.damp == 0.0 and o.diis_prec == 32
    assert o.precision == _lib.FCC_PREC_FP64


def test_status_strings(lib):
    from fermicc import _lib
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert lib.fcc_strerror(code)
    assert b"GB300" in lib.fcc_strerror(_lib.FCC_ERR_NO_DEVICE)


def test_bad_arguments_rejected_without_device(lib):
    from fermicc import _lib
    h = ctypes.c_void_p()
    assert lib.fcc_create(None, 5, 19, 84, 0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_create(ctypes.byref(h), 0, 19, 84, 0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_create(ctypes.byref(h), 5, -1, 84, 0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_upload_df(None, None, None, None, None, None, 0.0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_ccsd_run(None, None, None, 0, None) == _lib.FCC_ERR_BAD_ARG
    lib.fcc_destroy(None)


def test_no_cpu_fallback_without_gpu(lib):
    # with no usable sm_103 device the library refuses instead of computing elsewhere
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fermicc import _lib
    h = ctypes.c_void_p()
    assert lib.fcc_create(ctypes.byref(h), 5, 19, 84, 0) == _lib.FCC_ERR_NO_DEVICE


def test_scf_handle_rejects_bad_arguments_without_device(lib):
    from fermicc import _lib
    h = ctypes.c_void_p()
    assert lib.fcc_scf_create(None, 24, 84, 0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_scf_create(ctypes.byref(h), 0, 84, 0) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_scf_create(ctypes.byref(h), 24, 0, 0) == _lib.FCC_ERR_BAD_ARG
    rc = lib.fcc_scf_create(ctypes.byref(h), 24, 84, 0)
    if rc == 0:                                  # a GB300 is present
        lib.fcc_scf_destroy(h)
    else:
        assert rc == _lib.FCC_ERR_NO_DEVICE and not h.value
    assert lib.fcc_scf_build_fock(None, None, None, None, None) == _lib.FCC_ERR_BAD_ARG
    assert lib.fcc_scf_last_error(None) == b""
    lib.fcc_scf_destroy(None)
