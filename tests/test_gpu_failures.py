"""Error paths of the device code, exercised without faulting the GPU.

* A tensor-core GEMM whose producer issues no TMA loads: nothing is in
  flight, the MMA thread's bounded mbarrier wait (2 s) gives up, the kernel
  frees its TMEM and returns, the device error flag turns into
  FCC_ERR_TIMEOUT, and the next run on the same context converges normally.
* A NaN written into the doubles residual before the fused device update:
  the update's energy and rms reductions carry it and the run reports
  FCC_ERR_NAN; the context stays usable.
"""
import ctypes

import pytest

from conftest import inputs

pytestmark = pytest.mark.gpu


def _opts(precision):
    from fermicc import _lib
    lib = _lib.load()
    o = _lib.FccOpts()
    lib.fcc_default_opts(ctypes.byref(o))
    o.precision = precision
    o.e_conv, o.max_rms, o.max_iter = 1e-9, 1e-8, 60
    return o


def _run(ctx, precision):
    from fermicc import _lib
    res = _lib.FccCCSDResult()
    rc = ctx.lib.fcc_ccsd_run(ctx.h, ctypes.byref(_opts(precision)), None, 0, ctypes.byref(res))
    return rc, res


@pytest.fixture(scope="module")
def reference_energy():
    from fermicc import _lib
    from fermicc.rccsd import Context
    ctx = Context(inputs(2))
    rc, res = _run(ctx, _lib.FCC_PREC_FP64)
    assert rc == 0 and res.converged
    ctx.close()
    return res.correlation


def test_bounded_wait_gives_up_and_the_context_recovers(reference_energy):
    from fermicc import _lib
    from fermicc.rccsd import Context
    ctx = Context(inputs(2))
    lib = ctx.lib
    assert lib.fcc_test_inject(ctx.h, _lib.FCC_TEST_FAULT_NO_LOADS) == 0
    rc, _ = _run(ctx, _lib.FCC_PREC_MIXED)
    assert rc == _lib.FCC_ERR_TIMEOUT
    # the same context, from the MP2 guess again: a normal mixed run
    assert lib.fcc_set_guess(ctx.h, None, None) == 0
    rc, res = _run(ctx, _lib.FCC_PREC_MIXED)
    assert rc == 0 and res.converged
    assert abs(res.correlation - reference_energy) < 1e-8
    ctx.close()


def test_nan_in_the_residual_is_reported_and_the_context_recovers(reference_energy):
    from fermicc import _lib
    from fermicc.rccsd import Context
    ctx = Context(inputs(2))
    lib = ctx.lib
    assert lib.fcc_test_inject(ctx.h, _lib.FCC_TEST_FAULT_NAN) == 0
    rc, _ = _run(ctx, _lib.FCC_PREC_FP64)
    assert rc == _lib.FCC_ERR_NAN
    assert lib.fcc_set_guess(ctx.h, None, None) == 0
    rc, res = _run(ctx, _lib.FCC_PREC_FP64)
    assert rc == 0 and res.converged
    assert abs(res.correlation - reference_energy) < 1e-10
    ctx.close()


def test_fault_kinds_are_checked():
    from fermicc import _lib
    from fermicc.rccsd import Context
    ctx = Context(inputs(1))
    assert ctx.lib.fcc_test_inject(ctx.h, 7) == _lib.FCC_ERR_BAD_ARG
    assert ctx.lib.fcc_test_inject(None, 1) == _lib.FCC_ERR_BAD_ARG
    ctx.close()
