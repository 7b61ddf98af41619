"""GPU (T) against the CPU oracle (ijk.jl restatement), through the C ABI."""
import numpy as np
import pytest

from conftest import inputs
from oracle import rccsd as R
from oracle import triples as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["conv1", "df2"])
def test_triples_fp64_matches_oracle(case):
    from fermicc import Options, RCCSD, RCCSDpT
    inp = inputs(1, df=False) if case == "conv1" else inputs(2)
    Options.reset()
    Options.set("cc_e_conv", 1e-10)
    Options.set("cc_max_rms", 1e-9)
    ccsd = RCCSD.compute(inp)
    pt = RCCSDpT.compute(ccsd, inp)
    I = inp.conv if inp.Bvv is None else R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    # the oracle (T) on the GPU's own converged amplitudes isolates the (T) kernel
    et = T.triples_ijk(ccsd.T1, ccsd.T2, I["OVVV"], I["OOOV"], I["OVOV"], inp.eps_o, inp.eps_v)
    assert abs(pt.correction - et) < 1e-10
    assert abs(pt.energy - (ccsd.energy + et)) < 1e-10
    assert pt.correction < 0


@pytest.mark.parametrize("case", ["conv1", "df2", "df4"])
def test_triples_mixed_close_to_fp64(case):
    # split-BF16 W with FP32 accumulation; the T1/denominator/energy parts stay FP64
    from fermicc import Options, RCCSD, RCCSDpT
    inp = {"conv1": lambda: inputs(1, df=False), "df2": lambda: inputs(2), "df4": lambda: inputs(4)}[case]()
    Options.reset()
    Options.set("cc_max_rms", 1e-8)
    Options.set("cc_e_conv", 1e-8)
    ccsd = RCCSD.compute(inp)
    e64 = RCCSDpT.compute(ccsd, inp).correction
    Options.set("pt_gpu_precision", "mixed")
    emx = RCCSDpT.compute(ccsd, inp).correction
    assert abs(emx - e64) < 1e-6
    assert abs(emx - e64) < 1e-4 * abs(e64)


def test_triples_mixed_column_tiles_give_the_same_energy():
    # (H2O)8 has v = 152: the default tile width 160 covers it in one column
    # tile; width 128 needs two.  Same products in the same K order: the
    # energies agree to rounding.
    from conftest import inputs
    from fermicc import Options, RCCSD, _lib
    from fermicc.rccsd import Context
    inp = inputs(8)
    Options.reset()
    Options.set("cc_gpu_precision", "mixed")
    Options.set("cc_max_iter", 2)
    ctx = Context(inp)
    RCCSD.compute(inp, context=ctx)
    lib = _lib.load()
    e160 = ctx.triples(_lib.FCC_PREC_MIXED)
    assert lib.fcc_test_set_t3_bn(ctx.h, 128) == 0
    e128 = ctx.triples(_lib.FCC_PREC_MIXED)
    assert lib.fcc_test_set_t3_bn(ctx.h, 0) == 0
    assert abs(e128 - e160) < 1e-11, (e128, e160)
    ctx.close()
    Options.reset()
