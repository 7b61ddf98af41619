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
