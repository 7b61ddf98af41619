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
