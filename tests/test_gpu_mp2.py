"""DF-MP2 energy on the device against the restated reference pair loop."""
import pytest

from conftest import inputs
from oracle import rmp2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 4])
def test_df_mp2_energy_matches_the_reference_pair_loop(n):
    from fermicc import Options, RMP2, energy
    inp = inputs(n)
    ref = rmp2.rmp2_energy_df(inp.Bov, inp.eps_o, inp.eps_v)
    Options.reset()
    r = RMP2.compute(inp)
    assert abs(r.correlation - ref) < 1e-12 * max(1.0, abs(ref))
    assert abs(r.energy - (ref + inp.e_ref)) < 1e-10
    assert abs(energy("mp2", inp).correlation - r.correlation) < 1e-14


def test_mp2_is_the_cc_guess_energy():
    # the CC driver's guess energy is the MP2 energy of the same integrals
    from fermicc import Options, RCCSD, RMP2
    inp = inputs(2)
    Options.reset()
    Options.set("cc_max_iter", 1)
    cc = RCCSD.compute(inp)
    assert abs(cc.guessenergy - RMP2.compute(inp).energy) < 1e-10
    Options.reset()
