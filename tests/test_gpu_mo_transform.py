"""The DF MO transform on the device (DFERI.jl:15-69) against the host one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 4])
def test_device_mo_transform_gives_the_same_ccsd(n):
    from fermicc import Options, RCCSD
    from fermicc.inputs import scf
    from fermicc.rccsd import Context
    inp = scf.water_inputs(n, seed=0, keep_ao=True)
    Options.reset()
    Options.set("cc_max_rms", 1e-9)
    Options.set("cc_e_conv", 1e-10)
    host = Context(inp)
    dev = Context(inp, mo_transform=True)
    fit = Context(inp, mo_transform=True, fit=True)
    assert abs(host.mp2_energy() - dev.mp2_energy()) < 1e-11
    assert abs(host.mp2_energy() - fit.mp2_energy()) < 1e-11
    fit.close()
    a = RCCSD.compute(inp, context=host)
    b = RCCSD.compute(inp, context=dev)
    assert a.converged and b.converged
    assert abs(a.energy - b.energy) < 1e-10
    assert np.abs(a.T2 - b.T2).max() < 1e-8
    host.close()
    dev.close()
    Options.reset()


def test_device_mo_transform_checks_the_orbital_ranges():
    from fermicc.inputs import scf
    from fermicc.options import FermiException
    from fermicc.rccsd import Context
    inp = scf.water_inputs(2, seed=0, keep_ao=True)
    inp.ao = dict(inp.ao, core=inp.ao["core"] + 1)     # o no longer matches
    with pytest.raises(FermiException, match="orbital ranges"):
        Context(inp, mo_transform=True)
