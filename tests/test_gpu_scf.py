"""DF-RHF Fock build on the device (csrc/scf.cu) against the restated
build_fock! (oracle/rhf.py, RHFHelper.jl:88-93), and the RHFcuda driver
against the restated RHFa iterations (RHFa.jl:67-203)."""
import functools

import numpy as np
import pytest

from oracle import rhf as orhf

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=None)
def _problem(n, seed=0):
    from fermicc.inputs import molecule, scf
    return scf.df_ao_problem(molecule.waters(n, seed), keep_pqp=True)


@pytest.mark.parametrize("n", [1, 2, 4])
def test_device_fock_equals_the_restated_build_fock(n):
    from fermicc import DFFock
    p = _problem(n)
    naux, nbf, _ = p.b.shape
    f = DFFock(nbf, naux, b=p.b)
    rng = np.random.default_rng(n)
    A = rng.standard_normal((nbf, nbf)) * 0.05
    for D in (A + A.T, A):                              # build_fock! takes any matrix
        F, e = f.build(p.H, D)
        ref = orhf.build_fock_df(p.H, D, p.b)
        scale = np.abs(ref).max()
        assert np.abs(F - ref).max() < 1e-12 * scale
        assert abs(e - orhf.rhf_energy(D, p.H, ref)) < 1e-12 * max(1.0, abs(e))
    # occupied-orbital form: the same Fock matrix for D = Co Co^T
    C, _ = orhf.gwh_guess(p.S, p.H)
    Co = C[:, :p.ndocc]
    F1, e1 = f.build(p.H, Co @ Co.T)
    F2, e2 = f.build_occ(p.H, Co)
    assert np.abs(F1 - F2).max() < 1e-12 * np.abs(F1).max()
    assert abs(e1 - e2) < 1e-11
    f.close()


def test_device_fit_equals_the_uploaded_factors():
    from fermicc import DFFock
    p = _problem(2)
    naux, nbf, _ = p.b.shape
    a = DFFock(nbf, naux, b=p.b)
    b = DFFock(nbf, naux, Pqp=p.Pqp, Jh=p.Jh)
    D = np.eye(nbf) * 0.2
    Fa, ea = a.build(p.H, D)
    Fb, eb = b.build(p.H, D)
    assert np.abs(Fa - Fb).max() < 1e-11 * np.abs(Fa).max()
    assert abs(ea - eb) < 1e-10
    a.close()
    b.close()


@pytest.mark.parametrize("n", [2, 4])
def test_rhfcuda_reaches_the_restated_rhfa_solution(n):
    from fermicc import DFFock, Options, RHF
    from fermicc.inputs import scf
    p = _problem(n)
    naux, nbf, _ = p.b.shape
    Options.reset()
    f = DFFock(nbf, naux, b=p.b)
    r = RHF.compute(p.H, p.S, p.ndocc, p.e_nuc, f)
    C, Lam = orhf.gwh_guess(p.S, p.H)
    o = orhf.rhf(p.H, p.S, p.ndocc, p.e_nuc, lambda H, D: orhf.build_fock_df(H, D, p.b), C, Lam)
    assert r.converged and o.converged
    assert abs(r.iterations - o.iterations) <= 1
    assert abs(r.energy - o.energy) < 1e-10
    assert np.abs(r.eps[:p.ndocc] - o.eps[:p.ndocc]).max() < 1e-7
    assert abs(r.energy - scf.water_inputs(n, seed=0).e_ref) < 1e-9
    f.close()


def test_scf_errors_are_reported():
    from fermicc import DFFock, FermiException
    p = _problem(1)
    naux, nbf, _ = p.b.shape
    f = DFFock(nbf, naux)                               # no factors yet
    with pytest.raises(FermiException, match="call out of order"):
        f.build(p.H, np.eye(nbf))
    f.close()
    f = DFFock(nbf, naux, b=p.b)
    H = p.H.copy()
    H[0, 0] = np.nan
    with pytest.raises(FermiException, match="invalid argument"):
        f.build(H, np.eye(nbf))
    with pytest.raises(FermiException, match="invalid argument"):
        f.build_occ(p.H, np.zeros((nbf, nbf + 1)))
    F, _ = f.build(p.H, np.zeros((nbf, nbf)))           # still usable after the errors
    assert np.array_equal(F, p.H)
    f.close()


def test_pipeline_with_the_device_rhf_gives_the_same_ccsd():
    # RHF (device Fock build) -> MO factors -> CCSD, against the host SCF
    from fermicc import Options, RCCSD
    from fermicc.inputs import scf
    host = scf.water_inputs(2, seed=0)
    dev = scf.water_inputs(2, seed=0, rhf_device=True)
    assert abs(dev.e_ref - host.e_ref) < 1e-9
    assert np.abs(dev.eps_o - host.eps_o).max() < 1e-7
    Options.reset()
    Options.set("cc_max_rms", 1e-9)
    a = RCCSD.compute(host)
    b = RCCSD.compute(dev)
    assert a.converged and b.converged
    assert abs(a.correlation - b.correlation) < 1e-9
    Options.reset()
