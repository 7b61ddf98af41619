"""The restated DF-RHF (oracle/rhf.py) and the host side of the RHFcuda driver,
on the CPU.

The oracle's literal build_fock! einsums are checked against the stand-in
pipeline's factored J/K (independent code), its RHFa iterations against the
pipeline's converged SCF energy, and the RHFcuda driver's host logic (guess,
ODA, DIIS, convergence test) against the oracle loop, with the oracle's Fock
build standing in for the device one.
"""
import functools

import numpy as np
import pytest

from oracle import rhf as orhf


@functools.lru_cache(maxsize=None)
def _problem(n, seed=0):
    from fermicc.inputs import molecule, scf
    return scf.df_ao_problem(molecule.waters(n, seed))


def _factored_fock(H, D, b):
    naux, n, _ = b.shape
    J = np.einsum("Q,Qmn->mn", np.einsum("Qrs,rs->Q", b, D), b)
    K = np.einsum("Qmr,rs,Qns->mn", b, D, b, optimize=True)
    return H + 2 * J - K


def test_literal_fock_equals_factored_jk():
    p = _problem(2)
    rng = np.random.default_rng(3)
    n = p.H.shape[0]
    A = rng.standard_normal((n, n)) * 0.05
    for D in (A + A.T, A):                          # symmetric and general densities
        F = orhf.build_fock_df(p.H, D, p.b)
        assert np.abs(F - _factored_fock(p.H, D, p.b)).max() < 1e-12
    # with b expanded to four-index integrals, the conventional build agrees
    eri = np.einsum("Qmn,Qrs->mnrs", p.b, p.b)
    D = A + A.T
    assert np.abs(orhf.build_fock_conv(p.H, D, eri) - orhf.build_fock_df(p.H, D, p.b)).max() < 1e-12


@pytest.mark.parametrize("n", [1, 2])
def test_rhfa_iterations_reach_the_pipeline_scf_energy(n):
    from fermicc.inputs import scf
    p = _problem(n)
    C, Lam = orhf.gwh_guess(p.S, p.H)
    r = orhf.rhf(p.H, p.S, p.ndocc, p.e_nuc, lambda H, D: orhf.build_fock_df(H, D, p.b), C, Lam)
    assert r.converged
    ref = scf.water_inputs(n, seed=0)
    assert abs(r.energy - ref.e_ref) < 1e-9
    assert np.abs(r.eps[ref.meta["frozen"]:ref.meta["ndocc"]] - ref.eps_o).max() < 1e-6


def test_guesses_and_energy():
    p = _problem(1)
    for guess in (orhf.gwh_guess, orhf.core_guess):
        C, Lam = guess(p.S, p.H)
        assert np.abs(C.T @ p.S @ C - np.eye(C.shape[1])).max() < 1e-10      # S-orthonormal
    D = np.eye(p.H.shape[0]) * 0.1
    F = orhf.build_fock_df(p.H, D, p.b)
    assert orhf.rhf_energy(D, p.H, F) == pytest.approx(float(np.sum(D * (p.H + F))), rel=1e-15)


class _OracleFock:
    """A stand-in for DFFock with the oracle's build (host-logic test only)."""

    def __init__(self, b):
        self.b = b

    def build(self, H, D):
        F = orhf.build_fock_df(H, D, self.b)
        return F, orhf.rhf_energy(D, H, F)

    def build_occ(self, H, Co):
        return self.build(H, Co @ Co.T)


@pytest.mark.parametrize("occupied_form", [True, False])
def test_rhfcuda_driver_follows_the_rhfa_iterations(occupied_form):
    from fermicc import RHF, Options
    p = _problem(2)
    Options.reset()
    r = RHF.compute(p.H, p.S, p.ndocc, p.e_nuc, _OracleFock(p.b), occupied_form=occupied_form)
    C, Lam = orhf.gwh_guess(p.S, p.H)
    o = orhf.rhf(p.H, p.S, p.ndocc, p.e_nuc, lambda H, D: orhf.build_fock_df(H, D, p.b), C, Lam)
    assert r.converged and o.converged
    assert r.iterations == o.iterations
    assert abs(r.energy - o.energy) < 1e-11
    assert np.abs(r.eps - o.eps).max() < 1e-9


def test_rhfcuda_options_and_dispatch():
    from fermicc import FermiException, Options, RHF, get_rhf_alg
    from fermicc.rhf import RHFcuda
    Options.reset()
    assert isinstance(get_rhf_alg(), RHFcuda)
    assert Options.get("scf_guess") == "gwh" and Options.get("ndiis") == 8 and Options.get("oda") is True
    with pytest.raises(FermiException):
        get_rhf_alg(1)
    p = _problem(1)
    Options.set("scf_guess", "core")
    Options.set("scf_max_iter", 2)
    r = RHF.compute(p.H, p.S, p.ndocc, p.e_nuc, _OracleFock(p.b))
    assert not r.converged and r.iterations == 2
    Options.set("scf_guess", "sad")
    with pytest.raises(FermiException):
        RHF.compute(p.H, p.S, p.ndocc, p.e_nuc, _OracleFock(p.b))
    Options.reset()
