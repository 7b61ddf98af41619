"""The CPU oracle against independent known answers (no GPU)."""
import numpy as np
import pytest

from conftest import inputs
from oracle import rccsd as R
from oracle import spinorbital as SO
from oracle import t1dressed as TD
from oracle import triples as T


def _converge(inp, df, **kw):
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv) if df else inp.conv
    opts = R.CCOptions(cc_e_conv=1e-12, cc_max_rms=1e-10, **kw)
    res = R.rccsd(I, inp.eps_o, inp.eps_v, inp.e_ref, opts, Bvv=inp.Bvv if df else None)
    return I, res


@pytest.fixture(scope="module")
def conv_solution(water_conv):
    return _converge(water_conv, df=False)


def test_closed_shell_ccsd_equals_spin_orbital(water_conv, conv_solution):
    # an independently written spin-orbital CCSD (Stanton-Gauss) on the same
    # integrals must give the same correlation energy
    I, res = conv_solution
    assert res.converged
    g = SO.full_spatial_eri(I, water_conv.o, water_conv.v)
    anti, f, no, _ = SO.spin_orbital(g, np.concatenate([water_conv.eps_o, water_conv.eps_v]), water_conv.o)
    E, t1, t2 = SO.ccsd(anti, f, no)
    assert abs(E - res.correlation) < 1e-10


def test_triples_ijk_equals_spin_orbital(water_conv, conv_solution):
    I, res = conv_solution
    et = T.triples_ijk(res.T1, res.T2, I["OVVV"], I["OOOV"], I["OVOV"], water_conv.eps_o, water_conv.eps_v)
    g = SO.full_spatial_eri(I, water_conv.o, water_conv.v)
    anti, f, no, _ = SO.spin_orbital(g, np.concatenate([water_conv.eps_o, water_conv.eps_v]), water_conv.o)
    # spin-orbital amplitudes from the closed-shell ones
    nv = 2 * water_conv.v
    t1so = np.zeros((no, nv))
    t1so[0::2, 0::2] = res.T1
    t1so[1::2, 1::2] = res.T1
    t2so = np.zeros((no, no, nv, nv))
    t2 = res.T2
    t2so[0::2, 1::2, 0::2, 1::2] = t2
    t2so[1::2, 0::2, 1::2, 0::2] = t2
    t2so[0::2, 1::2, 1::2, 0::2] = -t2.transpose(0, 1, 3, 2)
    t2so[1::2, 0::2, 0::2, 1::2] = -t2.transpose(0, 1, 3, 2)
    aa = t2 - t2.transpose(0, 1, 3, 2)
    t2so[0::2, 0::2, 0::2, 0::2] = aa
    t2so[1::2, 1::2, 1::2, 1::2] = aa
    eso = SO.triples(anti, f, no, t1so, t2so)
    assert abs(et - eso) < 1e-11
    assert et < 0


def test_abc_algorithm(water_conv, conv_solution):
    # Fermi's abc.jl multiplies by T2_c where T2_a is needed (abc.jl:128,131):
    # the literal restatement disagrees with ijk, the corrected one agrees.
    I, res = conv_solution
    args = (res.T1, res.T2, I["OVVV"], I["OOOV"], I["OVOV"], water_conv.eps_o, water_conv.eps_v)
    e_ijk = T.triples_ijk(*args)
    e_abc_fixed = T.triples_abc(*args, corrected=True)
    e_abc_literal = T.triples_abc(*args, corrected=False)
    assert abs(e_ijk - e_abc_fixed) < 1e-12
    assert abs(e_ijk - e_abc_literal) > 1e-4


def test_df_ladder_equals_conventional_ladder(water_df):
    inp = water_df
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv, with_vvvv=True)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    rng = np.random.default_rng(1)
    T1 = T1 + 0.01 * rng.standard_normal(T1.shape)
    a = R.ladder_df(T1, T2, inp.Bvv)
    b = R.ladder_conv(T1, T2, I["VVVV"])
    assert np.abs(a - b).max() < 1e-13


@pytest.mark.parametrize("n", [1, 2])
def test_t1_dressed_residual_equals_reference_terms(n):
    # the formulation the GPU evaluates is the same function of (T1, T2) as
    # the reference's term-by-term sum, away from convergence too
    inp = inputs(n, seed=3)
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    rng = np.random.default_rng(7)
    T1 = T1 + 0.02 * rng.standard_normal(T1.shape)
    T2 = T2 + 0.01 * rng.standard_normal(T2.shape)
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    n1 = R.cc_update_T1(T1, T2, I)
    n2 = R.cc_update_T2(T1, T2, I, R.ladder_df(T1, T2, inp.Bvv))
    r1, r2 = TD.residual(T1, T2, inp.Boo, inp.Bov, inp.Bvv, inp.eps_o, inp.eps_v)
    assert np.abs(r1 + D1 * T1 - n1).max() < 1e-13
    assert np.abs(r2 + D2 * T2 - n2).max() < 1e-13


def test_energy_formula(water_df):
    # the energy of RCCSDHelper.jl:8-23 equals sum (2(kc|ld)-(kd|lc)) tau
    inp = water_df
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    rng = np.random.default_rng(2)
    T1 = 0.05 * rng.standard_normal((inp.o, inp.v))
    T2 = 0.05 * rng.standard_normal((inp.o, inp.o, inp.v, inp.v))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    ovov = I["OVOV"]
    Lt = 2 * np.einsum("kcld->klcd", ovov) - np.einsum("kdlc->klcd", ovov)
    e = np.sum(Lt * (T2 + np.einsum("kc,ld->klcd", T1, T1)))
    assert abs(e - R.cc_update_energy(T1, T2, ovov)) < 1e-12


def test_size_consistency():
    # two waters 50 Angstrom apart: E_corr(dimer) = 2 E_corr(monomer)
    from fermicc.inputs import molecule, scf
    w = molecule.waters(1, 0)
    far = w + [(e, p + np.array([50.0, 0.0, 0.0])) for e, p in w]
    mono = scf.df_inputs(w, frozen_core=True)
    dim = scf.df_inputs(far, frozen_core=True)
    e1 = _converge(mono, df=True)[1].correlation
    e2 = _converge(dim, df=True)[1].correlation
    assert abs(e2 - 2 * e1) < 1e-8


def test_diis_manager_semantics():
    # DIIS.jl / test_diis.jl: length, BoundsError with fewer than 2 vectors,
    # eviction of the largest error when full
    dm = R.DIISManager(size=3)
    assert len(dm) == 0
    dm.push(np.ones(4), np.ones(4))
    assert len(dm) == 1
    with pytest.raises(IndexError):
        dm.extrapolate()
    dm.push(2 * np.ones(4), 10 * np.ones(4))
    dm.push(3 * np.ones(4), 0.1 * np.ones(4))
    dm.push(4 * np.ones(4), 0.2 * np.ones(4))
    assert len(dm) == 3
    assert all(float(e.max()) < 5 for e in dm.errs)


def test_df_mp2_pair_loop_equals_the_mp2_guess_energy():
    # RMP2a.jl's pair loop and the CC driver's MP2 guess energy (RCCSDa.jl:46-89)
    # are the same number on the same factors
    from oracle import rmp2
    inp = inputs(1, df=True)
    e_pair = rmp2.rmp2_energy_df(inp.Bov, inp.eps_o, inp.eps_v)
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    e_guess = R.cc_update_energy(T1, T2, I["OVOV"])
    assert abs(e_pair - e_guess) < 1e-13


def test_ccd_limit_equals_spin_orbital_ccd(water_conv):
    # T1 held at zero in the closed-shell equations = an independent
    # spin-orbital CCD on the same integrals
    I = water_conv.conv
    opts = R.CCOptions(cc_e_conv=1e-12, cc_max_rms=1e-10)
    res = R.rccsd(I, water_conv.eps_o, water_conv.eps_v, water_conv.e_ref, opts, ccd=True)
    assert res.converged and np.abs(res.T1).max() == 0.0
    g = SO.full_spatial_eri(I, water_conv.o, water_conv.v)
    anti, f, no, _ = SO.spin_orbital(g, np.concatenate([water_conv.eps_o, water_conv.eps_v]), water_conv.o)
    E, t1, _ = SO.ccsd(anti, f, no, ccd=True)
    assert np.abs(t1).max() == 0.0
    assert abs(E - res.correlation) < 1e-10
    full = _converge(water_conv, df=False)[1]
    assert abs(full.correlation - res.correlation) > 1e-6       # singles matter: not a vacuous check


def test_rotation_and_translation_invariance():
    # the README water rotated by a random proper rotation and shifted: the same
    # RHF, CCSD and (T) energies
    from fermicc.inputs import molecule, scf
    w = molecule.waters(1, 0)
    rng = np.random.default_rng(11)
    Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    moved = [(e, Q @ p + np.array([1.3, -0.7, 2.1])) for e, p in w]
    a = scf.conv_inputs(w)
    b = scf.conv_inputs(moved)
    assert abs(a.e_ref - b.e_ref) < 1e-10
    ra = _converge(a, df=False)[1]
    rb = _converge(b, df=False)[1]
    # the SCF stops at |dE| < 1e-10 with the commutator below 1e-7: orbital
    # noise of that size reaches the correlation energy at ~1e-10
    assert abs(ra.correlation - rb.correlation) < 1e-9
    ta = T.triples_ijk(ra.T1, ra.T2, a.conv["OVVV"], a.conv["OOOV"], a.conv["OVOV"], a.eps_o, a.eps_v)
    tb = T.triples_ijk(rb.T1, rb.T2, b.conv["OVVV"], b.conv["OOOV"], b.conv["OVOV"], b.eps_o, b.eps_v)
    assert abs(ta - tb) < 1e-10


def test_first_update_from_zero_is_the_mp2_guess(water_conv):
    # one update_amp! from T1 = T2 = 0 gives T1 = 0 and the MP2 amplitudes of
    # RCCSDa.jl:53-89, hence the guess energy
    I = water_conv.conv
    D1, D2 = R.denominators(water_conv.eps_o, water_conv.eps_v)
    o, v = water_conv.o, water_conv.v
    T1, T2 = R.update_amp(np.zeros((o, v)), np.zeros((o, o, v, v)), I, D1, D2,
                          lambda t1, t2: R.ladder_conv(t1, t2, I["VVVV"]))
    G1, G2 = R.mp2_guess(I, D1, D2)
    assert np.abs(T1).max() < 1e-14 and np.abs(T2 - G2).max() < 1e-14
    assert abs(R.cc_update_energy(T1, T2, I["OVOV"]) - R.cc_update_energy(G1, G2, I["OVOV"])) < 1e-14
