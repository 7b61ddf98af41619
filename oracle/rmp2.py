"""Test-infrastructure oracle: the reference's DF-MP2 energy, restated.

Restates `RMP2_energy` for density-fitted integrals and RHF orbitals
(src/Methods/MollerPlesset/RMP2/RMP2a.jl:91-140): for every pair i <= j,
B_ab = sum_Q B[Q,a,i] B[Q,b,j] (:114), and
E += fac * sum_ab B_ab (2 B_ab - B_ba) / (e_i + e_j - e_a - e_b)
(:116-126) with fac = 2 for i != j and 1 for i == j (:127-128).
Only the tests and the benchmark's CPU leg use this module.
"""
import numpy as np


def rmp2_energy_df(Bov, eps_o, eps_v):
    """Bov[Q, i, a] (active occupied x virtual factors); returns E_MP2 (correlation)."""
    o = Bov.shape[1]
    E = 0.0
    for i in range(o):
        Bi = Bov[:, i, :]                                   # Bvo[:, :, i] (:112-113)
        for j in range(i, o):
            Bab = Bi.T @ Bov[:, j, :]                       # (:114)
            D = eps_o[i] + eps_o[j] - eps_v[:, None] - eps_v[None, :]
            e = np.sum(Bab * (2.0 * Bab - Bab.T) / D)       # (:116-126)
            E += (2.0 if i != j else 1.0) * e               # (:127-128)
    return E
