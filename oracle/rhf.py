"""Test-infrastructure oracle: Fermi's DF-RHF, restated on the CPU.

Only the tests and the benchmark's CPU leg use this module; the product path
builds the Fock matrix on the GPU (csrc/scf.cu) and never imports it.

Restated from src/Methods/HartreeFock/RHF/:

* ``build_fock_df``   RHFHelper.jl:88-93 -- F = H + 2 D[r,s] b[Q,m,n] b[Q,r,s]
                      - D[r,s] b[Q,m,r] b[Q,n,s], each ``@tensoropt`` line as one
                      literal einsum;
* ``build_fock_conv`` RHFHelper.jl:74-79 (four-index integrals);
* ``rhf_energy``      RHFHelper.jl:65-67;
* ``core_guess``      RHFHelper.jl:7-21;  ``gwh_guess``  RHFHelper.jl:28-59;
* ``rhf``             the RHFa iterations, RHFa.jl:67-203 (ODA damping while
                      Drms > oda_cutoff and ite < oda_shutoff, otherwise DIIS on
                      the Fock matrix after diis_start, convergence on |dE|,
                      Drms and ite > 5), with Fermi's DIISManager (DIIS.jl:21-96)
                      holding FP64 error vectors (DIISManager{Float64,Float64},
                      RHFa.jl:92).

Matrices are numpy arrays in the index order of their names; ``b`` is
``b[Q, mu, nu]``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .rccsd import DIISManager


def build_fock_df(H, D, b):
    """RHFHelper.jl:88-93."""
    F = H.copy()
    F += 2.0 * np.einsum("rs,Qmn,Qrs->mn", D, b, b, optimize=True)
    F -= np.einsum("rs,Qmr,Qns->mn", D, b, b, optimize=True)
    return F


def build_fock_conv(H, D, eri):
    """RHFHelper.jl:74-79: ERI[m,n,r,s] = (mn|rs)."""
    F = H.copy()
    F += 2.0 * np.einsum("rs,mnrs->mn", D, eri, optimize=True)
    F -= np.einsum("rs,mrns->mn", D, eri, optimize=True)
    return F


def rhf_energy(D, H, F) -> float:
    """RHFHelper.jl:65-67."""
    return float(np.sum(D * (H + F)))


def _inv_sqrt(S):
    w, U = np.linalg.eigh(S)
    return (U / np.sqrt(w)) @ U.T


def core_guess(S, H):
    """RHFHelper.jl:7-21: diagonalise the core Hamiltonian in the S^-1/2 basis."""
    Lam = _inv_sqrt(S)
    Ft = Lam @ H @ Lam.T
    _, Ct = np.linalg.eigh(Ft, UPLO="U")
    return Lam @ Ct, Lam


def gwh_guess(S, H):
    """RHFHelper.jl:28-59: generalised Wolfsberg-Helmholz guess."""
    Lam = _inv_sqrt(S)
    n = S.shape[0]
    F = np.empty_like(S)
    for i in range(n):
        F[i, i] = H[i, i]
        for j in range(i + 1, n):
            F[i, j] = 0.875 * S[i, j] * (H[i, i] + H[j, j])
            F[j, i] = F[i, j]
    Ft = Lam.T @ F @ Lam
    _, Ct = np.linalg.eigh(Ft, UPLO="U")
    return Lam @ Ct, Lam


@dataclass
class SCFOptions:
    """Fermi's SCF options with their defaults (src/Core/Options.jl:55-89)."""
    scf_max_iter: int = 50
    scf_max_rms: float = 1e-9
    scf_e_conv: float = 1e-10
    diis: bool = True
    ndiis: int = 8
    diis_start: int = 3
    oda: bool = True
    oda_cutoff: float = 1e-1
    oda_shutoff: int = 20


@dataclass
class RHFResult:
    energy: float
    eps: np.ndarray
    C: np.ndarray
    iterations: int
    converged: bool
    dE: float
    Drms: float


def rhf(H, S, ndocc: int, e_nuc: float, fock, C, Lam, opts: SCFOptions | None = None) -> RHFResult:
    """RHFa.jl:67-203.  ``fock(H, D)`` returns the Fock matrix (build_fock!)."""
    opts = opts or SCFOptions()
    ite, E, dE, Drms = 1, 0.0, 1.0, 1.0
    converged = False
    DM = DIISManager(size=opts.ndiis, err_dtype=np.float64) if opts.diis else None
    Co = C[:, :ndocc]
    D = Co @ Co.T                                              # :118-119
    D_old = D.copy()
    eps = np.zeros(C.shape[1])
    F = fock(H, D)                                             # :124-125
    Ft_, Dt_ = F.copy(), D.copy()
    N = D.size
    while ite <= opts.scf_max_iter:                            # :134
        Ft = Lam.T @ F @ Lam                                   # :137
        eps, Ct = np.linalg.eigh(Ft, UPLO="U")                 # :140 (Symmetric: upper triangle)
        C = Lam @ Ct                                           # :143
        Co = C[:, :ndocc]
        D = Co @ Co.T                                          # :146-147
        F = fock(H, D)                                         # :150
        Enew = rhf_energy(D, H, F) + e_nuc                     # :151-154
        if DM is not None:                                     # :157-160
            err = Lam.T @ (F @ D @ S - S @ D @ F) @ Lam
            DM.push(F, err)
        if opts.oda and Drms > opts.oda_cutoff and ite < opts.oda_shutoff:   # :166-179
            dD = D - Dt_
            s = np.trace(Ft_ @ dD)
            c = np.trace((F - Ft_) @ dD)
            lam = 1.0 if c <= -s / (2 * c) else -s / (2 * c)
            Ft_ = (1 - lam) * Ft_ + lam * F
            Dt_ = (1 - lam) * Dt_ + lam * D
            F = Ft_.copy()
        elif DM is not None and ite > opts.diis_start:        # :182-185
            F = DM.extrapolate()
        dD = D - D_old                                         # :188-189
        Drms = float(np.sqrt(np.sum(dD ** 2) / N))
        dE = Enew - E                                          # :192-194
        E = Enew
        D_old = D.copy()
        ite += 1
        if abs(dE) < opts.scf_e_conv and Drms < opts.scf_max_rms and ite > 5:   # :199-202
            converged = True
            break
    return RHFResult(E, eps, C, ite - 1, converged, dE, Drms)
