"""RHF and the coupled-cluster input tensors (the reference side of the boundary).

In Fermi.jl the coupled-cluster path receives, from upstream code that stays on
the reference side:

* RHF orbital energies and the SCF energy (``RHFOrbitals``,
  src/Core/Orbitals.jl:86-92; ``moints.orbitals.sd_energy`` read at
  src/Methods/CoupledCluster/RCCSD/RCCSDa.jl:97);
* for density fitting, the MO three-index factors
  ``b[Q,p,q] = sum_P (pq|P) [J^-1/2]_PQ`` (src/Core/Integrals/AtomicIntegrals.jl:31-40)
  sliced into ``BOO``, ``BOV``, ``BVV`` with the frozen core dropped
  (src/Core/Integrals/ROIntegrals/DFERI.jl:15-69);
* for the conventional path, the MO integral blocks OOOO..VVVV.

This module produces the same quantities for the stand-in basis sets: a
DF-RHF (the fitting basis plays the JK role, as JKFIT does in
src/Core/Integrals/IntegralHelper.jl:79-86) or a conventional RHF with exact
four-index integrals, both with Pulay DIIS on the commutator FDS - SDF.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import basis as bas
from . import ints
from .molecule import waters


@dataclass
class CCInputs:
    """Everything the coupled-cluster path reads, in logical index order.

    Arrays are numpy C-ordered with the index order of their names:
    ``Boo[Q,i,j]``, ``Bov[Q,i,a]``, ``Bvv[Q,a,b]`` (DF); ``OVOV[i,a,j,b]`` =
    (ia|jb) etc. (conventional).  The C ABI takes the column-major layout of
    Fermi's Julia arrays, i.e. ``np.asfortranarray`` of these.
    """
    o: int
    v: int
    naux: int
    eps_o: np.ndarray
    eps_v: np.ndarray
    e_ref: float
    e_nuc: float
    Boo: np.ndarray | None = None
    Bov: np.ndarray | None = None
    Bvv: np.ndarray | None = None
    conv: dict | None = None
    meta: dict = field(default_factory=dict)
    # AO-side data of the DF path (aoints["ERI"] = b[Q,mu,nu], the RHF
    # coefficients C[mu,p], all orbital energies, ndocc, frozen core), kept when
    # the MO transform is to run on the device
    ao: dict | None = None


def _sym_inv_sqrt(M: np.ndarray, what: str, tol: float = 1e-12) -> np.ndarray:
    w, U = np.linalg.eigh(M)
    if w.min() < tol * w.max():
        raise ValueError(f"{what} is numerically singular (min eigenvalue {w.min():.3e})")
    return (U / np.sqrt(w)) @ U.T


def _nuclear_repulsion(xyz: np.ndarray, Z: np.ndarray) -> float:
    e = 0.0
    for i in range(len(Z)):
        for j in range(i):
            e += Z[i] * Z[j] / np.linalg.norm(xyz[i] - xyz[j])
    return e


class _DIIS:
    def __init__(self, nmax: int = 8):
        self.F, self.E, self.nmax = [], [], nmax

    def push(self, F, err):
        self.F.append(F.copy()); self.E.append(err.copy())
        if len(self.F) > self.nmax:
            self.F.pop(0); self.E.pop(0)

    def extrapolate(self):
        n = len(self.F)
        B = -np.ones((n + 1, n + 1)); B[n, n] = 0.0
        for i in range(n):
            for j in range(n):
                B[i, j] = np.vdot(self.E[i], self.E[j])
        rhs = np.zeros(n + 1); rhs[n] = -1.0
        c = np.linalg.solve(B, rhs)[:n]
        return sum(ci * Fi for ci, Fi in zip(c, self.F))


def _scf(H, S, ndocc, jk, e_nuc, conv=1e-10, maxiter=200):
    X = _sym_inv_sqrt(S, "overlap")
    eps, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    diis = _DIIS()
    e_old = 0.0
    for it in range(maxiter):
        Co = C[:, :ndocc]
        D = Co @ Co.T
        J, K = jk(D, Co)
        F = H + 2 * J - K
        E = float(np.sum(D * (H + F))) + e_nuc
        err = F @ D @ S - S @ D @ F
        err = X.T @ err @ X
        diis.push(F, err)
        if it >= 1:
            F = diis.extrapolate()
        eps, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        if abs(E - e_old) < conv and np.abs(err).max() < 1e-7:
            # one more diagonalisation of the undamped Fock for clean orbitals
            Co = C[:, :ndocc]
            D = Co @ Co.T
            J, K = jk(D, Co)
            F = H + 2 * J - K
            E = float(np.sum(D * (H + F))) + e_nuc
            eps, Cp = np.linalg.eigh(X.T @ F @ X)
            C = X @ Cp
            return E, eps, C, it + 1
        e_old = E
    raise RuntimeError(f"RHF did not converge in {maxiter} iterations")


def _setup(atoms):
    bohr = [(e, p * bas.ANGSTROM_TO_BOHR) for e, p in atoms]
    xyz = np.array([p for _, p in bohr])
    Z = np.array([bas.Z_OF[e] for e, _ in bohr], dtype=np.float64)
    orb = bas.flatten(bohr, bas.orbital_shells)
    S, T, V = ints.one_body(orb, xyz, Z)
    f = 1.0 / np.sqrt(np.diag(S))
    S = S * f[:, None] * f[None, :]
    H = (T + V) * f[:, None] * f[None, :]
    nelec = int(Z.sum())
    ndocc = nelec // 2
    frozen = sum(bas.FROZEN_ORBITALS[e] for e, _ in atoms)
    return bohr, xyz, Z, orb, S, H, f, ndocc, frozen


@dataclass
class AOProblem:
    """The AO-side inputs of a DF-RHF (the IntegralHelper cache of Fermi):
    H = T + V, S, the fitting quantities (pq|P), J^-1/2 and
    b[Q,mu,nu] = sum_P (mu nu|P) [J^-1/2]_PQ (AtomicIntegrals.jl:31-40), the
    number of doubly occupied orbitals, the frozen-core count and Vnuc."""
    H: np.ndarray
    S: np.ndarray
    b: np.ndarray
    Pqp: np.ndarray | None
    Jh: np.ndarray
    ndocc: int
    frozen: int
    e_nuc: float


def df_ao_problem(atoms, keep_pqp: bool = False) -> AOProblem:
    """One-body matrices and DF factors of the stand-in basis for ``atoms``."""
    bohr, xyz, Z, orb, S, H, f, ndocc, frozen = _setup(atoms)
    aux = bas.flatten(bohr, bas.fitting_shells)
    J2 = ints.eri2c(aux)
    g = 1.0 / np.sqrt(np.diag(J2))
    J2 = J2 * g[:, None] * g[None, :]
    I3 = ints.eri3c(orb, aux) * f[:, None, None] * f[None, :, None] * g[None, None, :]
    Jh = _sym_inv_sqrt(J2, "fitting metric")
    n, naux = orb.nbf, aux.nbf
    # b[Q, mu, nu] = sum_P (mu nu|P) Jh[P, Q]
    b = (I3.reshape(n * n, naux) @ Jh).T.reshape(naux, n, n)
    return AOProblem(H=H, S=S, b=b, Pqp=I3 if keep_pqp else None, Jh=Jh, ndocc=ndocc, frozen=frozen,
                     e_nuc=_nuclear_repulsion(xyz, Z))


def df_inputs(atoms, frozen_core: bool = True, keep_ao: bool = False, rhf_device: bool = False) -> CCInputs:
    """DF-RHF on the stand-in basis, then BOO/BOV/BVV with the core dropped
    (and, with keep_ao, the AO factors and orbitals for a device MO transform).
    With rhf_device the RHF is fermicc's RHFcuda (RHFa iterations, Fock build on
    the GPU) instead of the host SCF below."""
    ao = df_ao_problem(atoms, keep_pqp=keep_ao)
    H, S, b, Jh, ndocc, frozen, e_nuc = ao.H, ao.S, ao.b, ao.Jh, ao.ndocc, ao.frozen, ao.e_nuc
    if not frozen_core:
        frozen = 0
    naux, n = b.shape[0], b.shape[1]
    I3_kept = ao.Pqp
    bflat = b.reshape(naux, n * n)

    def jk(D, Co):
        gam = bflat @ D.reshape(-1)
        J = (gam @ bflat).reshape(n, n)
        bi = (b.reshape(naux * n, n) @ Co).reshape(naux, n, -1)      # [Q, mu, i]
        bi2 = bi.transpose(1, 0, 2).reshape(n, -1)
        K = bi2 @ bi2.T
        return J, K

    if rhf_device:
        from ..rhf import RHF, DFFock
        fock = DFFock(n, naux, b=b)
        try:
            r = RHF.compute(H, S, ndocc, e_nuc, fock)
        finally:
            fock.close()
        if not r.converged:
            raise RuntimeError(f"RHF did not converge in {r.iterations} iterations")
        E, eps, C, nit = r.energy, r.eps, r.C, r.iterations
    else:
        E, eps, C, nit = _scf(H, S, ndocc, jk, e_nuc)
    Co = C[:, frozen:ndocc]
    Cv = C[:, ndocc:]
    bo = (b.reshape(naux * n, n) @ Co).reshape(naux, n, -1)           # [Q, mu, i]
    bv = (b.reshape(naux * n, n) @ Cv).reshape(naux, n, -1)           # [Q, mu, a]
    Boo = np.einsum("Qmi,mj->Qij", bo, Co, optimize=True)
    Bov = np.einsum("Qmi,ma->Qia", bo, Cv, optimize=True)
    Bvv = np.einsum("Qma,mb->Qab", bv, Cv, optimize=True)
    Bvv = 0.5 * (Bvv + Bvv.transpose(0, 2, 1))
    Boo = 0.5 * (Boo + Boo.transpose(0, 2, 1))
    return CCInputs(o=Co.shape[1], v=Cv.shape[1], naux=naux,
                    eps_o=eps[frozen:ndocc].copy(), eps_v=eps[ndocc:].copy(),
                    e_ref=E, e_nuc=e_nuc,
                    Boo=np.ascontiguousarray(Boo), Bov=np.ascontiguousarray(Bov),
                    Bvv=np.ascontiguousarray(Bvv),
                    meta=dict(nbf=n, ndocc=ndocc, frozen=frozen, scf_iters=nit, kind="df"),
                    ao=(dict(Bmn=b, Pqp=I3_kept, Jh=Jh, C=C, eps=eps.copy(), ndocc=ndocc, core=frozen)
                        if keep_ao else None))


def conv_inputs(atoms, frozen_core: bool = False) -> CCInputs:
    """Conventional RHF (exact four-index integrals) and the seven MO blocks."""
    bohr, xyz, Z, orb, S, H, f, ndocc, frozen = _setup(atoms)
    if not frozen_core:
        frozen = 0
    eri = ints.eri4c(orb)
    eri *= f[:, None, None, None] * f[None, :, None, None] * f[None, None, :, None] * f[None, None, None, :]
    n = orb.nbf

    def jk(D, Co):
        J = np.einsum("mnls,ls->mn", eri, D, optimize=True)
        K = np.einsum("mlns,ls->mn", eri, D, optimize=True)
        return J, K

    e_nuc = _nuclear_repulsion(xyz, Z)
    E, eps, C, nit = _scf(H, S, ndocc, jk, e_nuc)
    Co = C[:, frozen:ndocc]
    Cv = C[:, ndocc:]

    def mo(A, B_, C_, D_):
        return np.einsum("pqrs,pi,qj,rk,sl->ijkl", eri, A, B_, C_, D_, optimize=True)

    conv = dict(OOOO=mo(Co, Co, Co, Co), OOOV=mo(Co, Co, Co, Cv), OOVV=mo(Co, Co, Cv, Cv),
                OVOV=mo(Co, Cv, Co, Cv), OVVV=mo(Co, Cv, Cv, Cv), VVVV=mo(Cv, Cv, Cv, Cv))
    return CCInputs(o=Co.shape[1], v=Cv.shape[1], naux=0,
                    eps_o=eps[frozen:ndocc].copy(), eps_v=eps[ndocc:].copy(),
                    e_ref=E, e_nuc=e_nuc, conv=conv,
                    meta=dict(nbf=n, ndocc=ndocc, frozen=frozen, scf_iters=nit, kind="conv"))


def water_inputs(n: int, seed: int = 0, df: bool = True, keep_ao: bool = False,
                 rhf_device: bool = False) -> CCInputs:
    """The workloads: n = 1 (README water, conventional, no frozen core) or a
    seeded (H2O)n cluster with DF and one frozen core orbital per oxygen."""
    atoms = waters(n, seed)
    if df:
        out = df_inputs(atoms, frozen_core=(n > 1), keep_ao=keep_ao, rhf_device=rhf_device)
    else:
        out = conv_inputs(atoms, frozen_core=False)
    out.meta.update(waters=n, seed=seed)
    return out
