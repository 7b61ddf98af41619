"""DF-RHF with the Fock build on the GPU, mirroring Fermi's RHF interface.

Fermi selects an RHF implementation with ``rhf_alg`` (``get_rhf_alg``,
src/Methods/HartreeFock/RHF/RHF.jl:89-111: 1 = ``RHFa``, 2 = ``Direct``); this
backend adds ``RHFcuda`` as 3.  Its iterations are those of
``RHF(ints, C, Λ, ::RHFa)`` (RHFa.jl:67-203: ODA damping while the density
still moves by more than ``oda_cutoff``, then DIIS on the Fock matrix, and the
convergence test on |ΔE|, Drms and the iteration count), with every
``build_fock!`` call (RHFHelper.jl:88-93) and ``RHFEnergy`` (RHFHelper.jl:65-67)
run by ``libfermicc`` on the device, where ``aoints["ERI"]`` stays resident.
The diagonalisations of the nbf x nbf Fock matrix and the DIIS solve stay on the
host, as in Fermi.

``DFFock`` is the device Fock builder on its own (``fcc_scf_*`` in
include/fermicc.h); ``RHF.compute`` is the driver.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import options as Options
from .options import FermiException


class RHFcuda:
    """Singleton selecting this backend (``rhf_alg`` = 3)."""


def get_rhf_alg(n: int | None = None):
    n = Options.get("rhf_alg") if n is None else n
    if n == 3:
        return RHFcuda()
    raise FermiException(f"implementation number {n} not available for RHF.")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class DFFock:
    """Device Fock builder: F = H + 2 J[D] - K[D] from b[Q,mu,nu] kept on the GPU.

    ``b`` (naux x nbf x nbf, numpy index order [Q, mu, nu]) is uploaded once; or
    give ``Pqp`` ((pq|P), nbf x nbf x naux) and ``Jh`` (J^-1/2) to fit on the
    device (AtomicIntegrals.jl:37-38)."""

    def __init__(self, nbf: int, naux: int, b=None, Pqp=None, Jh=None, device: int | None = None):
        self.lib = _lib.load()
        self.nbf, self.naux = int(nbf), int(naux)
        dev = Options.get("cc_gpu_device") if device is None else device
        h = ctypes.c_void_p()
        rc = self.lib.fcc_scf_create(ctypes.byref(h), self.nbf, self.naux, dev)
        if rc != 0:
            raise FermiException(f"fcc_scf_create: {self.lib.fcc_strerror(rc).decode()}")
        self.h = h
        if b is not None:
            b = np.asarray(b, dtype=np.float64)
            if b.shape != (self.naux, self.nbf, self.nbf):
                raise FermiException(f"b has shape {b.shape}, expected {(self.naux, self.nbf, self.nbf)}")
            bf = np.asfortranarray(b)
            self._check(self.lib.fcc_scf_upload_b(self.h, _ptr(bf)), "fcc_scf_upload_b")
        elif Pqp is not None and Jh is not None:
            P = np.asfortranarray(np.asarray(Pqp, dtype=np.float64))
            J = np.asfortranarray(np.asarray(Jh, dtype=np.float64))
            if P.shape != (self.nbf, self.nbf, self.naux) or J.shape != (self.naux, self.naux):
                raise FermiException("Pqp / Jh shapes do not match (nbf, nbf, naux) / (naux, naux)")
            self._check(self.lib.fcc_scf_fit(self.h, _ptr(P), _ptr(J)), "fcc_scf_fit")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.fcc_scf_last_error(self.h).decode() if self.h else ""
            raise FermiException(f"{what}: {self.lib.fcc_strerror(rc).decode()} ({msg})")

    def build(self, H, D):
        """build_fock! for a density D; returns (F, sum(D .* (H .+ F)))."""
        n = self.nbf
        Hf = np.asfortranarray(H, dtype=np.float64)
        Df = np.asfortranarray(D, dtype=np.float64)
        if Hf.shape != (n, n) or Df.shape != (n, n):
            raise FermiException("H and D must be nbf x nbf")
        F = np.empty((n, n), order="F")
        e = ctypes.c_double()
        self._check(self.lib.fcc_scf_build_fock(self.h, _ptr(Hf), _ptr(Df), _ptr(F), ctypes.byref(e)),
                    "fcc_scf_build_fock")
        return np.ascontiguousarray(F), e.value

    def build_occ(self, H, Co):
        """The same for D = Co Co^T, with K factored through the occupied orbitals."""
        n = self.nbf
        Hf = np.asfortranarray(H, dtype=np.float64)
        Cf = np.asfortranarray(Co, dtype=np.float64)
        if Hf.shape != (n, n) or Cf.ndim != 2 or Cf.shape[0] != n:
            raise FermiException("H must be nbf x nbf and Co nbf x nocc")
        F = np.empty((n, n), order="F")
        e = ctypes.c_double()
        self._check(self.lib.fcc_scf_build_fock_occ(self.h, _ptr(Hf), _ptr(Cf), Cf.shape[1], _ptr(F),
                                                     ctypes.byref(e)), "fcc_scf_build_fock_occ")
        return np.ascontiguousarray(F), e.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.fcc_scf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _inv_sqrt(S):
    w, U = np.linalg.eigh(S)
    return (U / np.sqrt(w)) @ U.T


def _guess(S, H, kind: str):
    """RHF_core_guess / RHF_gwh_guess (RHFHelper.jl:7-59)."""
    Lam = _inv_sqrt(S)
    if kind == "core":
        F = H
    elif kind == "gwh":
        d = np.diag(H)
        F = 0.875 * S * (d[:, None] + d[None, :])
        np.fill_diagonal(F, d)
    else:
        raise FermiException(f"invalid scf_guess: {kind}")
    _, Ct = np.linalg.eigh(Lam.T @ F @ Lam, UPLO="U")
    return Lam @ Ct, Lam


class _DIIS:
    """Fermi's DIISManager{Float64,Float64} (DIIS.jl:21-96) for the Fock matrix."""

    def __init__(self, size: int):
        self.vecs, self.errs, self.size = [], [], size

    def push(self, V, E):
        if len(self.vecs) + 1 > self.size:
            k = int(np.argmax([np.linalg.norm(e) for e in self.errs]))
            del self.vecs[k], self.errs[k]
        self.vecs.append(V.copy())
        self.errs.append(E.copy())

    def extrapolate(self):
        n = len(self.vecs)
        B = np.ones((n + 1, n + 1))
        B[n, n] = 0.0
        for i, ei in enumerate(self.errs):
            for j, ej in enumerate(self.errs):
                B[i, j] = np.sum(ei * ej)
        r = np.zeros(n + 1)
        r[n] = 1.0
        c = np.linalg.solve(B, r)
        return sum(ci * v for ci, v in zip(c[:n], self.vecs))


@dataclass
class RHF:
    """Fields of Fermi's ``struct RHF`` (RHF.jl:69-77) that the CC path reads,
    plus the orbitals (``RHFOrbitals``: eps, C) and the iteration count."""
    energy: float
    ndocc: int
    nvir: int
    eps: np.ndarray
    C: np.ndarray
    e_conv: float
    d_conv: float
    iterations: int
    converged: bool

    @classmethod
    def compute(cls, H, S, ndocc: int, e_nuc: float, fock: DFFock, C=None, alg=None,
                occupied_form: bool = True) -> "RHF":
        """RHF(ints, C, Λ, alg) (RHFa.jl:67-203) with the device Fock build.

        ``C`` is the starting guess (default: ``scf_guess``, RHFa.jl:25-30);
        ``occupied_form`` builds K from the occupied orbitals (every density of
        the iterations is Co Co^T), otherwise from D as build_fock! does."""
        if not isinstance(alg if alg is not None else get_rhf_alg(), RHFcuda):
            raise FermiException("RHF.compute runs the RHFcuda algorithm only")
        H = np.asarray(H, dtype=np.float64)
        S = np.asarray(S, dtype=np.float64)
        guessC, Lam = _guess(S, H, Options.get("scf_guess"))
        C = guessC if C is None else np.asarray(C, dtype=np.float64)
        maxit = Options.get("scf_max_iter")
        Etol, Dtol = Options.get("scf_e_conv"), Options.get("scf_max_rms")
        do_diis, oda = Options.get("diis"), Options.get("oda")
        oda_cutoff, oda_shutoff = Options.get("oda_cutoff"), Options.get("oda_shutoff")
        diis_start = Options.get("diis_start")
        DM = _DIIS(Options.get("ndiis")) if do_diis else None

        def build(C_):
            Co = C_[:, :ndocc]
            D_ = Co @ Co.T
            F_, e_ = fock.build_occ(H, Co) if occupied_form else fock.build(H, D_)
            return D_, F_, e_

        ite, E, dE, Drms, converged = 1, 0.0, 1.0, 1.0, False
        D, F, _ = build(C)
        D_old = D.copy()
        Fd, Dd = F.copy(), D.copy()
        N = D.size
        eps = np.zeros(C.shape[1])
        while ite <= maxit:
            eps, Ct = np.linalg.eigh(Lam.T @ F @ Lam, UPLO="U")
            C = Lam @ Ct
            D, F, eelec = build(C)
            Enew = eelec + e_nuc
            if DM is not None:
                DM.push(F, Lam.T @ (F @ D @ S - S @ D @ F) @ Lam)
            if oda and Drms > oda_cutoff and ite < oda_shutoff:
                dD = D - Dd
                s = np.trace(Fd @ dD)
                c = np.trace((F - Fd) @ dD)
                lam = 1.0 if c <= -s / (2 * c) else -s / (2 * c)
                Fd = (1 - lam) * Fd + lam * F
                Dd = (1 - lam) * Dd + lam * D
                F = Fd.copy()
            elif DM is not None and ite > diis_start:
                F = DM.extrapolate()
            Drms = float(np.sqrt(np.sum((D - D_old) ** 2) / N))
            dE, E = Enew - E, Enew
            D_old = D
            ite += 1
            if abs(dE) < Etol and Drms < Dtol and ite > 5:
                converged = True
                break
        return cls(energy=E, ndocc=ndocc, nvir=C.shape[1] - ndocc, eps=eps, C=C, e_conv=dE, d_conv=Drms,
                   iterations=ite - 1, converged=converged)
