"""Host-side mirror of Fermi's RCCSD / RCCSD(T) method objects over libfermicc.

Fermi.jl selects coupled-cluster implementations through singleton algorithm
types (``get_rccsd_alg(Val(N))``, src/Methods/CoupledCluster/RCCSD/RCCSD.jl:76-88;
``get_pt_alg``, PerturbativeTriples/PerturbativeTriples.jl:32-49) and returns
``struct RCCSD`` (RCCSD.jl:61-69) and ``struct RCCSDpT``
(PerturbativeTriples.jl:21-25).  This module keeps those names and fields:

* ``RCCSDcuda`` / ``CudaPT``: the algorithm singletons of this backend
  (``cc_alg = 2``, ``pt_alg = 4``);
* ``RCCSD.compute(moints, T1guess=None, T2guess=None, alg=None)``: the core
  boundary ``RCCSD(moints, T1guess, T2guess, alg)`` (RCCSDa.jl:92);
* ``RCCSDpT.compute(ccsd, moints, alg=None)``: ``RCCSDpT(ccsd, moints, alg)``
  (ijk.jl:20);
* ``RMP2.compute(moints)``: the DF-RMP2 energy (MollerPlesset/RMP2/RMP2a.jl:91-140)
  from the same device integrals, ``mp2_alg = 3``;
* ``energy("mp2" | "ccsd" | "ccsd(t)", moints)``: the ``@energy`` entry
  (src/Tools/SinglePointEnergy.jl:8-11,46).

``moints`` is a :class:`fermicc.inputs.scf.CCInputs` (the MO integral cache).
Amplitudes stay on the GPU between CCSD and (T): the context is kept in the
returned object.  Every call goes through the C ABI; a failing status raises
``FermiException``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from . import options as Options
from .options import FermiException


@dataclass(frozen=True)
class RCCSDcuda:
    """GB300 implementation of RCCSD (``cc_alg = 2``)."""


@dataclass(frozen=True)
class CudaPT:
    """GB300 implementation of RCCSD(T) (``pt_alg = 4``)."""


@dataclass(frozen=True)
class RMP2cuda:
    """GB300 implementation of the (DF-)RMP2 energy (``mp2_alg = 3``)."""


def get_rmp2_alg(n: int | None = None):
    n = Options.get("mp2_alg") if n is None else n
    if n == 3:
        return RMP2cuda()
    raise FermiException(f"implementation number {n} not available for RMP2.")


def get_rccsd_alg(n: int | None = None):
    n = Options.get("cc_alg") if n is None else n
    if n == 2:
        return RCCSDcuda()
    raise FermiException(f"implementation number {n} not available for RCCSD.")


def get_pt_alg(n: int | None = None):
    n = Options.get("pt_alg") if n is None else n
    if n == 4:
        return CudaPT()
    raise FermiException(f"implementation number {n} not available for RCCSD(T).")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(lib, ctx, rc, what):
    if rc in (_lib.FCC_OK, _lib.FCC_NO_CONVERGE):
        return rc
    msg = lib.fcc_strerror(rc).decode()
    detail = lib.fcc_last_error(ctx).decode() if ctx else ""
    raise FermiException(f"{what}: {msg}" + (f" ({detail})" if detail else ""))


class Context:
    """One device-side coupled-cluster problem (an ``fcc_ctx``)."""

    def __init__(self, moints, device: int | None = None, mo_transform: bool = False, fit: bool = False):
        """mo_transform: build the MO factors on the device from moints.ao
        (aoints["ERI"] and the orbitals, the DFERI.jl:15-69 transform) instead
        of uploading BOO/BOV/BVV; with fit, from the AO integrals (pq|P) and
        J^-1/2 (the AtomicIntegrals.jl:37-38 fit on the device as well)."""
        self.lib = _lib.load()
        self.o, self.v = int(moints.o), int(moints.v)
        naux = int(moints.naux) if moints.Bvv is not None else 0
        dev = Options.get("cc_gpu_device") if device is None else device
        h = ctypes.c_void_p()
        rc = self.lib.fcc_create(ctypes.byref(h), self.o, self.v, naux, dev)
        _check(self.lib, None, rc, "fcc_create")
        self.h = h
        eo = np.ascontiguousarray(moints.eps_o, dtype=np.float64)
        ev = np.ascontiguousarray(moints.eps_v, dtype=np.float64)
        if naux > 0 and mo_transform:
            ao = getattr(moints, "ao", None)
            if ao is None:
                raise FermiException("mo_transform needs the AO factors and orbitals (moints.ao)")
            C = np.asfortranarray(ao["C"], dtype=np.float64)
            eps = np.ascontiguousarray(ao["eps"], dtype=np.float64)
            nbf, nmo = C.shape
            if fit:
                P = np.asfortranarray(ao["Pqp"], dtype=np.float64)      # [p, q, P], p fastest
                Jh = np.asfortranarray(ao["Jh"], dtype=np.float64)
                rc = self.lib.fcc_upload_ao3_df(h, _ptr(P), _ptr(Jh), _ptr(C), nbf, nmo, int(ao["core"]),
                                                int(ao["ndocc"]), _ptr(eps), float(moints.e_ref))
                _check(self.lib, h, rc, "fcc_upload_ao3_df")
            else:
                b = np.asfortranarray(ao["Bmn"], dtype=np.float64)   # [Q, mu, nu], Q fastest
                rc = self.lib.fcc_upload_ao_df(h, _ptr(b), _ptr(C), nbf, nmo, int(ao["core"]), int(ao["ndocc"]),
                                               _ptr(eps), float(moints.e_ref))
                _check(self.lib, h, rc, "fcc_upload_ao_df")
        elif naux > 0:
            Boo = np.asfortranarray(moints.Boo, dtype=np.float64)
            Bov = np.asfortranarray(moints.Bov, dtype=np.float64)
            Bvv = np.asfortranarray(moints.Bvv, dtype=np.float64)
            rc = self.lib.fcc_upload_df(h, _ptr(Boo), _ptr(Bov), _ptr(Bvv), _ptr(eo), _ptr(ev), float(moints.e_ref))
            _check(self.lib, h, rc, "fcc_upload_df")
        else:
            blocks = [np.asfortranarray(moints.conv[k], dtype=np.float64)
                      for k in ("OOOO", "OOOV", "OOVV", "OVOV", "OVVV", "VVVV")]
            rc = self.lib.fcc_upload_conv(h, *[_ptr(b) for b in blocks], _ptr(eo), _ptr(ev), float(moints.e_ref))
            _check(self.lib, h, rc, "fcc_upload_conv")

    def set_guess(self, T1, T2):
        if T1 is None and T2 is None:   # back to the MP2 guess (built on the device)
            _check(self.lib, self.h, self.lib.fcc_set_guess(self.h, None, None), "fcc_set_guess")
            return
        T1f = np.asfortranarray(T1, dtype=np.float64)
        T2f = np.asfortranarray(T2, dtype=np.float64)
        _check(self.lib, self.h, self.lib.fcc_set_guess(self.h, _ptr(T1f), _ptr(T2f)), "fcc_set_guess")

    def run(self, opts: _lib.FccOpts, log_cap: int = 256):
        log = (_lib.FccIterStats * log_cap)()
        res = _lib.FccCCSDResult()
        rc = self.lib.fcc_ccsd_run(self.h, ctypes.byref(opts), log, log_cap, ctypes.byref(res))
        _check(self.lib, self.h, rc, "fcc_ccsd_run")
        lines = [dict(ite=l.ite, energy=l.energy, dE=l.dE, rms=l.rms, seconds=l.seconds, diis=bool(l.diis),
                      precision=l.precision) for l in log[: min(res.iterations, log_cap)]]
        return rc, res, lines

    def amplitudes(self):
        """T1[i, a] and T2[i, j, a, b] as column-major arrays (Fermi's layout;
        the ABI writes that layout, so no host-side copy follows)."""
        T1 = np.empty((self.o, self.v), order="F")
        T2 = np.empty((self.o, self.o, self.v, self.v), order="F")
        _check(self.lib, self.h, self.lib.fcc_get_amps(self.h, _ptr(T1), _ptr(T2)), "fcc_get_amps")
        return T1, T2

    def save_checkpoint(self, path: str):
        """Write the current amplitudes (header + column-major T1, T2)."""
        _check(self.lib, self.h, self.lib.fcc_checkpoint_save(self.h, str(path).encode()), "fcc_checkpoint_save")

    def load_checkpoint(self, path: str):
        """Make the amplitudes of a checkpoint the starting point of the next run."""
        _check(self.lib, self.h, self.lib.fcc_checkpoint_load(self.h, str(path).encode()), "fcc_checkpoint_load")

    def set_checkpoint(self, path: str | None, every: int):
        """Checkpoint every `every` iterations of the next runs and at their end (0: off)."""
        p = str(path).encode() if path else None
        _check(self.lib, self.h, self.lib.fcc_set_checkpoint(self.h, p, int(every)), "fcc_set_checkpoint")

    def mp2_energy(self) -> float:
        """MP2 correlation energy of the uploaded integrals (RMP2a.jl:91-140)."""
        e = ctypes.c_double()
        _check(self.lib, self.h, self.lib.fcc_mp2_energy(self.h, ctypes.byref(e)), "fcc_mp2_energy")
        return e.value

    def triples(self, precision: int) -> float:
        et = ctypes.c_double()
        _check(self.lib, self.h, self.lib.fcc_triples(self.h, precision, ctypes.byref(et)), "fcc_triples")
        return et.value

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fcc_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _opts_from_options() -> _lib.FccOpts:
    lib = _lib.load()
    o = _lib.FccOpts()
    lib.fcc_default_opts(ctypes.byref(o))
    o.max_iter = Options.get("cc_max_iter")
    o.e_conv = Options.get("cc_e_conv")
    o.max_rms = Options.get("cc_max_rms")
    o.diis = int(Options.get("cc_diis"))
    o.ndiis = Options.get("cc_ndiis")
    o.diis_start = Options.get("diis_start")
    o.diis_relax = Options.get("cc_diis_relax")
    prec = Options.get("diis_prec")
    if prec not in ("single", "double"):
        raise FermiException(f"diis_prec {prec!r} is not supported by this backend (single or double)")
    o.diis_prec = 32 if prec == "single" else 64
    o.damp = Options.get("cc_damp_ratio")
    p = Options.get("cc_gpu_precision")
    prec = {"fp64": _lib.FCC_PREC_FP64, "mixed": _lib.FCC_PREC_MIXED, "exact": _lib.FCC_PREC_EXACT}
    if p not in prec:
        raise FermiException(f"cc_gpu_precision must be fp64, mixed or exact, got {p!r}")
    o.precision = prec[p]
    o.mixed_switch_rms = Options.get("cc_gpu_switch_rms")
    fin = Options.get("cc_gpu_finish")
    if fin not in ("exact", "fp64"):
        raise FermiException(f"cc_gpu_finish must be exact or fp64, got {fin!r}")
    o.mixed_finish = _lib.FCC_FINISH_EXACT if fin == "exact" else _lib.FCC_FINISH_FP64
    return o


@dataclass
class RMP2:
    """Fields of Fermi's ``struct RMP2`` (MollerPlesset/RMP2/RMP2.jl:50-53)."""
    correlation: float
    energy: float

    @classmethod
    def compute(cls, moints, alg=None, context: Context | None = None) -> "RMP2":
        alg = alg if alg is not None else get_rmp2_alg()
        if not isinstance(alg, RMP2cuda):
            raise FermiException(f"invalid arguments for RMP2 method: {type(alg).__name__}")
        ctx = context or Context(moints)
        e = ctx.mp2_energy()
        return cls(e, e + moints.e_ref)


@dataclass
class RCCSD:
    """Fields of Fermi's ``struct RCCSD`` plus the iteration table."""
    guessenergy: float
    correlation: float
    energy: float
    T1: np.ndarray
    T2: np.ndarray
    e_conv: float
    t_conv: float
    iterations: list = field(default_factory=list)
    converged: bool = False
    context: Context | None = field(default=None, repr=False)

    @classmethod
    def compute(cls, moints, T1guess=None, T2guess=None, alg=None, context: Context | None = None,
                guess_model=None) -> "RCCSD":
        alg = alg if alg is not None else get_rccsd_alg()
        if not isinstance(alg, RCCSDcuda):
            raise FermiException(f"invalid arguments for RCCSD method: {type(alg).__name__}")
        o_max = moints.o + moints.v
        if moints.o <= 0 or moints.v <= 0 or moints.o >= o_max:
            raise FermiException("invalid number of occupied / virtual orbitals")
        ctx = context or Context(moints)
        if (T1guess is None) != (T2guess is None):
            raise FermiException("give both T1guess and T2guess or neither")
        if T1guess is not None:
            ctx.set_guess(T1guess, T2guess)
        elif Options.get("cc_gpu_guess") == "mlp":
            from .mlp import DEFAULT_PARAMS, MLPGuess
            model = guess_model or MLPGuess(Options.get("cc_gpu_device"), DEFAULT_PARAMS)
            model.guess(ctx)
        elif Options.get("cc_gpu_guess") != "mp2":
            raise FermiException(f"cc_gpu_guess must be mp2 or mlp, got {Options.get('cc_gpu_guess')!r}")
        every = int(Options.get("cc_gpu_checkpoint_every"))
        path = Options.get("cc_gpu_checkpoint")
        if every < 0 or (every > 0 and not path):
            raise FermiException("cc_gpu_checkpoint_every > 0 needs a cc_gpu_checkpoint path")
        ctx.set_checkpoint(path if every > 0 else None, every)
        rc, res, lines = ctx.run(_opts_from_options())
        T1, T2 = ctx.amplitudes()
        return cls(res.guessenergy, res.correlation, res.energy, T1, T2, res.e_conv, res.t_conv,
                   lines, bool(res.converged), ctx)


@dataclass
class RCCSDpT:
    """Fields of Fermi's ``struct RCCSDpT``."""
    CCSD: RCCSD
    energy: float
    correction: float

    @classmethod
    def compute(cls, ccsd: RCCSD, moints=None, alg=None) -> "RCCSDpT":
        alg = alg if alg is not None else get_pt_alg()
        if not isinstance(alg, CudaPT):
            raise FermiException(f"invalid arguments for RCCSD(T) method: {type(alg).__name__}")
        if ccsd.context is None:
            raise FermiException("the RCCSD object holds no device context")
        p = Options.get("pt_gpu_precision")
        if p not in ("fp64", "mixed"):
            raise FermiException(f"pt_gpu_precision must be fp64 or mixed, got {p!r}")
        et = ccsd.context.triples(_lib.FCC_PREC_FP64 if p == "fp64" else _lib.FCC_PREC_MIXED)
        return cls(ccsd, et + ccsd.energy, et)


def energy(method: str, moints):
    """``@energy ccsd`` / ``@energy ccsd(t)`` on prepared MO integrals."""
    m = method.lower().replace(" ", "")
    if m in ("mp2", "rmp2"):
        return RMP2.compute(moints)
    if m in ("ccsd", "rccsd"):
        return RCCSD.compute(moints)
    if m in ("ccsd(t)", "rccsd(t)"):
        return RCCSDpT.compute(RCCSD.compute(moints), moints)
    raise FermiException(f"unknown method {method!r}")
