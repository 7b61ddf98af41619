"""Options for the coupled-cluster backend, mirroring ``Fermi.Options``.

Fermi keeps global option dictionaries (``Default`` / ``Current``), lower-cases
keys, rejects unknown keys and coerces values to the default's type
(src/Core/Options.jl:40-189); failures raise ``FermiException``
(src/Core/Options.jl:196-199).  This module keeps the same behaviour for the
keys the coupled-cluster path reads, plus the keys this backend adds:

* ``cc_alg``  -- 2 selects this backend (``RCCSDcuda``); Fermi's 1 is its Julia
  ``RCCSDa`` and is not provided here.
* ``pt_alg``  -- 4 selects this backend's (T) (``CudaPT``); Fermi's 1-3 are its
  Julia ``ijk`` / ``ijk2`` / ``abc``.
* ``mp2_alg`` -- 3 selects this backend's DF-RMP2 energy (``RMP2cuda``); Fermi's
  1-2 are its Julia ``RMP2a`` / ``RMP2b``.
* ``cc_gpu_precision`` -- "fp64", "mixed" (split-BF16 contractions, then
  exact-slice products, then an FP64-accurate finish) or "exact" (every
  residual from exact-slice products at 9 weight groups).
* ``cc_gpu_switch_rms`` -- residual at which the mixed form leaves the
  split-BF16 products.
* ``cc_gpu_finish`` -- finish of the mixed form: "exact" (exact-slice products
  at 9 weight groups, FP64-accurate) or "fp64" (DMMA).
* ``cc_gpu_guess`` -- "mp2" or "mlp" (learned T2 initialiser).
* ``pt_gpu_precision`` -- "fp64" or "mixed" for (T).
* ``cc_gpu_checkpoint`` / ``cc_gpu_checkpoint_every`` -- checkpoint file of the
  amplitudes, written every N iterations and at the end of a run (0: off).
* ``rhf_alg`` -- 3 selects this backend's DF-RHF (``RHFcuda``, device Fock
  build); Fermi's 1-2 are its Julia ``RHFa`` / ``Direct``.  The SCF keys
  (``scf_*``, ``diis``, ``ndiis``, ``oda*``, ``scf_guess``) keep Fermi's
  defaults (src/Core/Options.jl:55-89).
"""
from __future__ import annotations


class FermiException(Exception):
    """Same role as ``Fermi.Options.FermiException``."""


DEFAULT = {
    "cc_alg": 2,
    "pt_alg": 4,
    "mp2_alg": 3,
    "cc_max_iter": 50,
    "cc_max_rms": 1e-10,
    "cc_e_conv": 1e-10,
    "cc_diis": True,
    "cc_ndiis": 3,
    "cc_diis_relax": 3,
    "diis_start": 3,
    "diis_prec": "single",
    "cc_damp_ratio": 0.0,
    "drop_occ": 0,
    "drop_vir": 0,
    "df": True,
    "return_ints": False,
    "precision": "double",
    "cc_gpu_precision": "fp64",
    "cc_gpu_switch_rms": 1e-5,
    "cc_gpu_finish": "exact",
    "cc_gpu_guess": "mp2",
    "pt_gpu_precision": "fp64",
    "cc_gpu_device": 0,
    "cc_gpu_checkpoint": "",
    "cc_gpu_checkpoint_every": 0,
    "rhf_alg": 3,
    "scf_max_iter": 50,
    "scf_max_rms": 1e-9,
    "scf_e_conv": 1e-10,
    "scf_guess": "gwh",
    "diis": True,
    "ndiis": 8,
    "oda": True,
    "oda_cutoff": 1e-1,
    "oda_shutoff": 20,
}

_current: dict = {}


def _coerce(key: str, val):
    ref = DEFAULT[key]
    try:
        if isinstance(ref, bool):
            if isinstance(val, str):
                if val.lower() in ("true", "false"):
                    return val.lower() == "true"
                raise ValueError
            return bool(val)
        if isinstance(ref, int):
            if isinstance(val, float) and not val.is_integer():
                raise ValueError
            return int(val)
        if isinstance(ref, float):
            return float(val)
        if isinstance(ref, str):
            return str(val).lower()
    except (TypeError, ValueError):
        pass
    raise FermiException(f"invalid type for option {key}: {val!r}")


def set(key: str, val) -> None:  # noqa: A001 - mirrors Fermi.Options.set
    k = key.lower()
    if k not in DEFAULT:
        raise FermiException(f"invalid option: {key}")
    _current[k] = _coerce(k, val)


def get(key: str):
    k = key.lower()
    if k not in DEFAULT:
        raise FermiException(f"invalid option: {key}")
    return _current.get(k, DEFAULT[k])


def reset(key: str | None = None) -> None:
    if key is None:
        _current.clear()
    else:
        _current.pop(key.lower(), None)
