"""GB300 backend for Fermi.jl's RCCSD / DF-RCCSD / RCCSD(T) path.

Compute runs in hand-written sm_103a CUDA kernels behind the C ABI of
``libfermicc.so`` (include/fermicc.h); this package is the host-side mirror of
Fermi's method objects and options, plus the stand-in input pipeline
(``fermicc.inputs``) that produces the integrals Fermi would hand over.
"""
from . import options as Options
from .options import FermiException
from .rhf import RHF, DFFock, RHFcuda, get_rhf_alg
from .rccsd import (CudaPT, RCCSD, RCCSDcuda, RCCSDpT, RMP2, RMP2cuda, energy, get_pt_alg, get_rccsd_alg,
                    get_rmp2_alg)

__all__ = ["Options", "FermiException", "RCCSD", "RCCSDpT", "RCCSDcuda", "CudaPT", "RMP2", "RMP2cuda", "energy",
           "get_rccsd_alg", "get_pt_alg", "get_rmp2_alg", "RHF", "RHFcuda", "DFFock", "get_rhf_alg"]
