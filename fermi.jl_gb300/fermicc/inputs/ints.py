"""ctypes binding of the Gaussian-integral library (gauss_ints.c).

The shared object is built by ``__graft_entry__.build()``; ``load()`` also
builds it on first use if it is missing or older than its source, so the input
pipeline works on a fresh checkout of either machine (plain gcc, no CUDA).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from .basis import FlatBasis

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "gauss_ints.c")
_LIB = os.path.join(_HERE, "libfcc_ints.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        basis_args = [ctypes.c_int, dp, ip, ip, ip, dp, dp]
        lib.fcci_one_body.argtypes = basis_args + [ctypes.c_int, dp, dp, dp, dp, dp]
        lib.fcci_eri2c.argtypes = basis_args + [dp]
        lib.fcci_eri3c.argtypes = basis_args + basis_args + [dp]
        lib.fcci_eri4c.argtypes = basis_args + [dp]
        for f in (lib.fcci_one_body, lib.fcci_eri2c, lib.fcci_eri3c, lib.fcci_eri4c):
            f.restype = ctypes.c_int
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _bargs(b: FlatBasis):
    return [len(b.lq), _dp(b.xyz), _ip(b.lq), _ip(b.np_), _ip(b.po), _dp(b.ex), _dp(b.co)]


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"{what}: integral library rejected the basis (rc={rc})")


def one_body(b: FlatBasis, atom_xyz: np.ndarray, charges: np.ndarray):
    lib = load()
    n = b.nbf
    S = np.zeros((n, n)); T = np.zeros((n, n)); V = np.zeros((n, n))
    axyz = np.ascontiguousarray(atom_xyz, dtype=np.float64)
    Z = np.ascontiguousarray(charges, dtype=np.float64)
    _check(lib.fcci_one_body(*_bargs(b), len(Z), _dp(axyz), _dp(Z), _dp(S), _dp(T), _dp(V)), "one_body")
    return S, T, V


def eri2c(aux: FlatBasis):
    lib = load()
    out = np.zeros((aux.nbf, aux.nbf))
    _check(lib.fcci_eri2c(*_bargs(aux), _dp(out)), "eri2c")
    return out


def eri3c(b: FlatBasis, aux: FlatBasis):
    lib = load()
    out = np.zeros((b.nbf, b.nbf, aux.nbf))
    _check(lib.fcci_eri3c(*_bargs(b), *_bargs(aux), _dp(out)), "eri3c")
    return out


def eri4c(b: FlatBasis):
    lib = load()
    n = b.nbf
    out = np.zeros((n, n, n, n))
    _check(lib.fcci_eri4c(*_bargs(b), _dp(out)), "eri4c")
    return out
