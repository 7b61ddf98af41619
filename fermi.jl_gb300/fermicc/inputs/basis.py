"""Stand-in Gaussian basis sets with the shell structure of cc-pVDZ / cc-pVDZ-RI.

Fermi.jl reads basis sets from Gaussian94 files through GaussianBasis.jl
(``src/Core/Integrals/IntegralHelper.jl:79-89`` picks the orbital basis and
the RI / JK fitting basis; ``src/Core/Integrals/ERITypes.jl:84-95`` maps
``rifit auto`` to ``<basis>-rifit``).  No basis-set file ships with this package,
so the coupled-cluster inputs are produced on project-defined basis sets that
keep the published SHELL STRUCTURE and therefore the dimensions of every
tensor on the coupled-cluster path:

* orbital basis, spherical functions: O 3s2p1d (14), H 2s1p (5): 24 per water;
* fitting basis: O 7s5p4d2f (56), H 3s2p1d (14): 84 per water.

The exponents and contraction coefficients are NOT those of cc-pVDZ.  They are
defined here: contracted shells are least-squares fits of Slater-type radial
functions (exponents from Slater's screening rules) by even-tempered Gaussian
primitives; the remaining shells are single primitives.  Every energy produced
with them is "on the stand-in basis".

The same fitting basis is used for the SCF (Fermi's JKFIT role) and for the
coupled-cluster factors (RIFIT role).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ANGSTROM_TO_BOHR = 1.0 / 0.52917721092
Z_OF = {"H": 1, "O": 8}
# Frozen-core orbital count per element: the rule of Fermi's ``@freezecore``
# (src/Core/Options.jl:512-527 with src/Backend/PhysicalConstants.jl:218-226):
# elements 3-10 freeze their two 1s electrons, i.e. one orbital.
FROZEN_ORBITALS = {"H": 0, "O": 1}


def _even_tempered(first: float, ratio: float, n: int) -> np.ndarray:
    return first * ratio ** np.arange(n)


def _sto_fit(n_qn: int, l: int, zeta: float, nprim: int) -> tuple[np.ndarray, np.ndarray]:
    """Fit r^(n-1) exp(-zeta r) by sum_k c_k r^l exp(-a_k r^2), a_k even-tempered.

    Linear least squares with weight r^2 on a radial grid.  Returns exponents
    and coefficients of the (unnormalised) primitives r^l exp(-a r^2).
    """
    base = _even_tempered(0.06, 3.2, nprim)           # spans the 1/zeta^2 scale
    alphas = zeta * zeta * base
    r = np.linspace(1e-4, 30.0 / zeta, 6000)
    w = r * r
    target = r ** (n_qn - 1) * np.exp(-zeta * r)
    G = np.stack([r ** l * np.exp(-a * r * r) for a in alphas], axis=1)
    A = G.T @ (G * w[:, None])
    b = G.T @ (target * w)
    c = np.linalg.solve(A, b)
    return alphas, c


@dataclass
class Shell:
    """A contracted shell; ``coefs`` multiply unnormalised primitives."""
    l: int
    exps: np.ndarray
    coefs: np.ndarray


def _prim(a: float, l: int) -> Shell:
    return Shell(l, np.array([a]), np.array([1.0]))


def _fit(n_qn: int, l: int, zeta: float, nprim: int) -> Shell:
    a, c = _sto_fit(n_qn, l, zeta, nprim)
    return Shell(l, a, c)


def orbital_shells(element: str) -> list[Shell]:
    if element == "O":
        return [
            _fit(1, 0, 7.66, 6),      # 1s  (Slater zeta for O 1s)
            _fit(2, 0, 2.25, 3),      # 2s  (Slater zeta for O 2s/2p)
            _prim(0.30, 0),
            _fit(2, 1, 2.25, 3),      # 2p
            _prim(0.27, 1),
            _prim(1.20, 2),
        ]
    if element == "H":
        return [
            _fit(1, 0, 1.24, 3),
            _prim(0.16, 0),
            _prim(0.73, 1),
        ]
    raise ValueError(f"no stand-in orbital basis for {element}")


def fitting_shells(element: str) -> list[Shell]:
    if element == "O":
        s = [80.0, 30.0, 12.0, 5.0, 2.2, 1.0, 0.45]
        p = [12.0, 5.0, 2.2, 1.0, 0.45]
        d = [6.0, 2.6, 1.1, 0.5]
        f = [2.5, 1.0]
        return ([_prim(a, 0) for a in s] + [_prim(a, 1) for a in p]
                + [_prim(a, 2) for a in d] + [_prim(a, 3) for a in f])
    if element == "H":
        return ([_prim(a, 0) for a in (4.0, 1.2, 0.4)] + [_prim(a, 1) for a in (2.0, 0.6)]
                + [_prim(1.0, 2)])
    raise ValueError(f"no stand-in fitting basis for {element}")


def _double_factorial(n: int) -> float:
    return float(math.prod(range(n, 0, -2))) if n > 0 else 1.0


def prim_norm(a: float, l: int) -> float:
    """Normalisation of x^l exp(-a r^2)."""
    return (2 * a / math.pi) ** 0.75 * (4 * a) ** (l / 2) / math.sqrt(_double_factorial(2 * l - 1))


@dataclass
class FlatBasis:
    """Flat shell arrays in the layout the integral library expects."""
    xyz: np.ndarray
    lq: np.ndarray
    np_: np.ndarray
    po: np.ndarray
    ex: np.ndarray
    co: np.ndarray
    nbf: int
    shell_atom: list = field(default_factory=list)


def flatten(atoms: list[tuple[str, np.ndarray]], shells_of) -> FlatBasis:
    xyz, lq, npr, po, ex, co, sa = [], [], [], [], [], [], []
    off = 0
    nbf = 0
    for ia, (el, pos) in enumerate(atoms):
        for sh in shells_of(el):
            xyz.append(pos)
            lq.append(sh.l)
            npr.append(len(sh.exps))
            po.append(off)
            off += len(sh.exps)
            ex.extend(sh.exps.tolist())
            # coefficients multiply the unnormalised primitives x^l exp(-a r^2)
            co.extend(sh.coefs.tolist())
            nbf += 2 * sh.l + 1
            sa.append(ia)
    return FlatBasis(
        xyz=np.ascontiguousarray(np.array(xyz, dtype=np.float64).reshape(-1, 3)),
        lq=np.array(lq, dtype=np.int32), np_=np.array(npr, dtype=np.int32),
        po=np.array(po, dtype=np.int32), ex=np.array(ex, dtype=np.float64),
        co=np.array(co, dtype=np.float64), nbf=nbf, shell_atom=sa)
