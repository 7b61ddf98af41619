"""ORACLE (test infrastructure only): numpy statement of the GPU formulation.

The GPU path evaluates the CCSD residual in the T1-dressed density-fitted form
(Koch et al., J. Chem. Phys. 100, 4393 (1994); DePrince & Sherrill,
J. Chem. Theory Comput. 9, 2687 (2013)) instead of the reference's
term-by-term expansion (src/Methods/CoupledCluster/RCCSD/RCCSDHelper.jl:57-192).
This module states that formulation in plain numpy so the test suite can show,
on the CPU and for arbitrary amplitudes, that it is the same function as the
restated reference equations in ``oracle/rccsd.py``:

    reference pre-denominator amplitudes = residual + D * T.

Only tests import it.
"""
from __future__ import annotations

import numpy as np


def _e(s, *a):
    return np.einsum(s, *a, optimize=True)


def full_B(Boo, Bov, Bvv):
    Q, o, _ = Boo.shape
    v = Bvv.shape[1]
    B = np.zeros((Q, o + v, o + v))
    B[:, :o, :o] = Boo
    B[:, :o, o:] = Bov
    B[:, o:, :o] = Bov.transpose(0, 2, 1)
    B[:, o:, o:] = Bvv
    return B


def dressed(t1, B, eps):
    """Dressed factors Bt = X B Y^T and dressed Fock F = X h Y^T + G(Bt),
    X = 1 - T, Y = 1 + T^T, T[a,i] = t_ia, h = diag(eps) - G(B)."""
    Q, n, _ = B.shape
    o = t1.shape[0]
    T = np.zeros((n, n))
    T[o:, :o] = t1.T
    X = np.eye(n) - T
    Y = np.eye(n) + T.T
    Bt = _e("pt,Qtu,qu->Qpq", X, B, Y)

    def G(BB):
        return 2 * _e("Qpq,Qkk->pq", BB, BB[:, :o, :o]) - _e("Qpk,Qkq->pq", BB[:, :, :o], BB[:, :o, :])

    F = X @ (np.diag(eps) - G(B)) @ Y.T + G(Bt)
    return Bt, F


def residual(t1, t2, Boo, Bov, Bvv, eps_o, eps_v):
    """Full CCSD residuals (Omega_ia, Omega_ijab); zero at convergence."""
    o = t1.shape[0]
    B = full_B(Boo, Bov, Bvv)
    n = B.shape[1]
    Bt, F = dressed(t1, B, np.concatenate([eps_o, eps_v]))
    O, V = slice(0, o), slice(o, n)
    g = lambda p, q, r, s: _e("Qpq,Qrs->pqrs", Bt[:, p, q], Bt[:, r, s])
    u = 2 * t2 - t2.transpose(1, 0, 2, 3)
    ovov = g(O, V, O, V)
    R2 = _e("aibj->ijab", g(V, O, V, O))
    R2 += _e("ijcd,acbd->ijab", t2, g(V, V, V, V))
    R2 += _e("klab,kilj->ijab", t2, g(O, O, O, O) + _e("ijcd,kcld->kilj", t2, ovov))
    Cint = g(O, O, V, V) - 0.5 * _e("liad,kdlc->kiac", t2, ovov)
    C = -0.5 * _e("kjbc,kiac->ijab", t2, Cint) - _e("kibc,kjac->ijab", t2, Cint)
    L = 2 * ovov - ovov.transpose(0, 3, 2, 1)
    Dint = 2 * g(V, O, O, V) - _e("acki->aikc", g(V, V, O, O)) + 0.5 * _e("ilad,ldkc->aikc", u, L)
    D = 0.5 * _e("jkbc,aikc->ijab", u, Dint)
    Fvv = F[V, V] - _e("klbd,ldkc->bc", u, ovov)
    Foo = F[O, O] + _e("jlcd,kcld->kj", u, ovov)
    E = _e("ijac,bc->ijab", t2, Fvv) - _e("ikab,kj->ijab", t2, Foo)
    P = C + D + E
    R2 += P + P.transpose(1, 0, 3, 2)
    R1 = F[V, O].T.copy()
    R1 += _e("kicd,adkc->ia", u, g(V, V, O, V))
    R1 -= _e("klac,kilc->ia", u, g(O, O, O, V))
    R1 += _e("ikac,kc->ia", u, F[O, V])
    return R1, R2
