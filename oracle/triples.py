"""ORACLE (test infrastructure only): CPU restatement of Fermi.jl's RCCSD(T).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module.

* ``triples_ijk``  src/Methods/CoupledCluster/PerturbativeTriples/ijk.jl:20-149
  (Fermi's default ``pt_alg = 1``): loops i >= j >= k, builds W and V (v^3)
  from twelve contractions, then sums the six-fold permutation energy over
  a >= b >= c with weight (2 - d_ij - d_jk) / (D_ijkabc (1 + d_ab + d_bc)).
* ``triples_abc``  PerturbativeTriples/abc.jl:28-167 (``pt_alg = 3``): loops
  a >= b >= c over o^3 blocks.  ``corrected=False`` restates the file exactly
  as written; at abc.jl:128 and abc.jl:131 the reference multiplies by
  ``T2_c`` where the (jki)(bca) and (kji)(cba) permutations of the first term
  need ``T2_a``.  ``corrected=True`` uses ``T2_a`` there and agrees with
  ``triples_ijk``; the literal restatement does not.  The GPU path follows the
  default ijk algorithm.

Index conventions follow the reference: the ijk restatement first forms the
same permuted arrays as ijk.jl:24-32.  The scalar a >= b >= c loop of
ijk.jl:121-137 is evaluated here over the whole v^3 cube with a mask, which
sums the same terms.
"""
from __future__ import annotations

import numpy as np


def _e(subs, *ops):
    return np.einsum(subs, *ops, optimize=True)


def _wv_ijk(i, j, k, T1p, T2p, Vvvvo, Vvooo, Vvvoo):
    """W and V of ijk.jl:108-117 for one occupied triplet (0-based)."""
    T2_i, T2_j, T2_k = T2p[:, :, :, i], T2p[:, :, :, j], T2p[:, :, :, k]
    W = _e("dba,dc->abc", Vvvvo[:, :, :, i], T2p[:, :, j, k]) - _e("bl,acl->abc", Vvooo[:, :, i, j], T2_k)   # :109
    W += _e("dab,dc->abc", Vvvvo[:, :, :, j], T2p[:, :, i, k]) - _e("al,bcl->abc", Vvooo[:, :, j, i], T2_k)  # :110
    W += _e("dac,db->abc", Vvvvo[:, :, :, k], T2p[:, :, i, j]) - _e("al,cbl->abc", Vvooo[:, :, k, i], T2_j)  # :111
    W += _e("dbc,ad->abc", Vvvvo[:, :, :, k], T2p[:, :, i, j]) - _e("bl,cal->abc", Vvooo[:, :, k, j], T2_i)  # :112
    W += _e("dca,bd->abc", Vvvvo[:, :, :, i], T2p[:, :, j, k]) - _e("cl,abl->abc", Vvooo[:, :, i, k], T2_j)  # :113
    W += _e("dcb,ad->abc", Vvvvo[:, :, :, j], T2p[:, :, i, k]) - _e("cl,bal->abc", Vvooo[:, :, j, k], T2_i)  # :114
    V = (W + _e("a,bc->abc", T1p[:, i], Vvvoo[:, :, j, k]) + _e("ac,b->abc", Vvvoo[:, :, i, k], T1p[:, j])
         + _e("ab,c->abc", Vvvoo[:, :, i, j], T1p[:, k]))                                                     # :116
    return W, V


def _energy_block(W, V, Dd, mask_w):
    """Six-fold permutation energy of ijk.jl:129-133 summed over the cube,
    with ``mask_w[a,b,c]`` = 1/(1 + d_ab + d_bc) on a >= b >= c, else 0."""
    P = lambda A, s: np.einsum(s + "->abc", A)
    Wabc, Wacb, Wbac, Wbca, Wcab, Wcba = (P(W, "abc"), P(W, "acb"), P(W, "bac"), P(W, "bca"),
                                          P(W, "cab"), P(W, "cba"))
    Vabc, Vacb, Vbac, Vbca, Vcab, Vcba = (P(V, "abc"), P(V, "acb"), P(V, "bac"), P(V, "bca"),
                                          P(V, "cab"), P(V, "cba"))
    X = Wabc * Vabc + Wacb * Vacb + Wbac * Vbac + Wbca * Vbca + Wcab * Vcab + Wcba * Vcba   # :129
    Y = Vabc + Vbca + Vcab                                                                   # :130
    Z = Vacb + Vbac + Vcba                                                                   # :131
    Ef = (Y - 2 * Z) * (Wabc + Wbca + Wcab) + (Z - 2 * Y) * (Wacb + Wbac + Wcba) + 3 * X      # :132
    return float(np.sum(Ef * mask_w / Dd))


def triples_setup(T1, T2, OVVV, OOOV, OVOV):
    """Permuted copies of ijk.jl:24-32."""
    T1p = np.ascontiguousarray(T1.T)                         # (v, o)      :24
    T2p = np.ascontiguousarray(T2.transpose(3, 2, 1, 0))     # [b,a,j,i]   :25
    Vvvvo = np.ascontiguousarray(OVVV.transpose(3, 2, 1, 0))  # :28
    Vvooo = np.ascontiguousarray(np.einsum("ijka->aijk", OOOV))   # permutedims(OOOV,(4,1,2,3)) :31
    Vvvoo = np.ascontiguousarray(np.einsum("iajb->abij", OVOV))   # permutedims(OVOV,(2,4,1,3)) :32
    return T1p, T2p, Vvvvo, Vvooo, Vvvoo


def triplet_list(o: int):
    """The i >= j >= k loop order of ijk.jl:49,63,83 (0-based)."""
    return [(i, j, k) for i in range(o) for j in range(i + 1) for k in range(j + 1)]


def abc_weights(v: int) -> np.ndarray:
    a = np.arange(v)[:, None, None]
    b = np.arange(v)[None, :, None]
    c = np.arange(v)[None, None, :]
    mask = (a >= b) & (b >= c)
    return np.where(mask, 1.0 / (1.0 + (a == b) + (b == c)), 0.0)


def triples_ijk(T1, T2, OVVV, OOOV, OVOV, eps_o, eps_v, triplets=None) -> float:
    """E(T) of ijk.jl:20-149.  ``triplets`` restricts the sum to a subset of
    (i, j, k) (used to time a bounded sample); default is all i >= j >= k."""
    o, v = T1.shape
    T1p, T2p, Vvvvo, Vvooo, Vvvoo = triples_setup(T1, T2, OVVV, OOOV, OVOV)
    mw = abc_weights(v)
    fv = eps_v
    Dv = fv[:, None, None] + fv[None, :, None] + fv[None, None, :]
    E = 0.0
    for (i, j, k) in (triplets if triplets is not None else triplet_list(o)):
        wgt = 2 - (i == j) - (j == k)                         # :133
        if wgt == 0:
            continue
        W, V = _wv_ijk(i, j, k, T1p, T2p, Vvvvo, Vvooo, Vvvoo)
        Dd = eps_o[i] + eps_o[j] + eps_o[k] - Dv              # :86,119,123,126
        E += wgt * _energy_block(W, V, Dd, mw)
    return E


def triples_abc(T1, T2, OVVV, OOOV, OVOV, eps_o, eps_v, corrected: bool = False) -> float:
    """E(T) of abc.jl:28-167 (see the module docstring for ``corrected``)."""
    o, v = T1.shape
    ovvv = OVVV.transpose(0, 2, 1, 3)      # permutedims(OVVV,(1,3,2,4)): ovvv[i,b,a,c]=(ia|bc)  :37
    ooov = OOOV.transpose(0, 2, 1, 3)      # :38
    oovv = OVOV.transpose(0, 2, 1, 3)      # :39
    fo, fv = eps_o, eps_v
    ii = np.arange(o)
    I3 = ii[:, None, None]; J3 = ii[None, :, None]; K3 = ii[None, None, :]
    maskw = np.where((I3 >= J3) & (J3 >= K3), 1.0 / (1.0 + (I3 == J3) + (J3 == K3)), 0.0)
    Do = fo[:, None, None] + fo[None, :, None] + fo[None, None, :]
    E = 0.0
    for a in range(v):
        for b in range(a + 1):
            for c in range(b + 1):
                T2a, T2b, T2c = T2[:, :, :, a], T2[:, :, :, b], T2[:, :, :, c]
                second = T2a if corrected else T2c
                W = _e("id,jkd->ijk", ovvv[:, :, a, b], T2c) - _e("jkl,il->ijk", ooov[:, :, :, c], T2[:, :, a, b])      # :124
                W += _e("id,kjd->ijk", ovvv[:, :, a, c], T2b) - _e("kjl,il->ijk", ooov[:, :, :, b], T2[:, :, a, c])    # :125
                W += _e("jd,ikd->ijk", ovvv[:, :, b, a], T2c) - _e("ikl,jl->ijk", ooov[:, :, :, c], T2[:, :, b, a])    # :127
                W += _e("jd,kid->ijk", ovvv[:, :, b, c], second) - _e("kil,jl->ijk", ooov[:, :, :, a], T2[:, :, b, c])  # :128
                W += _e("kd,ijd->ijk", ovvv[:, :, c, a], T2b) - _e("ijl,kl->ijk", ooov[:, :, :, b], T2[:, :, c, a])    # :130
                W += _e("kd,jid->ijk", ovvv[:, :, c, b], second) - _e("jil,kl->ijk", ooov[:, :, :, a], T2[:, :, c, b])  # :131
                V = (W + _e("jk,i->ijk", oovv[:, :, b, c], T1[:, a]) + _e("ik,j->ijk", oovv[:, :, a, c], T1[:, b])
                     + _e("ij,k->ijk", oovv[:, :, a, b], T1[:, c]))                                                        # :133
                wab = 1 + (a == b) + (b == c)
                Dd = Do - (fv[a] + fv[b] + fv[c])
                # abc.jl:137-151 is the ijk energy with the roles of (ijk) and (abc) swapped
                E += 2.0 / wab * _energy_block(W, V, Dd, maskw)
    return E
