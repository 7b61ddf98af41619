"""ORACLE (test infrastructure only): an independent spin-orbital CCSD and (T).

This is a second, separately written formulation used to pin the closed-shell
restatement in ``oracle/rccsd.py`` / ``oracle/triples.py`` (Fermi.jl itself
cannot run here).  It shares no code with them: it works with antisymmetrised
spin-orbital integrals <pq||rs> and the published equations of

* J. F. Stanton, J. Gauss, J. D. Watts and R. J. Bartlett,
  J. Chem. Phys. 94, 4334 (1991) -- CCSD with the F/W intermediates;
* K. Raghavachari, G. W. Trucks, J. A. Pople and M. Head-Gordon,
  Chem. Phys. Lett. 157, 479 (1989) -- (T), written with connected and
  disconnected triples and the 1/36 prefactor over unrestricted sums.

For an RHF reference both must reproduce the closed-shell energies to
round-off.  Only small systems are practical (the full <pq||rs> is built).
"""
from __future__ import annotations

import numpy as np


def _e(s, *ops):
    return np.einsum(s, *ops, optimize=True)


def full_spatial_eri(blocks: dict, o: int, v: int) -> np.ndarray:
    """Assemble (pq|rs) over all o+v spatial MOs from the OOOO..VVVV blocks
    using the eight-fold permutational symmetry of real orbitals."""
    n = o + v
    g = np.zeros((n, n, n, n))
    O, V = slice(0, o), slice(o, n)
    sl = {"O": O, "V": V}

    perms = ((0, 1, 2, 3), (1, 0, 2, 3), (0, 1, 3, 2), (1, 0, 3, 2),
             (2, 3, 0, 1), (3, 2, 0, 1), (2, 3, 1, 0), (3, 2, 1, 0))
    for key in ("OOOO", "OOOV", "OOVV", "OVOV", "OVVV", "VVVV"):
        arr = blocks[key]
        S = [sl[c] for c in key]
        for pm in perms:
            g[S[pm[0]], S[pm[1]], S[pm[2]], S[pm[3]]] = arr.transpose(pm)
    return g


def full_spatial_eri_df(Boo, Bov, Bvv) -> np.ndarray:
    Q, o, _ = Boo.shape
    v = Bvv.shape[1]
    B = np.zeros((Q, o + v, o + v))
    B[:, :o, :o] = Boo
    B[:, :o, o:] = Bov
    B[:, o:, :o] = Bov.transpose(0, 2, 1)
    B[:, o:, o:] = Bvv
    return _e("Qpq,Qrs->pqrs", B, B)


def spin_orbital(g: np.ndarray, eps: np.ndarray, o: int):
    """Antisymmetrised <pq||rs> and orbital energies in the spin-orbital basis,
    ordered occupied (alpha, beta interleaved) then virtual."""
    n = g.shape[0]
    order = [p for p in range(o)] + [p for p in range(o, n)]
    so = [(p, s) for p in order for s in (0, 1)]
    N = len(so)
    sp = np.array([p for p, _ in so])
    ss = np.array([s for _, s in so])
    # <pq|rs> = (pr|qs) delta(sp,sr) delta(sq,ss)
    phys = g[np.ix_(sp, sp, sp, sp)].transpose(0, 2, 1, 3)
    spin_pr = (ss[:, None] == ss[None, :])
    mask = spin_pr[:, None, :, None] & spin_pr[None, :, None, :]
    phys = phys * mask
    anti = phys - phys.transpose(0, 1, 3, 2)
    return anti, eps[sp], 2 * o, N


def ccsd(anti, f_diag, no, conv=1e-12, max_iter=200, ccd=False):
    """Stanton-Gauss CCSD with Jacobi updates and a simple DIIS on (t1, t2);
    ``ccd`` keeps t1 at zero (CCD)."""
    N = anti.shape[0]
    o, v = slice(0, no), slice(no, N)
    nv = N - no
    fo, fv = f_diag[:no], f_diag[no:]
    Dia = fo[:, None] - fv[None, :]
    Dijab = fo[:, None, None, None] + fo[None, :, None, None] - fv[None, None, :, None] - fv[None, None, None, :]
    oovv, ovov = anti[o, o, v, v], None
    t1 = np.zeros((no, nv))
    t2 = anti[o, o, v, v] / Dijab
    hist_t, hist_e = [], []
    E_old = 0.0
    for it in range(max_iter):
        tau_t = t2 + 0.5 * (_e("ia,jb->ijab", t1, t1) - _e("ib,ja->ijab", t1, t1))
        tau = t2 + _e("ia,jb->ijab", t1, t1) - _e("ib,ja->ijab", t1, t1)
        Fae = _e("mf,mafe->ae", t1, anti[o, v, v, v]) - 0.5 * _e("mnaf,mnef->ae", tau_t, oovv)
        Fmi = _e("ne,mnie->mi", t1, anti[o, o, o, v]) + 0.5 * _e("inef,mnef->mi", tau_t, oovv)
        Fme = _e("nf,mnef->me", t1, oovv)
        Wmnij = (anti[o, o, o, o] + _e("je,mnie->mnij", t1, anti[o, o, o, v])
                 - _e("ie,mnje->mnij", t1, anti[o, o, o, v]) + 0.25 * _e("ijef,mnef->mnij", tau, oovv))
        Wabef = (anti[v, v, v, v] - _e("mb,amef->abef", t1, anti[v, o, v, v])
                 + _e("ma,bmef->abef", t1, anti[v, o, v, v]) + 0.25 * _e("mnab,mnef->abef", tau, oovv))
        Wmbej = (anti[o, v, v, o] + _e("jf,mbef->mbej", t1, anti[o, v, v, v])
                 - _e("nb,mnej->mbej", t1, anti[o, o, v, o])
                 - _e("jnfb,mnef->mbej", 0.5 * t2 + _e("jf,nb->jnfb", t1, t1), oovv))
        r1 = (_e("ie,ae->ia", t1, Fae) - _e("ma,mi->ia", t1, Fmi) + _e("imae,me->ia", t2, Fme)
              - _e("nf,naif->ia", t1, anti[o, v, o, v]) - 0.5 * _e("imef,maef->ia", t2, anti[o, v, v, v])
              - 0.5 * _e("mnae,nmei->ia", t2, anti[o, o, v, o]))
        Fbe = Fae - 0.5 * _e("mb,me->be", t1, Fme)
        Fmj = Fmi + 0.5 * _e("je,me->mj", t1, Fme)
        tmp = _e("ijae,be->ijab", t2, Fbe)
        r2 = anti[o, o, v, v] + tmp - tmp.transpose(0, 1, 3, 2)
        tmp = _e("imab,mj->ijab", t2, Fmj)
        r2 -= tmp - tmp.transpose(1, 0, 2, 3)
        r2 += 0.5 * _e("mnab,mnij->ijab", tau, Wmnij) + 0.5 * _e("ijef,abef->ijab", tau, Wabef)
        tmp = _e("imae,mbej->ijab", t2, Wmbej) - _e("ie,ma,mbej->ijab", t1, t1, anti[o, v, v, o])
        r2 += tmp - tmp.transpose(1, 0, 2, 3) - tmp.transpose(0, 1, 3, 2) + tmp.transpose(1, 0, 3, 2)
        tmp = _e("ie,abej->ijab", t1, anti[v, v, v, o])
        r2 += tmp - tmp.transpose(1, 0, 2, 3)
        tmp = _e("ma,mbij->ijab", t1, anti[o, v, o, o])
        r2 -= tmp - tmp.transpose(0, 1, 3, 2)
        n1, n2 = r1 / Dia, r2 / Dijab
        if ccd:
            n1 = np.zeros_like(n1)
        err = np.concatenate([(n1 - t1).ravel(), (n2 - t2).ravel()])
        vec = np.concatenate([n1.ravel(), n2.ravel()])
        hist_t.append(vec); hist_e.append(err)
        if len(hist_t) > 8:
            hist_t.pop(0); hist_e.pop(0)
        if len(hist_t) >= 3:
            m = len(hist_t)
            B = -np.ones((m + 1, m + 1)); B[m, m] = 0
            for a in range(m):
                for b in range(m):
                    B[a, b] = hist_e[a] @ hist_e[b]
            rhs = np.zeros(m + 1); rhs[m] = -1
            c = np.linalg.solve(B, rhs)[:m]
            vec = sum(ci * hv for ci, hv in zip(c, hist_t))
        t1 = vec[: no * nv].reshape(no, nv)
        t2 = vec[no * nv:].reshape(no, no, nv, nv)
        E = 0.25 * _e("ijab,ijab->", oovv, t2) + 0.5 * _e("ijab,ia,jb->", oovv, t1, t1)
        if abs(E - E_old) < conv and np.abs(err).max() < 1e-9:
            return float(E), t1, t2
        E_old = E
    raise RuntimeError("spin-orbital CCSD did not converge")


def triples(anti, f_diag, no, t1, t2) -> float:
    """(T) with connected/disconnected triples over unrestricted sums / 36."""
    N = anti.shape[0]
    o, v = slice(0, no), slice(no, N)
    fo, fv = f_diag[:no], f_diag[no:]
    vvvo = anti[v, v, v, o]      # <bc||ei> = <ei||bc> for real orbitals
    ovoo = anti[o, v, o, o]
    oovv = anti[o, o, v, v]
    Dv = -(fv[:, None, None] + fv[None, :, None] + fv[None, None, :])
    E = 0.0

    def P_ia(fn, i, j, k):
        return fn(i, j, k) - fn(j, i, k) - fn(k, j, i)

    def perm_abc(X):
        # P(a/bc) X[a,b,c] = X[a,b,c] - X[b,a,c] - X[c,b,a]
        return X - X.transpose(1, 0, 2) - X.transpose(2, 1, 0)

    for i in range(no):
        for j in range(no):
            for k in range(no):
                if len({i, j, k}) < 3:
                    continue

                def conn(i_, j_, k_):
                    # sum_e t_{jk ae} <ei||bc> - sum_m t_{im bc} <ma||jk>
                    a1 = _e("ae,bce->abc", t2[j_, k_], vvvo[:, :, :, i_])
                    a2 = _e("mbc,ma->abc", t2[i_], ovoo[:, :, j_, k_])
                    return a1 - a2

                def disc(i_, j_, k_):
                    return _e("a,bc->abc", t1[i_], oovv[j_, k_])

                c = perm_abc(P_ia(conn, i, j, k))
                d = perm_abc(P_ia(disc, i, j, k))
                D = fo[i] + fo[j] + fo[k] + Dv
                E += float(np.sum(c * (c + d) / D))
    return E / 36.0
