"""ORACLE (test infrastructure only): CPU restatement of Fermi.jl's RCCSD.

This module is the reference the GB300 coupled-cluster path is tested against.  Only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
may import it; the product path never calls into ``oracle/``.

It restates, term by term and in FP64 numpy, the closed-shell CCSD of
Fermi.jl v0.5.0:

* ``cc_update_energy``      src/Methods/CoupledCluster/RCCSD/RCCSDHelper.jl:8-23
* ``cc_update_T1``          RCCSDHelper.jl:57-85
* ``cc_update_T2``          RCCSDHelper.jl:123-192
* ladder, conventional      RCCSDHelper.jl:194-202
* ladder, density fitted    RCCSDHelper.jl:204-220 (the per-``a`` slab loop)
* ``update_amp``            RCCSDHelper.jl:304-349 (RHF orbitals: no off-diagonal Fock)
* MP2 guess + denominators  src/Methods/CoupledCluster/RCCSD/RCCSDa.jl:46-89
* iteration driver          RCCSDa.jl:92-244
* DIIS                      src/Core/DIIS.jl:21-96
* DF four-index blocks      src/Core/Integrals/ROIntegrals/DFERI.jl:71-196

Each ``@tensor`` statement of the reference becomes one ``einsum`` whose
subscripts are the reference's index strings; the trailing comment gives the
reference line.  Arrays use the reference's logical index order
(``T2[i,j,a,b]``, ``OVOV[i,a,j,b] = (ia|jb)``, ``Bvv[Q,a,b]``).

Parity status: Fermi.jl cannot run here (no Julia, no libcint, no basis
files), so no reference output pins this restatement directly.  It is pinned
by independent known-answer checks in the test suite (a separately written
spin-orbital CCSD and (T) on the same integrals, the three (T) algorithms
agreeing, DF ladder == conventional ladder, size consistency).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _e(subs: str, *ops):
    return np.einsum(subs, *ops, optimize=True)


# ----------------------------------------------------------------- integrals
def df_blocks(Boo, Bov, Bvv, with_vvvv: bool = False) -> dict:
    """MO integral blocks from the DF factors (DFERI.jl:71-196).

    ``VVVV`` is only built on request: the reference builds it lazily but never
    reads it in DF mode (RCCSDHelper.jl:60 destructures it; the DF ladder at
    :204-220 uses BVV)."""
    out = dict(
        OOOO=_e("Qij,Qkl->ijkl", Boo, Boo),     # DFERI.jl:90
        OOOV=_e("Qij,Qka->ijka", Boo, Bov),     # DFERI.jl:116
        OOVV=_e("Qij,Qab->ijab", Boo, Bvv),     # DFERI.jl:141
        OVOV=_e("Qia,Qjb->iajb", Bov, Bov),     # DFERI.jl:158
        OVVV=_e("Qia,Qbc->iabc", Bov, Bvv),     # DFERI.jl:182
    )
    if with_vvvv:
        out["VVVV"] = _e("Qab,Qcd->abcd", Bvv, Bvv)  # DFERI.jl:194
    return out


# -------------------------------------------------------------------- energy
def cc_update_energy(T1, T2, OVOV) -> float:
    """RCCSDHelper.jl:8-23."""
    B = 2.0 * _e("klcd->lckd", T2)                       # :17
    B -= _e("lc,kd->lckd", T1, T1)                        # :18
    B -= _e("lkcd->lckd", T2)                             # :19
    E = _e("lckd,kcld->", B, OVOV)                        # :20
    E += 2.0 * _e("lc,kd,lckd->", T1, T1, OVOV)           # :21
    return float(E)


# ------------------------------------------------------------------------ T1
def cc_update_T1(T1, T2, I) -> np.ndarray:
    """D_ia * T1_ia before the denominator (RCCSDHelper.jl:57-85)."""
    OOOV, OOVV, OVOV, OVVV = I["OOOV"], I["OOVV"], I["OVOV"], I["OVVV"]
    t = -1.0 * _e("kc,ikca->ia", T1, OOVV)                       # :64
    t += 2 * _e("kc,kcia->ia", T1, OVOV)                          # :65
    t += -1.0 * _e("kicd,kdac->ia", T2, OVVV)                     # :66
    t += 2 * _e("ikcd,kdac->ia", T2, OVVV)                        # :67
    t += -2 * _e("klac,kilc->ia", T2, OOOV)                       # :68
    t += 1.0 * _e("lkac,kilc->ia", T2, OOOV)                      # :69
    t += -2 * _e("kc,la,likc->ia", T1, T1, OOOV)                  # :70
    t += -1.0 * _e("kc,id,kdac->ia", T1, T1, OVVV)                # :71
    t += 2 * _e("kc,id,kcad->ia", T1, T1, OVVV)                   # :72
    t += 1.0 * _e("kc,la,kilc->ia", T1, T1, OOOV)                 # :73
    t += -2 * _e("kc,ilad,lckd->ia", T1, T2, OVOV)                # :74
    t += -2 * _e("kc,liad,kcld->ia", T1, T2, OVOV)                # :75
    t += 1.0 * _e("kc,liad,lckd->ia", T1, T2, OVOV)               # :76
    t += -2 * _e("ic,lkad,lckd->ia", T1, T2, OVOV)                # :77
    t += 1.0 * _e("ic,lkad,kcld->ia", T1, T2, OVOV)               # :78
    t += -2 * _e("la,ikdc,kcld->ia", T1, T2, OVOV)                # :79
    t += 1.0 * _e("la,ikcd,kcld->ia", T1, T2, OVOV)               # :80
    t += 1.0 * _e("kc,id,la,lckd->ia", T1, T1, T1, OVOV)          # :81
    t += -2 * _e("kc,id,la,kcld->ia", T1, T1, T1, OVOV)           # :82
    t += 4 * _e("kc,ilad,kcld->ia", T1, T2, OVOV)                 # :83
    return t


# ------------------------------------------------------------------------ T2
def ladder_conv(T1, T2, VVVV) -> np.ndarray:
    """RCCSDHelper.jl:194-202."""
    tau = T2 + _e("ia,jb->ijab", T1, T1)                          # :199
    return _e("ijcd,cadb->ijab", tau, VVVV)                       # :200


def ladder_df(T1, T2, Bvv) -> np.ndarray:
    """RCCSDHelper.jl:204-220: one v^3 slab (cd|ab) per virtual ``a``."""
    tau = T2 + _e("ia,jb->ijab", T1, T1)                          # :208
    o, v = T1.shape
    out = np.zeros((o, o, v, v))
    tau2 = tau.reshape(o * o, v * v)
    for a in range(v):                                            # :214
        Ba = Bvv[:, :, a]                                         # :215 Ba[Q,c]
        cdb = _e("Qc,Qdb->cdb", Ba, Bvv)                          # :216
        out[:, :, a, :] += (tau2 @ cdb.reshape(v * v, v)).reshape(o, o, v)   # :217-218
    return out


def cc_update_T2(T1, T2, I, ladder) -> np.ndarray:
    """D_ijab * T2_ijab before the denominator (RCCSDHelper.jl:123-192).

    ``ladder`` is the already computed (VV|VV) contribution (line :129)."""
    OOOO, OOOV, OOVV, OVOV, OVVV = I["OOOO"], I["OOOV"], I["OOVV"], I["OVOV"], I["OVVV"]
    t = ladder.copy()
    t += 1.0 * _e("iajb->ijab", OVOV)                                        # :134
    t += 1.0 * _e("ka,lb,ikjl->ijab", T1, T1, OOOO)                          # :135
    t += 1.0 * _e("klab,ikjl->ijab", T2, OOOO)                               # :136
    t += -1.0 * _e("ic,jd,ka,kcbd->ijab", T1, T1, T1, OVVV)                  # :137
    t += -1.0 * _e("ic,jd,kb,kdac->ijab", T1, T1, T1, OVVV)                  # :138
    t += 1.0 * _e("ic,ka,lb,ljkc->ijab", T1, T1, T1, OOOV)                   # :139
    t += 1.0 * _e("jc,ka,lb,kilc->ijab", T1, T1, T1, OOOV)                   # :140
    t += 1.0 * _e("klac,ijdb,kcld->ijab", T2, T2, OVOV)                      # :141
    t += -2 * _e("ikac,ljbd,kcld->ijab", T2, T2, OVOV)                       # :142
    t += -2 * _e("lkac,ijdb,kcld->ijab", T2, T2, OVOV)                       # :143
    t += 1.0 * _e("kiac,ljdb,lckd->ijab", T2, T2, OVOV)                      # :144
    t += 1.0 * _e("ikac,ljbd,lckd->ijab", T2, T2, OVOV)                      # :145
    t += -2 * _e("ikac,jlbd,lckd->ijab", T2, T2, OVOV)                       # :146
    t += 1.0 * _e("kiac,ljbd,kcld->ijab", T2, T2, OVOV)                      # :147
    t += -2 * _e("kiac,jlbd,kcld->ijab", T2, T2, OVOV)                       # :148
    t += 1.0 * _e("ijac,lkbd,kcld->ijab", T2, T2, OVOV)                      # :149
    t += -2 * _e("ijac,klbd,kcld->ijab", T2, T2, OVOV)                       # :150
    t += 1.0 * _e("kjac,ildb,lckd->ijab", T2, T2, OVOV)                      # :151
    t += 4 * _e("ikac,jlbd,kcld->ijab", T2, T2, OVOV)                        # :152
    t += 1.0 * _e("ijdc,lkab,kcld->ijab", T2, T2, OVOV)                      # :153
    t += 1.0 * _e("ic,jd,ka,lb,kcld->ijab", T1, T1, T1, T1, OVOV)            # :154
    t += 1.0 * _e("ic,jd,lkab,lckd->ijab", T1, T1, T2, OVOV)                 # :155
    t += 1.0 * _e("ka,lb,ijdc,lckd->ijab", T1, T1, T2, OVOV)                 # :156
    P = 1.0 * _e("jc,iacb->ijab", T1, OVVV)                                  # :157
    P += -1.0 * _e("kb,jkia->ijab", T1, OOOV)                                # :158
    P += -1.0 * _e("kiac,kcjb->ijab", T2, OVOV)                              # :159
    P += -1.0 * _e("ic,ka,kcjb->ijab", T1, T1, OVOV)                         # :160
    P += -1.0 * _e("ic,kb,jkca->ijab", T1, T1, OOVV)                         # :161
    P += 2 * _e("ikac,kcjb->ijab", T2, OVOV)                                 # :162
    P += -1.0 * _e("ikac,jkcb->ijab", T2, OOVV)                              # :163
    P += -1.0 * _e("kjac,ikcb->ijab", T2, OOVV)                              # :164
    P += -2 * _e("lb,ikac,ljkc->ijab", T1, T2, OOOV)                         # :165
    P += 1.0 * _e("lb,kiac,ljkc->ijab", T1, T2, OOOV)                        # :166
    P += -1.0 * _e("jc,ikdb,kcad->ijab", T1, T2, OVVV)                       # :167
    P += -1.0 * _e("jc,kiad,kdbc->ijab", T1, T2, OVVV)                       # :168
    P += -1.0 * _e("jc,ikad,kcbd->ijab", T1, T2, OVVV)                       # :169
    P += 1.0 * _e("jc,lkab,likc->ijab", T1, T2, OOOV)                        # :170
    P += 1.0 * _e("lb,ikac,kjlc->ijab", T1, T2, OOOV)                        # :171
    P += -1.0 * _e("ka,ijdc,kdbc->ijab", T1, T2, OVVV)                       # :172
    P += 1.0 * _e("ka,ilcb,ljkc->ijab", T1, T2, OOOV)                        # :173
    P += 2 * _e("jc,ikad,kdbc->ijab", T1, T2, OVVV)                          # :174
    P += -1.0 * _e("kc,ijad,kdbc->ijab", T1, T2, OVVV)                       # :175
    P += 2 * _e("kc,ijad,kcbd->ijab", T1, T2, OVVV)                          # :176
    P += 1.0 * _e("kc,ilab,kjlc->ijab", T1, T2, OOOV)                        # :177
    P += -2 * _e("kc,ilab,ljkc->ijab", T1, T2, OOOV)                         # :178
    P += 1.0 * _e("jkcd,ilab,kcld->ijab", T2, T2, OVOV)                      # :179
    P += -2 * _e("kc,jd,ilab,kcld->ijab", T1, T1, T2, OVOV)                  # :180
    P += 1.0 * _e("kc,jd,ilab,lckd->ijab", T1, T1, T2, OVOV)                 # :181
    P += -2 * _e("kc,la,ijdb,kcld->ijab", T1, T1, T2, OVOV)                  # :182
    P += 1.0 * _e("kc,la,ijdb,lckd->ijab", T1, T1, T2, OVOV)                 # :183
    P += 1.0 * _e("ic,ka,ljbd,kcld->ijab", T1, T1, T2, OVOV)                 # :184
    P += -2 * _e("ic,ka,jlbd,kcld->ijab", T1, T1, T2, OVOV)                  # :185
    P += 1.0 * _e("ic,ka,ljdb,lckd->ijab", T1, T1, T2, OVOV)                 # :186
    P += 1.0 * _e("ic,lb,kjad,kcld->ijab", T1, T1, T2, OVOV)                 # :187
    P += -2 * _e("ikdc,ljab,kcld->ijab", T2, T2, OVOV)                       # :188
    t += P + P.transpose(1, 0, 3, 2)                                         # :190
    return t


# ------------------------------------------------------------- denominators
def denominators(eps_o, eps_v):
    """D1[i,a] = e_i - e_a and D2[i,j,a,b] = e_i + e_j - e_a - e_b
    (RCCSDa.jl:60-83, RCCSDHelper.jl:322-345)."""
    d1 = eps_o[:, None] - eps_v[None, :]
    d2 = eps_o[:, None, None, None] + eps_o[None, :, None, None] - eps_v[None, None, :, None] - eps_v[None, None, None, :]
    return d1, d2


def update_amp(T1, T2, I, D1, D2, ladder_fn):
    """RCCSDHelper.jl:304-349 for RHF orbitals."""
    newT1 = cc_update_T1(T1, T2, I)
    newT2 = cc_update_T2(T1, T2, I, ladder_fn(T1, T2))
    return newT1 / D1, newT2 / D2


def mp2_guess(I, D1, D2):
    """RCCSDa.jl:53-89: T1 = Fia / D1 (Fia = 0 for RHF orbitals, Fock.jl:95),
    T2 = permutedims(OVOV, (1,3,2,4)) / D2."""
    T1 = np.zeros_like(D1)
    T2 = I["OVOV"].transpose(0, 2, 1, 3) / D2
    return T1, T2


# ---------------------------------------------------------------------- DIIS
class DIISManager:
    """DIIS.jl:21-96.  Vectors kept in FP64, error vectors in ``err_dtype``
    (float32 = Fermi's default ``diis_prec = "single"``, RCCSDa.jl:122-125)."""

    def __init__(self, size: int = 3, err_dtype=np.float32):
        self.vecs, self.errs, self.max_vec, self.err_dtype = [], [], size, err_dtype

    def __len__(self):
        return len(self.vecs)

    def push(self, V, E):                                  # DIIS.jl:38-50
        if len(self) + 1 > self.max_vec:
            norms = [np.linalg.norm(e.astype(np.float64).ravel()) for e in self.errs]
            idx = int(np.argmax(norms))
            del self.vecs[idx]
            del self.errs[idx]
        self.vecs.append(np.array(V, dtype=np.float64, copy=True))
        self.errs.append(np.array(E, dtype=self.err_dtype, copy=True))

    def extrapolate(self, add_res: bool = False):          # DIIS.jl:59-96
        if len(self) < 2:
            raise IndexError("DIIS cannot extrapolate from one vector")
        N = len(self) + 1
        B = np.ones((N, N))
        B[-1, -1] = 0.0
        for n1, e1 in enumerate(self.errs):
            for n2, e2 in enumerate(self.errs):
                B[n1, n2] = float(np.sum(e1 * e2))          # in the error precision
        resid = np.zeros(N)
        resid[-1] = 1.0
        ci = np.linalg.solve(B, resid)
        out = sum(c * v for c, v in zip(ci[:-1], self.vecs))
        if add_res:
            out = out + sum(c * e.astype(np.float64) for c, e in zip(ci[:-1], self.errs))
        return out


# -------------------------------------------------------------------- driver
@dataclass
class CCOptions:
    """Fermi's CC options with their defaults (src/Core/Options.jl:40-104)."""
    cc_max_iter: int = 50
    cc_e_conv: float = 1e-10
    cc_max_rms: float = 1e-10
    cc_diis: bool = True
    cc_ndiis: int = 3
    cc_diis_relax: int = 3
    diis_start: int = 3
    diis_prec: str = "single"
    cc_damp_ratio: float = 0.0


@dataclass
class RCCSDResult:
    """Fields of ``struct RCCSD`` (src/Methods/CoupledCluster/RCCSD/RCCSD.jl:61-69)."""
    guessenergy: float
    correlation: float
    energy: float
    T1: np.ndarray
    T2: np.ndarray
    e_conv: float
    t_conv: float
    iterations: list = field(default_factory=list)
    converged: bool = False


def rccsd(I: dict, eps_o, eps_v, e_ref: float, opts: CCOptions | None = None,
          T1guess=None, T2guess=None, Bvv=None, ccd: bool = False) -> RCCSDResult:
    """RCCSDa.jl:92-244.  With ``Bvv`` given the DF ladder is used, otherwise
    ``I["VVVV"]`` (conventional).  ``ccd`` holds T1 at zero (the CCD limit,
    a known-answer check against a spin-orbital CCD; not a Fermi option)."""
    opts = opts or CCOptions()
    D1, D2 = denominators(eps_o, eps_v)
    if T1guess is None or T2guess is None:
        T1guess, T2guess = mp2_guess(I, D1, D2)
    if Bvv is not None:
        ladder = lambda t1, t2: ladder_df(t1, t2, Bvv)
    else:
        ladder = lambda t1, t2: ladder_conv(t1, t2, I["VVVV"])
    err_dtype = {"double": np.float64, "single": np.float32}.get(opts.diis_prec, np.float16)
    newT1, newT2 = np.array(T1guess, dtype=np.float64), np.array(T2guess, dtype=np.float64)
    if ccd:
        newT1[:] = 0.0
    Ecc = cc_update_energy(newT1, newT2, I["OVOV"])                   # :168
    Eguess = Ecc + e_ref
    dE, rms, ite = 1.0, 1.0, 1
    dm1 = DIISManager(opts.cc_ndiis, err_dtype) if opts.cc_diis else None
    dm2 = DIISManager(opts.cc_ndiis, err_dtype) if opts.cc_diis else None
    log = []
    r1 = r2 = 1.0
    while abs(dE) > opts.cc_e_conv or rms > opts.cc_max_rms:          # :178
        if ite > opts.cc_max_iter:                                    # :179-182
            break
        T1, T2 = newT1.copy(), newT2.copy()                           # :185-186
        oldE = Ecc
        newT1, newT2 = update_amp(T1, T2, I, D1, D2, ladder)          # :190
        if ccd:
            newT1 = np.zeros_like(newT1)
        r1 = float(np.sqrt(np.sum((newT1 - T1) ** 2) / T1.size))      # :193
        r2 = float(np.sqrt(np.sum((newT2 - T2) ** 2) / T2.size))      # :194
        diis = False
        if opts.cc_diis:
            if not ccd:                                               # (T1 = 0: no T1 subspace)
                dm1.push(newT1, newT1 - T1)                           # :200-201
            dm2.push(newT2, newT2 - T2)
            if ite >= opts.diis_start and ite % opts.cc_diis_relax == 0:   # :204
                newT2 = dm2.extrapolate(add_res=True)                 # :206
                if not ccd:
                    newT1 = dm1.extrapolate(add_res=True)             # :207
                diis = True
        dp = opts.cc_damp_ratio
        if dp > 0:                                                    # :213-216
            newT1 = (1 - dp) * newT1 + dp * T1
            newT2 = (1 - dp) * newT2 + dp * T2
        Ecc = cc_update_energy(newT1, newT2, I["OVOV"])               # :218
        rms = max(r1, r2)                                             # :220
        dE = Ecc - oldE                                               # :221
        log.append(dict(ite=ite, energy=Ecc, dE=dE, rms=rms, diis=diis))
        ite += 1
    conv = abs(dE) < opts.cc_e_conv and rms < opts.cc_max_rms         # :231
    return RCCSDResult(Eguess, Ecc, Ecc + e_ref, newT1, newT2, dE, rms, log, conv)
