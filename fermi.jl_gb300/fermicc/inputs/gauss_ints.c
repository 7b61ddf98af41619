/*
 * Gaussian-basis molecular integrals for the stand-in input pipeline.
 *
 * The coupled-cluster path consumes density-fitted three-index factors and
 * orbital energies that, in Fermi.jl, come from libcint through
 * GaussianBasis.jl (src/Core/Integrals/AtomicIntegrals.jl:16-51).  Neither
 * libcint nor the basis-set files are available here, so this file computes
 * the same kinds of integrals from first principles:
 *
 *   overlap S, kinetic T, nuclear attraction V       (one-electron)
 *   (P|Q)                                             (two-centre Coulomb)
 *   (mn|P)                                            (three-centre Coulomb)
 *   (mn|ls)                                           (four-centre Coulomb)
 *
 * Method: McMurchie & Davidson, J. Comput. Phys. 26, 218 (1978): Hermite
 * expansion coefficients E^{ij}_t of Gaussian overlap distributions and the
 * Hermite Coulomb integrals R_{tuv} built by the standard recursion from the
 * Boys function.  Cartesian shells are combined into real solid harmonics
 * with the closed-form coefficients of Helgaker, Jorgensen & Olsen,
 * "Molecular Electronic-Structure Theory" (Wiley 2000), eq. 6.4.47-6.4.50.
 *
 * Shell description (flat arrays, shared by every entry point):
 *   nsh             number of shells
 *   xyz[3*s]        centre of shell s (bohr)
 *   lq[s]           angular momentum (0..4)
 *   np[s], po[s]    number of primitives and offset into ex/co
 *   ex[], co[]      primitive exponents and contraction coefficients (the
 *                   caller folds primitive normalisation into co)
 * Functions are spherical; shell s contributes 2l+1 functions in the order
 * m = -l..l.  Outputs are row-major (C order).  Contracted functions are NOT
 * renormalised here; the caller rescales with the diagonal of S or (P|P).
 *
 * Every entry point returns 0 on success, -1 on a bad argument.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define LMAX 4
#define LTOT (4 * LMAX + 1)

/* ------------------------------------------------------------------ Boys */
/* F_n(T) for n = 0..nmax.  Small T: the convergent series
 *   F_n(T) = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
 * evaluated at n = nmax, then downward recursion
 *   F_{n-1} = (2T F_n + exp(-T)) / (2n-1).
 * Large T: F_0 = sqrt(pi/T) erf(sqrt T) / 2 and upward recursion
 *   F_{n+1} = ((2n+1) F_n - exp(-T)) / (2T), stable for T > nmax. */
static void boys(int nmax, double T, double *F) {
    if (T < 1e-14) {
        for (int n = 0; n <= nmax; ++n) F[n] = 1.0 / (2 * n + 1);
        return;
    }
    double eT = exp(-T);
    if (T < 18.0) {
        double term = 1.0 / (2 * nmax + 1), sum = term;
        for (int k = 1; k < 400; ++k) {
            term *= 2.0 * T / (2 * nmax + 2 * k + 1);
            sum += term;
            if (term < 1e-17 * sum) break;
        }
        F[nmax] = eT * sum;
        for (int n = nmax; n > 0; --n) F[n - 1] = (2.0 * T * F[n] + eT) / (2 * n - 1);
    } else {
        double st = sqrt(T);
        F[0] = 0.5 * sqrt(M_PI) / st * erf(st);
        for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - eT) / (2.0 * T);
    }
}

/* ------------------------------------------- Cartesian / spherical tables */
static int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int nsph(int l) { return 2 * l + 1; }

/* Cartesian component c of shell l: exponents (ax, ay, az) in the order
 * ax = l..0, ay = l-ax..0. */
static void cart_exps(int l, int c, int *ax, int *ay, int *az) {
    int idx = 0;
    *ax = l; *ay = 0; *az = 0;
    for (int a = l; a >= 0; --a)
        for (int b = l - a; b >= 0; --b) {
            if (idx == c) { *ax = a; *ay = b; *az = l - a - b; return; }
            ++idx;
        }
}
static int cart_index(int l, int ax, int ay) {
    /* inverse of cart_exps */
    int idx = 0;
    for (int a = l; a > ax; --a) idx += l - a + 1;
    return idx + (l - ax - ay);
}

static double fact(int n) { double r = 1; for (int i = 2; i <= n; ++i) r *= i; return r; }
static double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    return fact(n) / (fact(k) * fact(n - k));
}

/* sph[l][m+l][c]: real solid harmonic S_lm as a combination of the
 * Cartesian monomials x^ax y^ay z^az of shell l (HJO eq. 6.4.47-6.4.50). */
static double SPH[LMAX + 1][2 * LMAX + 1][(LMAX + 1) * (LMAX + 2) / 2];
static int sph_ready = 0;

static void build_sph(void) {
    memset(SPH, 0, sizeof(SPH));
    for (int l = 0; l <= LMAX; ++l) {
        for (int m = -l; m <= l; ++m) {
            int am = abs(m);
            double vm = (m < 0) ? 0.5 : 0.0;
            double Nlm = 1.0 / (pow(2.0, am) * fact(l)) *
                         sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0));
            for (int t = 0; t <= (l - am) / 2; ++t)
                for (int u = 0; u <= t; ++u) {
                    /* v runs over vm, vm+1, ..., floor(am/2 - vm) + vm */
                    int vcount = (int)floor(am / 2.0 - vm) + 1;
                    for (int vi = 0; vi < vcount; ++vi) {
                        double v = vm + vi;
                        double sgn = (((int)llround(t + v - vm)) % 2 == 0) ? 1.0 : -1.0;
                        double C = sgn * pow(0.25, t) * binom(l, t) * binom(l - t, am + t) *
                                   binom(t, u) * binom(am, (int)llround(2 * v));
                        int px = 2 * t + am - (int)llround(2 * (u + v));
                        int py = (int)llround(2 * (u + v));
                        int pz = l - 2 * t - am;
                        if (px < 0 || py < 0 || pz < 0) continue;
                        SPH[l][m + l][cart_index(l, px, py)] += Nlm * C;
                    }
                }
        }
    }
    sph_ready = 1;
}

/* ------------------------------------------------- Hermite E coefficients */
/* E[i][j][t] for one Cartesian direction, i <= la, j <= lb, t <= i + j.
 * Stored flat with strides (lb+1)*(LTOT) and LTOT. */
#define EIDX(i, j, t) (((i) * (LMAX + 1) + (j)) * (2 * LMAX + 1) + (t))
#define ESIZE ((LMAX + 1) * (LMAX + 1) * (2 * LMAX + 1))

static void hermite_E(int la, int lb, double a, double b, double XAB, double *E) {
    double p = a + b;
    double XPA, XPB, K;
    if (p == 0.0) { XPA = 0; XPB = 0; K = 1.0; }
    else {
        double mu = a * b / p;
        XPA = -b / p * XAB;   /* P - A with XAB = A - B */
        XPB = a / p * XAB;    /* P - B */
        K = exp(-mu * XAB * XAB);
    }
    double ip2 = (p == 0.0) ? 0.0 : 0.5 / p;
    memset(E, 0, sizeof(double) * ESIZE);
    E[EIDX(0, 0, 0)] = K;
    /* build up i with j = 0 */
    for (int i = 0; i < la; ++i)
        for (int t = 0; t <= i + 1; ++t) {
            double v = 0.0;
            if (t > 0) v += ip2 * E[EIDX(i, 0, t - 1)];
            if (t <= i) v += XPA * E[EIDX(i, 0, t)];
            if (t + 1 <= i) v += (t + 1) * E[EIDX(i, 0, t + 1)];
            E[EIDX(i + 1, 0, t)] = v;
        }
    /* build up j for every i */
    for (int j = 0; j < lb; ++j)
        for (int i = 0; i <= la; ++i)
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = 0.0;
                if (t > 0) v += ip2 * E[EIDX(i, j, t - 1)];
                if (t <= i + j) v += XPB * E[EIDX(i, j, t)];
                if (t + 1 <= i + j) v += (t + 1) * E[EIDX(i, j, t + 1)];
                E[EIDX(i, j + 1, t)] = v;
            }
}

/* -------------------------------------------- Hermite Coulomb R_{tuv} */
/* R[t][u][v] (n = 0) for t+u+v <= L at exponent alpha and vector PC.
 * Work array Rn holds (L+1)^4 values. */
#define RIDX(n, t, u, v, L1) ((((n) * (L1) + (t)) * (L1) + (u)) * (L1) + (v))

static void hermite_R(int L, double alpha, double X, double Y, double Z, double *Rn) {
    int L1 = L + 1;
    double F[LTOT + 2];
    double T = alpha * (X * X + Y * Y + Z * Z);
    boys(L, T, F);
    for (int n = L; n >= 0; --n) {
        int maxo = L - n;
        for (int t = 0; t <= maxo; ++t)
            for (int u = 0; u + t <= maxo; ++u)
                for (int v = 0; v + u + t <= maxo; ++v) {
                    double val;
                    if (t > 0) {
                        val = X * Rn[RIDX(n + 1, t - 1, u, v, L1)];
                        if (t > 1) val += (t - 1) * Rn[RIDX(n + 1, t - 2, u, v, L1)];
                    } else if (u > 0) {
                        val = Y * Rn[RIDX(n + 1, t, u - 1, v, L1)];
                        if (u > 1) val += (u - 1) * Rn[RIDX(n + 1, t, u - 2, v, L1)];
                    } else if (v > 0) {
                        val = Z * Rn[RIDX(n + 1, t, u, v - 1, L1)];
                        if (v > 1) val += (v - 1) * Rn[RIDX(n + 1, t, u, v - 2, L1)];
                    } else {
                        val = pow(-2.0 * alpha, n) * F[n];
                    }
                    Rn[RIDX(n, t, u, v, L1)] = val;
                }
    }
}

/* ------------------------------------------------------ shell bookkeeping */
typedef struct {
    int nsh;
    const double *xyz;
    const int *lq, *np, *po;
    const double *ex, *co;
    int *off;     /* spherical offset of each shell */
    int nbf;
} basis_t;

static int basis_init(basis_t *B, int nsh, const double *xyz, const int *lq, const int *np,
                      const int *po, const double *ex, const double *co) {
    if (nsh < 0 || (nsh > 0 && (!xyz || !lq || !np || !po || !ex || !co))) return -1;
    B->nsh = nsh; B->xyz = xyz; B->lq = lq; B->np = np; B->po = po; B->ex = ex; B->co = co;
    B->off = (int *)malloc(sizeof(int) * (nsh + 1));
    if (!B->off) return -1;
    int n = 0;
    for (int s = 0; s < nsh; ++s) {
        if (lq[s] < 0 || lq[s] > LMAX || np[s] <= 0) { free(B->off); return -1; }
        B->off[s] = n;
        n += nsh > 0 ? nsph(lq[s]) : 0;
    }
    B->off[nsh] = n;
    B->nbf = n;
    if (!sph_ready) build_sph();
    return 0;
}

/* The "null" shell: an s function with exponent 0 and coefficient 1, used to
 * turn the four-centre routine into the three- and two-centre ones. */
static const double NULL_XYZ[3] = {0, 0, 0};
static const double NULL_EX[1] = {0.0};
static const double NULL_CO[1] = {1.0};

typedef struct { const double *c; int l, np; const double *ex, *co; } sh_t;

static sh_t get_shell(const basis_t *B, int s) {
    sh_t r;
    if (s < 0) { r.c = NULL_XYZ; r.l = 0; r.np = 1; r.ex = NULL_EX; r.co = NULL_CO; return r; }
    r.c = B->xyz + 3 * s; r.l = B->lq[s]; r.np = B->np[s];
    r.ex = B->ex + B->po[s]; r.co = B->co + B->po[s];
    return r;
}

/* Cartesian (ab|cd) for contracted shells, out[((a*nb+b)*nc+c)*nd+d]. */
static void eri_cart(const sh_t *A, const sh_t *Bs, const sh_t *C, const sh_t *D, double *out) {
    int la = A->l, lb = Bs->l, lc = C->l, ld = D->l;
    int na = ncart(la), nb = ncart(lb), nc = ncart(lc), nd = ncart(ld);
    int L = la + lb + lc + ld, L1 = L + 1;
    double Eab[3][ESIZE], Ecd[3][ESIZE];
    double *Rn = (double *)malloc(sizeof(double) * L1 * L1 * L1 * L1);
    memset(out, 0, sizeof(double) * na * nb * nc * nd);
    double AB[3], CD[3];
    for (int k = 0; k < 3; ++k) { AB[k] = A->c[k] - Bs->c[k]; CD[k] = C->c[k] - D->c[k]; }
    /* Hermite-basis intermediate: H[(tuv)][c][d] per primitive quartet */
    int Lab = la + lb, Lcd = lc + ld;
    int nH1 = (Lab + 1) * (Lab + 1) * (Lab + 1);
    double *H = (double *)malloc(sizeof(double) * nH1 * nc * nd);
    for (int pa = 0; pa < A->np; ++pa)
        for (int pb = 0; pb < Bs->np; ++pb) {
            double a = A->ex[pa], b = Bs->ex[pb], p = a + b;
            double cab = A->co[pa] * Bs->co[pb];
            double P[3];
            for (int k = 0; k < 3; ++k)
                P[k] = (p == 0.0) ? A->c[k] : (a * A->c[k] + b * Bs->c[k]) / p;
            for (int k = 0; k < 3; ++k) hermite_E(la, lb, a, b, AB[k], Eab[k]);
            for (int pc = 0; pc < C->np; ++pc)
                for (int pd = 0; pd < D->np; ++pd) {
                    double c = C->ex[pc], d = D->ex[pd], q = c + d;
                    double ccd = C->co[pc] * D->co[pd];
                    double Q[3];
                    for (int k = 0; k < 3; ++k)
                        Q[k] = (q == 0.0) ? C->c[k] : (c * C->c[k] + d * D->c[k]) / q;
                    for (int k = 0; k < 3; ++k) hermite_E(lc, ld, c, d, CD[k], Ecd[k]);
                    double alpha = p * q / (p + q);
                    hermite_R(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], Rn);
                    double pref = 2.0 * pow(M_PI, 2.5) / (p * q * sqrt(p + q)) * cab * ccd;
                    /* H[tuv][c][d] = sum_{tau,nu,phi} (-1)^{tau+nu+phi} E^cd R_{t+tau,...} */
                    memset(H, 0, sizeof(double) * nH1 * nc * nd);
                    for (int ic = 0; ic < nc; ++ic) {
                        int cx, cy, cz; cart_exps(lc, ic, &cx, &cy, &cz);
                        for (int id = 0; id < nd; ++id) {
                            int dx, dy, dz; cart_exps(ld, id, &dx, &dy, &dz);
                            for (int tau = 0; tau <= cx + dx; ++tau) {
                                double ex_ = Ecd[0][EIDX(cx, dx, tau)];
                                if (ex_ == 0.0) continue;
                                for (int nu = 0; nu <= cy + dy; ++nu) {
                                    double ey_ = Ecd[1][EIDX(cy, dy, nu)];
                                    if (ey_ == 0.0) continue;
                                    for (int phi = 0; phi <= cz + dz; ++phi) {
                                        double ez_ = Ecd[2][EIDX(cz, dz, phi)];
                                        if (ez_ == 0.0) continue;
                                        double w = ex_ * ey_ * ez_ * (((tau + nu + phi) & 1) ? -1.0 : 1.0);
                                        for (int t = 0; t <= Lab; ++t)
                                            for (int u = 0; u + t <= Lab; ++u)
                                                for (int v = 0; v + u + t <= Lab; ++v)
                                                    H[((t * (Lab + 1) + u) * (Lab + 1) + v) * nc * nd + ic * nd + id] +=
                                                        w * Rn[RIDX(0, t + tau, u + nu, v + phi, L1)];
                                    }
                                }
                            }
                        }
                    }
                    (void)Lcd;
                    for (int ia = 0; ia < na; ++ia) {
                        int ax, ay, az; cart_exps(la, ia, &ax, &ay, &az);
                        for (int ib = 0; ib < nb; ++ib) {
                            int bx, by, bz; cart_exps(lb, ib, &bx, &by, &bz);
                            double *o = out + (ia * nb + ib) * nc * nd;
                            for (int t = 0; t <= ax + bx; ++t) {
                                double ex_ = Eab[0][EIDX(ax, bx, t)];
                                if (ex_ == 0.0) continue;
                                for (int u = 0; u <= ay + by; ++u) {
                                    double ey_ = Eab[1][EIDX(ay, by, u)];
                                    if (ey_ == 0.0) continue;
                                    for (int v = 0; v <= az + bz; ++v) {
                                        double ez_ = Eab[2][EIDX(az, bz, v)];
                                        if (ez_ == 0.0) continue;
                                        double w = pref * ex_ * ey_ * ez_;
                                        const double *h = H + ((t * (Lab + 1) + u) * (Lab + 1) + v) * nc * nd;
                                        for (int k = 0; k < nc * nd; ++k) o[k] += w * h[k];
                                    }
                                }
                            }
                        }
                    }
                }
        }
    free(H);
    free(Rn);
}

/* Transform a Cartesian block with dims (na, nb, nc, nd) to spherical
 * (2la+1, ...), one index at a time. */
static void cart_to_sph4(const int l[4], const double *cart, double *sph) {
    int nC[4], nS[4];
    for (int k = 0; k < 4; ++k) { nC[k] = ncart(l[k]); nS[k] = nsph(l[k]); }
    int maxsz = 1;
    for (int k = 0; k < 4; ++k) maxsz *= nC[k];
    double *buf0 = (double *)malloc(sizeof(double) * maxsz);
    double *buf1 = (double *)malloc(sizeof(double) * maxsz);
    memcpy(buf0, cart, sizeof(double) * maxsz);
    int dims[4] = {nC[0], nC[1], nC[2], nC[3]};
    for (int k = 0; k < 4; ++k) {
        /* transform index k: dims[k] nC -> nS */
        int pre = 1, post = 1;
        for (int q = 0; q < k; ++q) pre *= dims[q];
        for (int q = k + 1; q < 4; ++q) post *= dims[q];
        for (int a = 0; a < pre; ++a)
            for (int m = 0; m < nS[k]; ++m)
                for (int b = 0; b < post; ++b) {
                    double s = 0.0;
                    for (int c = 0; c < nC[k]; ++c) s += SPH[l[k]][m][c] * buf0[(a * nC[k] + c) * post + b];
                    buf1[(a * nS[k] + m) * post + b] = s;
                }
        dims[k] = nS[k];
        double *t = buf0; buf0 = buf1; buf1 = t;
    }
    int tot = nS[0] * nS[1] * nS[2] * nS[3];
    memcpy(sph, buf0, sizeof(double) * tot);
    free(buf0); free(buf1);
}

static void eri_sph(const sh_t *A, const sh_t *Bs, const sh_t *C, const sh_t *D, double *out) {
    int l[4] = {A->l, Bs->l, C->l, D->l};
    int n = ncart(l[0]) * ncart(l[1]) * ncart(l[2]) * ncart(l[3]);
    double *cart = (double *)malloc(sizeof(double) * n);
    eri_cart(A, Bs, C, D, cart);
    cart_to_sph4(l, cart, out);
    free(cart);
}

/* ------------------------------------------------------------- one-body */
/* Overlap, kinetic and nuclear attraction for a Cartesian shell pair. */
static void one_body_cart(const sh_t *A, const sh_t *Bs, int natm, const double *axyz,
                          const double *Z, double *S, double *T, double *V) {
    int la = A->l, lb = Bs->l, na = ncart(la), nb = ncart(lb);
    int L = la + lb, L1 = L + 1;
    double E[3][ESIZE], E2[3][ESIZE];
    double *Rn = (double *)malloc(sizeof(double) * L1 * L1 * L1 * L1);
    memset(S, 0, sizeof(double) * na * nb);
    memset(T, 0, sizeof(double) * na * nb);
    memset(V, 0, sizeof(double) * na * nb);
    double AB[3];
    for (int k = 0; k < 3; ++k) AB[k] = A->c[k] - Bs->c[k];
    for (int pa = 0; pa < A->np; ++pa)
        for (int pb = 0; pb < Bs->np; ++pb) {
            double a = A->ex[pa], b = Bs->ex[pb], p = a + b;
            double cc = A->co[pa] * Bs->co[pb];
            double P[3];
            for (int k = 0; k < 3; ++k) P[k] = (a * A->c[k] + b * Bs->c[k]) / p;
            for (int k = 0; k < 3; ++k) {
                hermite_E(la, lb, a, b, AB[k], E[k]);
                /* for the kinetic operator we need j up to lb+2 */
                hermite_E(la, lb + 2 <= LMAX ? lb + 2 : LMAX, a, b, AB[k], E2[k]);
            }
            double sp = sqrt(M_PI / p);
            for (int ia = 0; ia < na; ++ia) {
                int ai[3]; cart_exps(la, ia, &ai[0], &ai[1], &ai[2]);
                for (int ib = 0; ib < nb; ++ib) {
                    int bi[3]; cart_exps(lb, ib, &bi[0], &bi[1], &bi[2]);
                    double s1[3], t1[3];
                    for (int k = 0; k < 3; ++k) {
                        int i = ai[k], j = bi[k];
                        s1[k] = E2[k][EIDX(i, j, 0)] * sp;
                        double sp2 = E2[k][EIDX(i, j + 2, 0)] * sp;
                        double sm2 = (j >= 2) ? E2[k][EIDX(i, j - 2, 0)] * sp : 0.0;
                        t1[k] = -2.0 * b * b * sp2 + b * (2 * j + 1) * s1[k] - 0.5 * j * (j - 1) * sm2;
                    }
                    S[ia * nb + ib] += cc * s1[0] * s1[1] * s1[2];
                    T[ia * nb + ib] += cc * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
                }
            }
            for (int at = 0; at < natm; ++at) {
                hermite_R(L, p, P[0] - axyz[3 * at], P[1] - axyz[3 * at + 1], P[2] - axyz[3 * at + 2], Rn);
                double pref = -Z[at] * 2.0 * M_PI / p * cc;
                for (int ia = 0; ia < na; ++ia) {
                    int ax, ay, az; cart_exps(la, ia, &ax, &ay, &az);
                    for (int ib = 0; ib < nb; ++ib) {
                        int bx, by, bz; cart_exps(lb, ib, &bx, &by, &bz);
                        double s = 0.0;
                        for (int t = 0; t <= ax + bx; ++t)
                            for (int u = 0; u <= ay + by; ++u)
                                for (int v = 0; v <= az + bz; ++v)
                                    s += E[0][EIDX(ax, bx, t)] * E[1][EIDX(ay, by, u)] * E[2][EIDX(az, bz, v)] *
                                         Rn[RIDX(0, t, u, v, L1)];
                        V[ia * nb + ib] += pref * s;
                    }
                }
            }
        }
    free(Rn);
}

static void cart_to_sph2(int la, int lb, const double *cart, double *sph) {
    int nca = ncart(la), ncb = ncart(lb), nsa = nsph(la), nsb = nsph(lb);
    for (int m = 0; m < nsa; ++m)
        for (int n = 0; n < nsb; ++n) {
            double s = 0.0;
            for (int i = 0; i < nca; ++i) {
                double ci = SPH[la][m][i];
                if (ci == 0.0) continue;
                for (int j = 0; j < ncb; ++j) s += ci * SPH[lb][n][j] * cart[i * ncb + j];
            }
            sph[m * nsb + n] = s;
        }
}

/* ================================================================ C ABI */

int fcci_one_body(int nsh, const double *xyz, const int *lq, const int *np, const int *po,
                  const double *ex, const double *co, int natm, const double *axyz, const double *Z,
                  double *S, double *T, double *V) {
    basis_t B;
    if (basis_init(&B, nsh, xyz, lq, np, po, ex, co)) return -1;
    if (lq) for (int s = 0; s < nsh; ++s) if (lq[s] > LMAX - 2) { free(B.off); return -1; }
    int n = B.nbf;
#pragma omp parallel for schedule(dynamic)
    for (int sa = 0; sa < nsh; ++sa)
        for (int sb = 0; sb <= sa; ++sb) {
            sh_t A = get_shell(&B, sa), Bs = get_shell(&B, sb);
            int nsa = nsph(A.l), nsb = nsph(Bs.l);
            double cS[64], cT[64], cV[64], sS[64], sT[64], sV[64];
            one_body_cart(&A, &Bs, natm, axyz, Z, cS, cT, cV);
            cart_to_sph2(A.l, Bs.l, cS, sS);
            cart_to_sph2(A.l, Bs.l, cT, sT);
            cart_to_sph2(A.l, Bs.l, cV, sV);
            for (int i = 0; i < nsa; ++i)
                for (int j = 0; j < nsb; ++j) {
                    int mu = B.off[sa] + i, nu = B.off[sb] + j;
                    S[mu * n + nu] = S[nu * n + mu] = sS[i * nsb + j];
                    T[mu * n + nu] = T[nu * n + mu] = sT[i * nsb + j];
                    V[mu * n + nu] = V[nu * n + mu] = sV[i * nsb + j];
                }
        }
    free(B.off);
    return 0;
}

/* (P|Q) over the auxiliary basis, out[P*naux+Q]. */
int fcci_eri2c(int nsh, const double *xyz, const int *lq, const int *np, const int *po,
               const double *ex, const double *co, double *out) {
    basis_t B;
    if (basis_init(&B, nsh, xyz, lq, np, po, ex, co)) return -1;
    int n = B.nbf;
#pragma omp parallel for schedule(dynamic)
    for (int sp = 0; sp < nsh; ++sp)
        for (int sq = 0; sq <= sp; ++sq) {
            sh_t P = get_shell(&B, sp), Q = get_shell(&B, sq), N = get_shell(&B, -1);
            int np_ = nsph(P.l), nq = nsph(Q.l);
            double buf[81];
            eri_sph(&P, &N, &Q, &N, buf);
            for (int i = 0; i < np_; ++i)
                for (int j = 0; j < nq; ++j) {
                    int a = B.off[sp] + i, b = B.off[sq] + j;
                    out[a * n + b] = out[b * n + a] = buf[i * nq + j];
                }
        }
    free(B.off);
    return 0;
}

/* (mn|P), out[(m*nbf+n)*naux+P]. */
int fcci_eri3c(int nsh, const double *xyz, const int *lq, const int *np, const int *po,
               const double *ex, const double *co, int nsha, const double *axyz, const int *alq,
               const int *anp, const int *apo, const double *aex, const double *aco, double *out) {
    basis_t B, A;
    if (basis_init(&B, nsh, xyz, lq, np, po, ex, co)) return -1;
    if (basis_init(&A, nsha, axyz, alq, anp, apo, aex, aco)) { free(B.off); return -1; }
    for (int s = 0; s < nsh; ++s)
        if (lq[s] > 2) { free(B.off); free(A.off); return -1; }
    int n = B.nbf, na = A.nbf;
    int npair = nsh * (nsh + 1) / 2;
#pragma omp parallel for schedule(dynamic)
    for (int pr = 0; pr < npair; ++pr) {
        int sa = (int)((sqrt(8.0 * pr + 1.0) - 1.0) / 2.0);
        while (sa * (sa + 1) / 2 > pr) --sa;
        while ((sa + 1) * (sa + 2) / 2 <= pr) ++sa;
        int sb = pr - sa * (sa + 1) / 2;
        sh_t Sa = get_shell(&B, sa), Sb = get_shell(&B, sb), N = get_shell(&B, -1);
        int nsa = nsph(Sa.l), nsb = nsph(Sb.l);
        double buf[5 * 5 * 9];
        for (int sc = 0; sc < nsha; ++sc) {
            sh_t Sc = get_shell(&A, sc);
            int nsc = nsph(Sc.l);
            eri_sph(&Sa, &Sb, &Sc, &N, buf);
            for (int i = 0; i < nsa; ++i)
                for (int j = 0; j < nsb; ++j)
                    for (int k = 0; k < nsc; ++k) {
                        int mu = B.off[sa] + i, nu = B.off[sb] + j, P = A.off[sc] + k;
                        double v = buf[(i * nsb + j) * nsc + k];
                        out[((size_t)mu * n + nu) * na + P] = v;
                        out[((size_t)nu * n + mu) * na + P] = v;
                    }
        }
    }
    free(B.off); free(A.off);
    return 0;
}

/* (mn|ls), out[((m*n+n)*n+l)*n+s], full array (small bases only). */
int fcci_eri4c(int nsh, const double *xyz, const int *lq, const int *np, const int *po,
               const double *ex, const double *co, double *out) {
    basis_t B;
    if (basis_init(&B, nsh, xyz, lq, np, po, ex, co)) return -1;
    size_t n = (size_t)B.nbf;
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int sa = 0; sa < nsh; ++sa)
        for (int sb = 0; sb < nsh; ++sb) {
            double buf[9 * 9 * 9 * 9];
            sh_t Sa = get_shell(&B, sa), Sb = get_shell(&B, sb);
            for (int sc = 0; sc < nsh; ++sc)
                for (int sd = 0; sd < nsh; ++sd) {
                    sh_t Sc = get_shell(&B, sc), Sd = get_shell(&B, sd);
                    eri_sph(&Sa, &Sb, &Sc, &Sd, buf);
                    int na_ = nsph(Sa.l), nb_ = nsph(Sb.l), nc_ = nsph(Sc.l), nd_ = nsph(Sd.l);
                    for (int i = 0; i < na_; ++i)
                        for (int j = 0; j < nb_; ++j)
                            for (int k = 0; k < nc_; ++k)
                                for (int l = 0; l < nd_; ++l)
                                    out[(((B.off[sa] + i) * n + B.off[sb] + j) * n + B.off[sc] + k) * n + B.off[sd] + l] =
                                        buf[((i * nb_ + j) * nc_ + k) * nd_ + l];
                }
        }
    free(B.off);
    return 0;
}

/* number of spherical functions of a shell list (helper for callers) */
int fcci_nbf(int nsh, const int *lq) {
    int n = 0;
    for (int s = 0; s < nsh; ++s) {
        if (lq[s] < 0 || lq[s] > LMAX) return -1;
        n += 2 * lq[s] + 1;
    }
    return n;
}
