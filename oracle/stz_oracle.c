/* CPU oracle for the quasi-static STZ time step: TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's quasi-static step and of the tgmg
 * V-cycle solver it calls.  Each function names the reference lines it
 * restates (paths inside the SURGroup/STZ tree).  The arithmetic follows the
 * reference expression by expression where that is cheap; the coarse-grid
 * Galerkin operators are formed by a generic R*A*P product (the reference
 * generates straight-line code for the same product, tgmg_compile.pl), so
 * they agree with the reference's to rounding.
 *
 * Built with -ffp-contract=off so that x86 and Arm builds round alike.
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 */
#include "stz_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double a, b, c, d; } m2; /* row-major 2x2: (a b; c d) */
typedef struct { double x, y; } v2;

static inline v2 mv(m2 A, v2 z) { v2 r = {A.a * z.x + A.b * z.y, A.c * z.x + A.d * z.y}; return r; }
static inline m2 mm(m2 A, m2 B) {
    m2 r = {A.a * B.a + A.b * B.c, A.a * B.b + A.b * B.d, A.c * B.a + A.d * B.c, A.c * B.b + A.d * B.d};
    return r;
}
static inline m2 madd(m2 A, m2 B) { m2 r = {A.a + B.a, A.b + B.b, A.c + B.c, A.d + B.d}; return r; }
static inline m2 mscale(m2 A, double s) { m2 r = {A.a * s, A.b * s, A.c * s, A.d * s}; return r; }
/* 1/M as esim/shared/mat.hh operator/(double,mat). */
static inline m2 minv(m2 f) {
    double idet = 1. / (f.a * f.d - f.b * f.c);
    m2 r = {f.d * idet, -f.b * idet, -f.c * idet, f.a * idet};
    return r;
}
static const m2 MZERO = {0, 0, 0, 0};

/* ---------------------------------------------------------------------- */
/* Multigrid hierarchy (esim/tgmg/tgmg.hh:48-495)                          */

#define MAXLEV 16
typedef struct {
    int m, n, mn, sm, sn;
    v2 *b, *z;  /* coarse levels own these; the top level aliases src/vel */
    m2 *st;     /* 10 per point: dl dc dr cl cc cr ul uc ur inv(cc) */
    v2 *r;      /* residual scratch */
} level;

struct stzo_sim {
    stzo_params P;
    int m, n, mn;
    double lx, ly, dx, dy, xsp, ysp, mu_inv, bcs;
    double time;
    double *u, *v, *p, *q, *s, *tau, *chi, *X, *Y, *ddev;
    double *cp, *cq, *cs, *ctau, *cchi, *cX, *cY, *cu, *cv;
    v2 *vel, *src;
    /* qs_multi constants (qs_multi.cc:9-15, 31-55) */
    double Kq, qK, Kmu, xsp2, ysp2, xyfac, tmufac1, tmufac2;
    double viscdt_prev, Kmx, Kmy, mx, my, cxx, cyy;
    m2 regh, regv, regc, regci, regcb, regcbi;
    int tol_mode;
    double acc, rtol;
    /* tgmg hierarchy: lv[0] is the top (node) grid */
    int nl;
    level lv[MAXLEV + 1];
    /* tgmg_predict (tgmg_predict.hh:6-33, tgmg_config.hh:26-45) */
    int lim, mult, decay, max_thresh, extra_iters;
    long vcount;
};

/* Index helpers: every per-point array holds rows -1..n, m entries each. */
#define CI(S, i, j) ((size_t)((j) + 1) * (S)->m + (i))

static double bdry_vel(const stzo_sim *s) {  /* shear_sim.hh:120 */
    return s->time < 1 ? s->time * s->P.u_bdry : s->P.u_bdry;
}
static double bdry_pos(const stzo_sim *s) {  /* shear_sim.hh:124 */
    return s->time < 1 ? s->P.u_bdry * s->time * s->time * 0.5 : s->P.u_bdry * (s->time - 0.5);
}

/* ---------------------------------------------------------------------- */
/* STZ plasticity laws (esim/sb/main/stz_model.hh:9-207).  The yield stress
 * s_y replaces the reference's hard-wired unit scale s0(1) and its `sbar<1`
 * tests; s_y=1 restores the reference exactly. */

static double dplastic(const stzo_params *P, double sbar, double chi, double *dchi1, double *dchi2) {
    const double s0 = P->s_y, thetainv = 1 / P->theta;
    const double Om = P->Omegaeps0, De = P->Delta, tau0 = P->tau0;
    if (P->stz_model == 0 || P->stz_model == 1) {
        double sC1, sC2, sC, sT;
        if (P->stz_model == 0) { /* stz_model.hh:58-67 */
            sC1 = exp(-De * thetainv);
            sC2 = cosh(Om * sbar * thetainv);
            sC = sC1 * sC2;
            sT = tanh(Om * sbar * thetainv);
        } else { /* stz_model.hh:76-87 */
            double x = Om * sbar / De;
            sC1 = exp(-De * thetainv);
            sC = exp(-De * cosh(x) * thetainv) * cosh(De * sinh(x) * thetainv);
            sC2 = sC / sC1;
            sT = tanh(De * sinh(x) * thetainv);
        }
        /* Dplastic_common, stz_model.hh:30-48 */
        double sbart = sbar > 1e-12 ? sbar : 1e-12, bfac = exp(-1 / chi),
               pM = 1 + sbart * sT / s0 + P->rho / (2 * sC2),
               M = s0 / (2 * sbart) * (pM - sqrt(pM * pM - 4 * sbart * sT / s0)),
               Dpl = bfac * sC * (sT - M) / tau0,
               Gamma = 2 * tau0 * Dpl * sbar / (s0 * bfac);
        bfac /= tau0 * P->c0;
        *dchi1 = bfac * Gamma;
        *dchi2 = bfac * P->kappa * sC1 * P->rho;
        return Dpl;
    }
    *dchi2 = 0;
    if (sbar < s0) { *dchi1 = 0; return 0; }
    double sC, sT, tmp;
    if (P->stz_model == 3) { /* stz_model.hh:179-206 */
        double x = Om * sbar / De;
        sC = 0.5 * (exp(-De * thetainv * exp(x)) + exp(-De * thetainv * exp(-x)));
        sT = tanh(De * sinh(x) * thetainv);
    } else { /* stz_model.hh:103-151 */
        int tm = P->t_model;
        if (tm == -1 || De >= Om * sbar)
            sC = 0.5 * (exp((Om * sbar - De) * thetainv) + exp((-Om * sbar - De) * thetainv));
        else switch (tm) {
            case 0: sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + 1); break;
            case 1: tmp = Om * sbar / De;
                    sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + sqrt(0.5 * (1 + tmp * tmp))); break;
            case 2: tmp = Om * sbar / De;
                    sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + (0.5 * (1 + tmp * tmp))); break;
            case 3: { double t_grad = 0.5 * Om / De;
                      double t_icpt = 0; /* stz_model.hh:97: default intercept */
                      sC = t_icpt + sbar * t_grad; } break;
            case 4: sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + (Om * sbar - De) * thetainv + 1); break;
            default: sC = 0;
        }
        sT = tm != 3 ? tanh(Om * sbar * thetainv) : 1;
    }
    double bfac = exp(-1 / chi), Dpl = bfac * sC * (sT - s0 / sbar) / tau0,
           Gamma = 2 * tau0 * Dpl * sbar / (s0 * bfac);
    *dchi1 = bfac * Gamma / (tau0 * P->c0);
    return Dpl;
}

/* shear_sim::adaptive_plastic_term, shear_sim.cc:513-548 */
static double adaptive_plastic_term(const stzo_params *P, double sbar, double *chiv, double *ddev, double dt) {
    const double small_dev_cutoff = 1e-12, theta = 0;
    int adapt = 1;
    double dtl = dt, osbar = sbar, dplas, dchi1, dchi2, adt;
    if (sbar < small_dev_cutoff) { *ddev = 0; return 0; }
    do {
        dplas = 2 * P->t_scale * P->mu * dplastic(P, sbar, *chiv, &dchi1, &dchi2);
        if (fabs(dtl * dplas) > P->adapt_fac) {
            adt = P->adapt_fac / fabs(dplas);
            dtl -= adt;
        } else {
            adapt = 0;
            adt = dtl;
        }
        sbar -= adt * dplas;
        *chiv += (dchi1 * (P->chi_inf - *chiv) + dchi2 * (theta - *chiv)) * P->t_scale * adt;
    } while (adapt);
    *ddev = osbar - sbar;
    return *ddev / osbar;
}

/* ---------------------------------------------------------------------- */
/* ENO helpers, shear_sim.cc:588-655 */

static inline double eno2(double p0, double p1, double p2, double p3) {
    return fabs(p0 - 2 * p1 + p2) > fabs(p1 - 2 * p2 + p3) ? 3 * p1 - 4 * p2 + p3 : p0 - p2;
}

/* chi diffusion, shear_sim::chi_diffusion, shear_sim.cc:364-386: added to
 * cchi from the old chi and the step's ddev (adds exact zeros when both
 * coefficients vanish, so it is skipped then) */
static void chi_diffusion(stzo_sim *S, double dt) {
    const int m = S->m, n = S->n;
    const double hx = 0.5 * S->xsp * dt, hy = 0.5 * S->ysp * dt;
    if (S->P.chi_diff != 0 || S->P.chi_len != 0) {
        const double hxxcd = 2 * S->xsp * hx * S->P.chi_diff, hyycd = 2 * S->ysp * hy * S->P.chi_diff,
                     hccd = 2 * (hxxcd + hyycd);
        const double dfac = 0.25 * S->P.chi_len * S->P.chi_len * S->mu_inv, dfacx = dfac * S->xsp * S->xsp,
                     dfacy = dfac * S->ysp * S->ysp;
        const double *ch = S->chi, *dd = S->ddev;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
                size_t c = CI(S, i, j), cl = CI(S, il, j), cr = CI(S, ir, j), cd = CI(S, i, j - 1),
                       cu = CI(S, i, j + 1);
                double Dd = dd[c] + dd[cd], Dl = dd[c] + dd[cl], Dr = dd[c] + dd[cr], Du = dd[c] + dd[cu];
                S->cchi[c] += hxxcd * (ch[cr] + ch[cl]) + hyycd * (ch[cu] + ch[cd]) - hccd * ch[c]
                              + dfacx * (Dr * ch[cr] - (Dr + Dl) * ch[c] + Dl * ch[cl])
                              + dfacy * (Du * ch[cu] - (Du + Dd) * ch[c] + Dd * ch[cd]);
            }
    }
}

/* ---------------------------------------------------------------------- */
/* Advection + plasticity, shear_sim::advection_step, shear_sim.cc:296-361 */

static void advection_step(stzo_sim *S, double dt) {
    const int m = S->m, n = S->n;
    const double hx = 0.5 * S->xsp * dt, hy = 0.5 * S->ysp * dt, lx = S->lx;
    const double *u = S->u, *v = S->v, *X = S->X, *Y = S->Y;
    const double *fld[5] = {S->p, S->q, S->s, S->tau, S->chi};
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < m; i++) {
            const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
            const int il2 = i <= 1 ? i + m - 2 : i - 2, ir2 = i >= m - 2 ? i + 2 - m : i + 2;
            const size_t c = CI(S, i, j);
            double uc, vc, two_omega, dtmp;
            if (j > 0) {
                double Xx, Xy, Yx, Yy;
                uc = u[c]; vc = v[c];
                if (uc > 0) {
                    Xx = hx * eno2(X[CI(S, ir, j)] + (i == m - 1 ? lx : 0), X[c],
                                   X[CI(S, il, j)] + (i == 0 ? -lx : 0), X[CI(S, il2, j)] + (i <= 1 ? -lx : 0));
                    Yx = hx * eno2(Y[CI(S, ir, j)], Y[c], Y[CI(S, il, j)], Y[CI(S, il2, j)]);
                } else {
                    Xx = -hx * eno2(X[CI(S, il, j)] + (i == 0 ? -lx : 0), X[c],
                                    X[CI(S, ir, j)] + (i == m - 1 ? lx : 0), X[CI(S, ir2, j)] + (i >= m - 2 ? lx : 0));
                    Yx = -hx * eno2(Y[CI(S, il, j)], Y[c], Y[CI(S, ir, j)], Y[CI(S, ir2, j)]);
                }
                if (vc > 0) {
                    if (j > 1) {
                        Xy = hy * eno2(X[CI(S, i, j + 1)], X[c], X[CI(S, i, j - 1)], X[CI(S, i, j - 2)]);
                        Yy = hy * eno2(Y[CI(S, i, j + 1)], Y[c], Y[CI(S, i, j - 1)], Y[CI(S, i, j - 2)]);
                    } else {
                        Xy = 2 * hy * (X[c] - X[CI(S, i, j - 1)]);
                        Yy = 2 * hy * (Y[c] - Y[CI(S, i, j - 1)]);
                    }
                } else {
                    if (j < n - 1) {
                        Xy = -hy * eno2(X[CI(S, i, j - 1)], X[c], X[CI(S, i, j + 1)], X[CI(S, i, j + 2)]);
                        Yy = -hy * eno2(Y[CI(S, i, j - 1)], Y[c], Y[CI(S, i, j + 1)], Y[CI(S, i, j + 2)]);
                    } else {
                        Xy = 2 * -hy * (X[c] - X[CI(S, i, j + 1)]);
                        Yy = 2 * -hy * (Y[c] - Y[CI(S, i, j + 1)]);
                    }
                }
                S->cX[c] = -uc * Xx - vc * Xy;
                S->cY[c] = -uc * Yx - vc * Yy;
            }
            /* staggered velocity, spin */
            const size_t cr = CI(S, ir, j), cu = CI(S, i, j + 1), cur = CI(S, ir, j + 1);
            uc = 0.25 * (u[c] + u[cr] + u[cu] + u[cur]);
            vc = 0.25 * (v[c] + v[cr] + v[cu] + v[cur]);
            two_omega = hx * (-v[c] + v[cr] - v[cu] + v[cur]) - hy * (-u[c] - u[cr] + u[cu] + u[cur]);
            double f1[5], f2[5];
            for (int k = 0; k < 5; k++) {
                const double *F = fld[k];
                if (uc > 0) f1[k] = hx * eno2(F[CI(S, ir, j)], F[c], F[CI(S, il, j)], F[CI(S, il2, j)]);
                else f1[k] = -hx * eno2(F[CI(S, il, j)], F[c], F[CI(S, ir, j)], F[CI(S, ir2, j)]);
                if (vc > 0) {
                    if (j > 0) f2[k] = hy * eno2(F[CI(S, i, j + 1)], F[c], F[CI(S, i, j - 1)], F[CI(S, i, j - 2)]);
                    else f2[k] = 2 * hy * (F[c] - F[CI(S, i, j - 1)]);
                } else {
                    if (j < n - 1) f2[k] = -hy * eno2(F[CI(S, i, j - 1)], F[c], F[CI(S, i, j + 1)], F[CI(S, i, j + 2)]);
                    else f2[k] = 2 * -hy * (F[c] - F[CI(S, i, j + 1)]);
                }
            }
            const double pv = S->p[c], qv = S->q[c], sv = S->s[c], tv = S->tau[c];
            double cchi = S->chi[c] - uc * f1[4] - vc * f2[4], ddev;
            dtmp = adaptive_plastic_term(&S->P, sqrt(3 * qv * qv + sv * sv + tv * tv), &cchi, &ddev, dt);
            S->cchi[c] = cchi;
            S->ddev[c] = ddev;
            S->cp[c] = -uc * f1[0] - vc * f2[0];
            S->cq[c] = -uc * f1[1] - vc * f2[1] - dtmp * qv;
            S->cs[c] = -uc * f1[2] - vc * f2[2] + two_omega * tv - dtmp * sv;
            S->ctau[c] = -uc * f1[3] - vc * f2[3] - two_omega * sv - dtmp * tv;
            (void)pv;
        }
    }
    chi_diffusion(S, dt);
    /* apply the updates, shear_sim.cc:356-360 and fields.hh:61-80 */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            size_t c = CI(S, i, j);
            if (j > 0) { S->X[c] += S->cX[c]; S->Y[c] += S->cY[c]; }
            S->p[c] += S->cp[c];
            S->q[c] += S->cq[c];
            S->s[c] += S->cs[c];
            S->tau[c] += S->ctau[c];
            S->chi[c] = S->cchi[c];
        }
}

/* ---------------------------------------------------------------------- */
/* Explicit (direct) step, shear_sim::step_forward, shear_sim.cc:185-276:
 * velocity and reference map advected with ENO2 at the nodes, plus the net
 * force of the stress (net_force, shear_sim.cc:447-453, prefactors -hx,-hy)
 * and a 5-point viscous term; the cells take the advection, the elastic
 * rate from the velocity gradient and the plastic term.  The constant chi
 * diffusion enters cchi before the plastic term and again in chi_diffusion
 * (the reference adds it twice), and ddev is stored times the old |s|.
 * The raw stress drop is returned per cell in raw_ddev for eps_pl. */

static void direct_step(stzo_sim *S, double dt, double *raw_ddev) {
    const int m = S->m, n = S->n;
    const double third = 1. / 3;
    const double hx = 0.5 * S->xsp * dt, hy = 0.5 * S->ysp * dt, lx = S->lx;
    const double visc = S->P.viscosity;
    const double hxxv = 2 * S->xsp * hx * visc, hyyv = 2 * S->ysp * hy * visc, hcv = 2 * (hxxv + hyyv);
    const double hxxcd = 2 * S->xsp * hx * S->P.chi_diff, hyycd = 2 * S->ysp * hy * S->P.chi_diff,
                 hccd = 2 * (hxxcd + hyycd);
    const double K = S->P.K, mu = S->P.mu, mu_inv = S->mu_inv;
    const double *u = S->u, *v = S->v, *X = S->X, *Y = S->Y;
    const double *fld[5] = {S->p, S->q, S->s, S->tau, S->chi};
    double *cu = S->cu, *cv = S->cv;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < m; i++) {
            const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
            const int il2 = i <= 1 ? i + m - 2 : i - 2, ir2 = i >= m - 2 ? i + 2 - m : i + 2;
            const size_t c = CI(S, i, j);
            double uc, vc;
            if (j > 0) {
                double ux, vx, uy, vy, Xx, Yx, Xy, Yy;
                uc = u[c]; vc = v[c];
                if (uc > 0) {
                    ux = hx * eno2(u[CI(S, ir, j)], u[c], u[CI(S, il, j)], u[CI(S, il2, j)]);
                    vx = hx * eno2(v[CI(S, ir, j)], v[c], v[CI(S, il, j)], v[CI(S, il2, j)]);
                    Xx = hx * eno2(X[CI(S, ir, j)] + (i == m - 1 ? lx : 0), X[c],
                                   X[CI(S, il, j)] + (i == 0 ? -lx : 0), X[CI(S, il2, j)] + (i <= 1 ? -lx : 0));
                    Yx = hx * eno2(Y[CI(S, ir, j)], Y[c], Y[CI(S, il, j)], Y[CI(S, il2, j)]);
                } else {
                    ux = -hx * eno2(u[CI(S, il, j)], u[c], u[CI(S, ir, j)], u[CI(S, ir2, j)]);
                    vx = -hx * eno2(v[CI(S, il, j)], v[c], v[CI(S, ir, j)], v[CI(S, ir2, j)]);
                    Xx = -hx * eno2(X[CI(S, il, j)] + (i == 0 ? -lx : 0), X[c],
                                    X[CI(S, ir, j)] + (i == m - 1 ? lx : 0), X[CI(S, ir2, j)] + (i >= m - 2 ? lx : 0));
                    Yx = -hx * eno2(Y[CI(S, il, j)], Y[c], Y[CI(S, ir, j)], Y[CI(S, ir2, j)]);
                }
                if (vc > 0) {
                    if (j > 1) {
                        const size_t a = CI(S, i, j + 1), b = CI(S, i, j - 1), d = CI(S, i, j - 2);
                        uy = hy * eno2(u[a], u[c], u[b], u[d]);
                        vy = hy * eno2(v[a], v[c], v[b], v[d]);
                        Xy = hy * eno2(X[a], X[c], X[b], X[d]);
                        Yy = hy * eno2(Y[a], Y[c], Y[b], Y[d]);
                    } else {
                        const size_t b = CI(S, i, j - 1);
                        uy = 2 * hy * (u[c] - u[b]);
                        vy = 2 * hy * (v[c] - v[b]);
                        Xy = 2 * hy * (X[c] - X[b]);
                        Yy = 2 * hy * (Y[c] - Y[b]);
                    }
                } else {
                    if (j < n - 1) {
                        const size_t a = CI(S, i, j - 1), b = CI(S, i, j + 1), d = CI(S, i, j + 2);
                        uy = -hy * eno2(u[a], u[c], u[b], u[d]);
                        vy = -hy * eno2(v[a], v[c], v[b], v[d]);
                        Xy = -hy * eno2(X[a], X[c], X[b], X[d]);
                        Yy = -hy * eno2(Y[a], Y[c], Y[b], Y[d]);
                    } else {
                        const size_t b = CI(S, i, j + 1);
                        uy = 2 * -hy * (u[c] - u[b]);
                        vy = 2 * -hy * (v[c] - v[b]);
                        Xy = 2 * -hy * (X[c] - X[b]);
                        Yy = 2 * -hy * (Y[c] - Y[b]);
                    }
                }
                /* net force from the cells (i-1,j-1), (i,j-1), (i-1,j), (i,j) */
                const size_t c0 = CI(S, il, j - 1), c1 = CI(S, i, j - 1), c2 = CI(S, il, j), c3 = c;
                const double *P = S->p, *Q = S->q, *SS = S->s, *T = S->tau;
                const double xf = -hx, yf = -hy;
                const double fx = (-P[c0] + P[c1] - P[c2] + P[c3] - Q[c0] + Q[c1] - Q[c2] + Q[c3] + SS[c0] - SS[c1] +
                                   SS[c2] - SS[c3]) * xf + (T[c0] + T[c1] - T[c2] - T[c3]) * yf;
                const double fy = (T[c0] - T[c1] + T[c2] - T[c3]) * xf +
                                  (-P[c0] - P[c1] + P[c2] + P[c3] - Q[c0] - Q[c1] + Q[c2] + Q[c3] - SS[c0] - SS[c1] +
                                   SS[c2] + SS[c3]) * yf;
                const size_t cr = CI(S, ir, j), cl = CI(S, il, j), cup = CI(S, i, j + 1), cdn = CI(S, i, j - 1);
                const double uvisc = hxxv * (u[cr] + u[cl]) + hyyv * (u[cup] + u[cdn]) - hcv * uc;
                const double vvisc = hxxv * (v[cr] + v[cl]) + hyyv * (v[cup] + v[cdn]) - hcv * vc;
                cu[c] = -uc * ux - vc * uy + mu_inv * (fx + uvisc);
                cv[c] = -uc * vx - vc * vy + mu_inv * (fy + vvisc);
                S->cX[c] = -uc * Xx - vc * Xy;
                S->cY[c] = -uc * Yx - vc * Yy;
            }
            /* deformation rate, staggered velocity, spin */
            const size_t cr = CI(S, ir, j), cup = CI(S, i, j + 1), cur = CI(S, ir, j + 1);
            uc = 0.25 * (u[c] + u[cr] + u[cup] + u[cur]);
            vc = 0.25 * (v[c] + v[cr] + v[cup] + v[cur]);
            const double ux = hx * (-u[c] + u[cr] - u[cup] + u[cur]), uy = hy * (-u[c] - u[cr] + u[cup] + u[cur]);
            const double vx = hx * (-v[c] + v[cr] - v[cup] + v[cur]), vy = hy * (-v[c] - v[cr] + v[cup] + v[cur]);
            const double two_omega = vx - uy;
            double f1[5], f2[5];
            for (int k = 0; k < 5; k++) {
                const double *F = fld[k];
                if (uc > 0) f1[k] = hx * eno2(F[CI(S, ir, j)], F[c], F[CI(S, il, j)], F[CI(S, il2, j)]);
                else f1[k] = -hx * eno2(F[CI(S, il, j)], F[c], F[CI(S, ir, j)], F[CI(S, ir2, j)]);
                if (vc > 0) {
                    if (j > 0) f2[k] = hy * eno2(F[CI(S, i, j + 1)], F[c], F[CI(S, i, j - 1)], F[CI(S, i, j - 2)]);
                    else f2[k] = 2 * hy * (F[c] - F[CI(S, i, j - 1)]);
                } else {
                    if (j < n - 1) f2[k] = -hy * eno2(F[CI(S, i, j - 1)], F[c], F[CI(S, i, j + 1)], F[CI(S, i, j + 2)]);
                    else f2[k] = 2 * -hy * (F[c] - F[CI(S, i, j + 1)]);
                }
            }
            const double *ch = S->chi;
            const double qv = S->q[c], sv = S->s[c], tv = S->tau[c];
            const double sbar = sqrt(3 * qv * qv + sv * sv + tv * tv);
            double cchi = ch[c] - uc * f1[4] - vc * f2[4] + hxxcd * (ch[cr] + ch[CI(S, il, j)]) +
                          hyycd * (ch[cup] + ch[CI(S, i, j - 1)]) - hccd * ch[c];
            double ddev;
            const double dtmp = adaptive_plastic_term(&S->P, sbar, &cchi, &ddev, dt);
            S->cchi[c] = cchi;
            S->cp[c] = -uc * f1[0] - vc * f2[0] - K * (ux + vy);
            S->cq[c] = -uc * f1[1] - vc * f2[1] - mu * third * (ux + vy) - dtmp * qv;
            S->cs[c] = -uc * f1[2] - vc * f2[2] + two_omega * tv + mu * (ux - vy) - dtmp * sv;
            S->ctau[c] = -uc * f1[3] - vc * f2[3] - two_omega * sv + mu * (vx + uy) - dtmp * tv;
            if (raw_ddev) raw_ddev[(size_t)j * m + i] = ddev;
            S->ddev[c] = ddev * sbar;
        }
    }
    chi_diffusion(S, dt);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            size_t c = CI(S, i, j);
            if (j > 0) {
                S->u[c] += cu[c];
                S->v[c] += cv[c];
                S->X[c] += S->cX[c];
                S->Y[c] += S->cY[c];
            }
            S->p[c] += S->cp[c];
            S->q[c] += S->cq[c];
            S->s[c] += S->cs[c];
            S->tau[c] += S->ctau[c];
            S->chi[c] = S->cchi[c];
        }
}

/* ---------------------------------------------------------------------- */
/* Boundaries, shear_sim::set_boundaries, shear_sim.cc:552-581 */

static void set_boundaries(stzo_sim *S) {
    const int m = S->m, n = S->n;
    const double bv = bdry_vel(S), bp = bdry_pos(S);
    double *F[5] = {S->p, S->q, S->s, S->tau, S->chi};
    for (int i = 0; i < m; i++) {
        size_t c0 = CI(S, i, 0);
        S->u[c0] = -bv;
        S->v[c0] = 0;
        S->X[c0] = S->P.ax + i * S->dx + bp;
        S->Y[c0] = S->P.ay;
        for (int k = 0; k < 5; k++) F[k][CI(S, i, -1)] = 2 * F[k][c0] - F[k][CI(S, i, 1)];
    }
    for (int i = 0; i < m; i++) {
        size_t cn = CI(S, i, n);
        S->u[cn] = bv;
        S->v[cn] = 0;
        S->X[cn] = S->P.ax + i * S->dx - bp;
        S->Y[cn] = S->P.by;
        for (int k = 0; k < 5; k++) F[k][cn] = 2 * F[k][CI(S, i, n - 1)] - F[k][CI(S, i, n - 2)];
    }
}

/* ---------------------------------------------------------------------- */
/* qs_multi operator (qs_multi.hh:11-57) as the top multigrid level */

static inline int top_bdry(const level *L, int ij) { return ij >= L->mn - L->m || ij < L->m; }

/* a_xx entries of qs_multi.hh:22-31, ordered dl dc dr cl cc cr ul uc ur */
static m2 top_entry(const stzo_sim *S, int ij, int k) {
    const level *L = &S->lv[0];
    int b = top_bdry(L, ij);
    m2 r = MZERO;
    switch (k) {
        case 0: case 8: if (!b) { r.b = S->qK; r.c = S->qK; } break;
        case 2: case 6: if (!b) { r.b = -S->qK; r.c = -S->qK; } break;
        case 3: case 5: if (!b) r = S->regh; break;
        case 1: case 7: if (!b) r = S->regv; break;
        case 4: r = b ? S->regcb : S->regc; break;
    }
    return r;
}

/* qs_multi::mul_a, qs_multi.hh:41-50 */
static inline v2 top_mul_a(const stzo_sim *S, const v2 *z, int i, int ij) {
    const level *L = &S->lv[0];
    const int m = L->m;
    v2 r = {0, 0};
    if (top_bdry(L, ij)) return r;
    const v2 *zp = z + ij, *zd = zp + (i == 0 ? m - 1 : -1), *zu = zp + (i == m - 1 ? 1 - m : 1);
    r.x = S->Kmx * (zd->x + zu->x) + S->my * (zp[-m].x + zp[m].x)
          + S->qK * (zd[-m].y + zu[m].y - zu[-m].y - zd[m].y);
    r.y = S->mx * (zd->y + zu->y) + S->Kmy * (zp[-m].y + zp[m].y)
          + S->qK * (zd[-m].x + zu[m].x - zu[-m].x - zd[m].x);
    return r;
}

/* coarse level product with the stored stencil (tgmg.in.cc:536-547 and the
 * tsub_contrib expansion of tgmg_compile.pl:82-113); non-periodic y */
static inline v2 lev_mul_a(const level *L, const v2 *z, int i, int ij) {
    const int m = L->m, mn = L->mn;
    const m2 *e = L->st + 10 * (size_t)ij;
    const int hasd = ij >= m, hasu = ij < mn - m;
    const int dl = i == 0 ? m - 1 : -1, dr = i == m - 1 ? 1 - m : 1;
    v2 r = {0, 0}, t;
    const v2 *f = z + ij;
#define ACC(K, OFF) t = mv(e[K], f[OFF]); r.x += t.x; r.y += t.y;
    if (hasd) { ACC(0, -m + dl) ACC(1, -m) ACC(2, -m + dr) }
    ACC(3, dl) ACC(5, dr)
    if (hasu) { ACC(6, m + dl) ACC(7, m) ACC(8, m + dr) }
#undef ACC
    return r;
}

static inline v2 level_res(const stzo_sim *S, int l, int i, int ij) {
    const level *L = &S->lv[l];
    v2 a, c;
    if (l == 0) {
        a = top_mul_a(S, L->z, i, ij);
        c = mv(top_bdry(L, ij) ? S->regcb : S->regc, L->z[ij]);
    } else {
        a = lev_mul_a(L, L->z, i, ij);
        c = mv(L->st[10 * (size_t)ij + 4], L->z[ij]);
    }
    v2 r = {L->b[ij].x - a.x - c.x, L->b[ij].y - a.y - c.y};
    return r;
}

/* tgmg_base::gauss_seidel, gs_mode 0, non-periodic y: odd rows, then even
 * rows, each row left to right (tgmg.in.cc:128-148) */
static void gauss_seidel(stzo_sim *S, int l) {
    level *L = &S->lv[l];
    const int m = L->m, n = L->n;
    for (int pass = 1; pass >= 0; pass--) {
#pragma omp parallel for schedule(static) if (L->mn > 4096)
        for (int j = pass; j < n; j += 2) {
            for (int i = 0, ij = j * m; i < m; i++, ij++) {
                v2 a, bb;
                if (l == 0) {
                    a = top_mul_a(S, L->z, i, ij);
                    bb.x = L->b[ij].x - a.x; bb.y = L->b[ij].y - a.y;
                    L->z[ij] = mv(top_bdry(L, ij) ? S->regcbi : S->regci, bb);
                } else {
                    a = lev_mul_a(L, L->z, i, ij);
                    bb.x = L->b[ij].x - a.x; bb.y = L->b[ij].y - a.y;
                    L->z[ij] = mv(L->st[10 * (size_t)ij + 9], bb);
                }
            }
        }
    }
}

/* mds(), tgmg.in.cc:55-64: sum of squared residuals (rows summed in order) */
static double mds(stzo_sim *S, int l) {
    level *L = &S->lv[l];
    const int m = L->m, n = L->n;
    double *rowsum = (double *)malloc(sizeof(double) * n);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
        double cl = 0;
        for (int i = 0, ij = j * m; i < m; i++, ij++) {
            v2 r = level_res(S, l, i, ij);
            cl += r.x * r.x + r.y * r.y;
        }
        rowsum[j] = cl;
    }
    double c = 0;
    for (int j = 0; j < n; j++) c += rowsum[j];
    free(rowsum);
    return c;
}

/* 1D transfer weights (apply_t, tgmg.in.cc:552-621): the coarse points that
 * feed fine index f, for a fine line of length um. */
static int p1d(int f, int um, int prd, int *c, double *w) {
    int sm = (um + (prd ? 1 : 2)) >> 1;
    if (!(f & 1)) { c[0] = f >> 1; w[0] = 1; return 1; }
    if (!prd && !(um & 1) && f == um - 1) { c[0] = sm - 1; w[0] = 1; return 1; }
    c[0] = f >> 1; w[0] = 0.5;
    c[1] = (prd && f == um - 1) ? 0 : (f >> 1) + 1; w[1] = 0.5;
    return 2;
}

/* apply_r (tgmg.in.cc:626-647 and the generated r_*_line routines): residual
 * of level l restricted into b of level l+1 with R = P^T, summed per coarse
 * point over its fine support. */
static void apply_r(stzo_sim *S, int l) {
    level *F = &S->lv[l], *C = &S->lv[l + 1];
    const int m = F->m, n = F->n;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0, ij = j * m; i < m; i++, ij++) F->r[ij] = level_res(S, l, i, ij);
#pragma omp parallel for schedule(static)
    for (int J = 0; J < C->n; J++)
        for (int I = 0; I < C->m; I++) {
            v2 acc = {0, 0};
            for (int fy = 2 * J - 2; fy <= 2 * J + 2; fy++) {
                if (fy < 0 || fy >= n) continue;
                int cy[2], ny; double wy[2], py = 0;
                ny = p1d(fy, n, 0, cy, wy);
                for (int b = 0; b < ny; b++) if (cy[b] == J) py += wy[b];
                if (py == 0) continue;
                for (int dfx = -2; dfx <= 2; dfx++) {
                    int fx = ((2 * I + dfx) % m + m) % m;
                    int cx[2], nx; double wx[2], px = 0;
                    nx = p1d(fx, m, 1, cx, wx);
                    for (int a = 0; a < nx; a++) if (cx[a] == I) px += wx[a];
                    if (px == 0) continue;
                    v2 r = F->r[fy * m + fx];
                    acc.x += px * py * r.x;
                    acc.y += px * py * r.y;
                }
            }
            C->b[J * C->m + I] = acc;
        }
}

/* apply_t, tgmg.in.cc:552-621: bilinear prolongation of level l's z added to
 * level l-1's z. */
static void apply_t(stzo_sim *S, int l) {
    level *C = &S->lv[l], *F = &S->lv[l - 1];
    const int m = F->m, n = F->n;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
        int cy[2], nyc; double wy[2];
        nyc = p1d(j, n, 0, cy, wy);
        for (int i = 0, ij = j * m; i < m; i++, ij++) {
            int cx[2], nxc; double wx[2];
            nxc = p1d(i, m, 1, cx, wx);
            v2 acc = {0, 0};
            for (int b = 0; b < nyc; b++)
                for (int a = 0; a < nxc; a++) {
                    double w = wx[a] * wy[b];
                    v2 zc = C->z[cy[b] * C->m + cx[a]];
                    acc.x += w * zc.x;
                    acc.y += w * zc.y;
                }
            F->z[ij].x += acc.x;
            F->z[ij].y += acc.y;
        }
    }
}

/* Galerkin coarse operator of level l+1 (tgmg_base::rat, tgmg.in.cc:667-736,
 * and compute_rat[_bdry] generated by tgmg_compile.pl:151-338): for every
 * coarse point I and neighbour J, sum_k sum_l P(k,I) A(k,l) P(l,J). */
static void compute_rat(stzo_sim *S, int l) {
    level *F = &S->lv[l], *C = &S->lv[l + 1];
    const int fm = F->m, fn = F->n, cm = C->m, cn = C->n;
    /* fine points feeding each coarse index, per dimension */
#pragma omp parallel for schedule(dynamic, 4)
    for (int J = 0; J < cn; J++) {
        for (int I = 0; I < cm; I++) {
            m2 acc[9];
            for (int k = 0; k < 9; k++) acc[k] = MZERO;
            /* fine support of the coarse basis function at (I,J) */
            for (int fy = 2 * J - 2; fy <= 2 * J + 2; fy++) {
                if (fy < 0 || fy >= fn) continue;
                int cy[2], ny; double wy[2];
                ny = p1d(fy, fn, 0, cy, wy);
                double pyk = 0;
                for (int b = 0; b < ny; b++) if (cy[b] == J) pyk += wy[b];
                if (pyk == 0) continue;
                for (int dfx = -2; dfx <= 2; dfx++) {
                    int fx = ((2 * I + dfx) % fm + fm) % fm;
                    int cx[2], nx; double wx[2];
                    nx = p1d(fx, fm, 1, cx, wx);
                    double pxk = 0;
                    for (int a = 0; a < nx; a++) if (cx[a] == I) pxk += wx[a];
                    if (pxk == 0) continue;
                    double rk = pxk * pyk;
                    int kij = fy * fm + fx;
                    /* fine stencil of point k */
                    for (int sy = -1; sy <= 1; sy++) {
                        int ly = fy + sy;
                        if (ly < 0 || ly >= fn) continue;
                        for (int sx = -1; sx <= 1; sx++) {
                            int lxx = ((fx + sx) % fm + fm) % fm;
                            int ks = (sy + 1) * 3 + (sx + 1);
                            m2 A;
                            if (l == 0) A = top_entry(S, kij, ks);
                            else A = F->st[10 * (size_t)kij + ks];
                            if (A.a == 0 && A.b == 0 && A.c == 0 && A.d == 0) continue;
                            int lcy[2], lny, lcx[2], lnx; double lwy[2], lwx[2];
                            lny = p1d(ly, fn, 0, lcy, lwy);
                            lnx = p1d(lxx, fm, 1, lcx, lwx);
                            for (int b = 0; b < lny; b++)
                                for (int a = 0; a < lnx; a++) {
                                    int oy = lcy[b] - J;
                                    int ox = lcx[a] - I;
                                    if (ox > cm / 2) ox -= cm;
                                    if (ox < -(cm / 2)) ox += cm;
                                    if (oy < -1 || oy > 1 || ox < -1 || ox > 1) {
                                        fprintf(stderr, "stz_oracle: RAP coupling outside 3x3\n");
                                        abort();
                                    }
                                    acc[(oy + 1) * 3 + (ox + 1)] =
                                        madd(acc[(oy + 1) * 3 + (ox + 1)], mscale(A, rk * lwx[a] * lwy[b]));
                                }
                        }
                    }
                }
            }
            m2 *t = C->st + 10 * ((size_t)J * cm + I);
            for (int k = 0; k < 9; k++) t[k] = acc[k];
            t[9] = minv(acc[4]);
        }
    }
}

static void clear_z(level *L) { memset(L->z, 0, sizeof(v2) * L->mn); }

/* down_gs_iterations (tgmg.hh:273-279): from zero, then cyc-1 more sweeps */
static void down_gs(stzo_sim *S, int l, int cyc) {
    clear_z(&S->lv[l]);
    for (int i = 0; i < cyc; i++) gauss_seidel(S, l);
}

/* tgmg::v_cycle with cyc_down=cyc_up=1, hcyc_bottom=10 (tgmg.in.cc:313-359) */
static void v_cycle(stzo_sim *S) {
    const int ml = S->nl - 1;
    gauss_seidel(S, 0);
    if (ml > 0) {
        apply_r(S, 0);
        down_gs(S, 1, 1);
        for (int i = 1; i < ml; i++) {
            if (i > 1) down_gs(S, i, 1);
            apply_r(S, i);
        }
        down_gs(S, ml, 10);
        for (int k = 0; k < 10; k++) gauss_seidel(S, ml);
        for (int i = ml; i > 1; i--) {
            apply_t(S, i);
            gauss_seidel(S, i - 1);
        }
        apply_t(S, 1);
    }
    gauss_seidel(S, 0);
}

static double sqnorm_b(stzo_sim *S) {
    level *L = &S->lv[0];
    double c = 0;
    for (int k = 0; k < L->mn; k++) c += L->b[k].x * L->b[k].x + L->b[k].y * L->b[k].y;
    return c;
}

/* error measure and its threshold: l2_error()=mds()/mn against acc
 * (tgmg.hh:146, tgmg.in.cc:276), or relative 2-norm of the residual */
static int converged(stzo_sim *S, double err, double bb) {
    if (S->tol_mode == 0) return err < S->acc;
    return err <= S->rtol * S->rtol * bb;
}
static double error_measure(stzo_sim *S) {
    double d = mds(S, 0);
    return S->tol_mode == 0 ? d / S->lv[0].mn : d;
}

/* tgmg::solve(type 4, tgmg_predict&), tgmg.in.cc:266-301 */
static int solve_adaptive(stzo_sim *S) {
    int nc = S->lim / S->mult;
    double bb = S->tol_mode ? sqnorm_b(S) : 0;
    for (int i = 0; i < nc; i++) v_cycle(S);
    double err = error_measure(S);
    if (converged(S, err, bb)) {
        if (S->lim > 0) S->lim -= 1 + S->lim / S->decay;
    } else {
        int k = 0;
        do {
            S->lim += ++k * S->mult;
            if (S->lim > S->max_thresh) return 0;
            nc += k;
            for (int i = 0; i < k; i++) v_cycle(S);
            err = error_measure(S);
        } while (!converged(S, err, bb));
    }
    S->vcount += nc;
    for (int i = 0; i < S->extra_iters; i++) v_cycle(S);
    return !isnan(err);
}

/* qs_multi::init, qs_multi.cc:31-55 */
static void qs_init(stzo_sim *S, double viscdt) {
    if (viscdt == S->viscdt_prev) return;
    S->viscdt_prev = viscdt;
    S->Kmx = (S->Kmu + viscdt) * S->xsp2;
    S->Kmy = (S->Kmu + viscdt) * S->ysp2;
    S->mx = (S->P.mu + viscdt) * S->xsp2;
    S->my = (S->P.mu + viscdt) * S->ysp2;
    S->cxx = -2 * (S->tmufac1 + viscdt * S->xyfac);
    S->cyy = -2 * (S->tmufac2 + viscdt * S->xyfac);
    m2 h = {S->Kmx, 0, 0, S->my}, vv = {S->mx, 0, 0, S->Kmy}, c = {S->cxx, 0, 0, S->cyy},
       ci = {1 / S->cxx, 0, 0, 1 / S->cyy}, cb = {S->bcs * S->cxx, 0, 0, S->bcs * S->cyy},
       cbi = {1 / (S->bcs * S->cxx), 0, 0, 1 / (S->bcs * S->cyy)};
    S->regh = h; S->regv = vv; S->regc = c; S->regci = ci; S->regcb = cb; S->regcbi = cbi;
    for (int l = 0; l + 1 < S->nl; l++) compute_rat(S, l);
}

/* shear_sim::projection_step, shear_sim.cc:391-438 */
static int projection_step(stzo_sim *S, double dt) {
    const int m = S->m, n = S->n;
    const double third = 1 / 3.0;
    const double hx = 0.5 * S->xsp * dt, hy = 0.5 * S->ysp * dt, xfac = 0.5 / dt * S->xsp,
                 yfac = 0.5 / dt * S->ysp;
    qs_init(S, S->P.viscosity / dt);
    const double xbc = S->bcs * S->cxx, bv = bdry_vel(S);
    for (int i = 0; i < m; i++) { S->src[i].x = -xbc * bv; S->src[i].y = 0; }
#pragma omp parallel for schedule(static)
    for (int j = 1; j < n; j++)
        for (int i = 0; i < m; i++) {
            const int il = i == 0 ? m - 1 : i - 1;
            /* net_force, shear_sim.cc:447-453: f0,f1 below, f2,f3 above */
            size_t k0 = CI(S, il, j - 1), k1 = CI(S, i, j - 1), k2 = CI(S, il, j), k3 = CI(S, i, j);
            const double *p = S->p, *q = S->q, *s = S->s, *t = S->tau;
            v2 f;
            f.x = (-p[k0] + p[k1] - p[k2] + p[k3] - q[k0] + q[k1] - q[k2] + q[k3] + s[k0] - s[k1] + s[k2] - s[k3]) * xfac
                  + (t[k0] + t[k1] - t[k2] - t[k3]) * yfac;
            f.y = (t[k0] - t[k1] + t[k2] - t[k3]) * xfac
                  + (-p[k0] - p[k1] + p[k2] + p[k3] - q[k0] - q[k1] + q[k2] + q[k3] - s[k0] - s[k1] + s[k2] + s[k3]) * yfac;
            S->src[j * m + i] = f;
        }
    for (int i = 0; i < m; i++) { S->src[n * m + i].x = xbc * bv; S->src[n * m + i].y = 0; }
    if (!solve_adaptive(S)) return 0;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            size_t c = CI(S, i, j);
            const v2 *vp = S->vel + (j * m + i), *vo = vp + (i == m - 1 ? 1 - m : 1);
            S->u[c] = vp->x;
            S->v[c] = vp->y;
            double ux = hx * (-vp->x + vo->x - vp[m].x + vo[m].x), uy = hy * (-vp->x - vo->x + vp[m].x + vo[m].x),
                   vx = hx * (-vp->y + vo->y - vp[m].y + vo[m].y), vy = hy * (-vp->y - vo->y + vp[m].y + vo[m].y);
            S->p[c] += -S->P.K * (ux + vy);
            S->q[c] += -S->P.mu * third * (ux + vy);
            S->s[c] += S->P.mu * (ux - vy);
            S->tau[c] += S->P.mu * (uy + vx);
        }
    set_boundaries(S);
    return 1;
}

/* ---------------------------------------------------------------------- */

stzo_sim *stzo_create(const stzo_params *p) {
    stzo_sim *S = (stzo_sim *)calloc(1, sizeof(stzo_sim));
    S->P = *p;
    const int m = p->m, n = p->n;
    S->m = m; S->n = n; S->mn = m * n;
    S->lx = p->bx - p->ax; S->ly = p->by - p->ay;
    S->dx = S->lx / m; S->dy = S->ly / n;
    S->xsp = 1. / S->dx; S->ysp = 1. / S->dy;
    S->mu_inv = 1 / p->mu;
    S->bcs = 4;
    size_t np = (size_t)(n + 2) * m;
    double **arr[19] = {&S->u, &S->v, &S->p, &S->q, &S->s, &S->tau, &S->chi, &S->X, &S->Y, &S->ddev,
                        &S->cp, &S->cq, &S->cs, &S->ctau, &S->cchi, &S->cX, &S->cY, &S->cu, &S->cv};
    for (int k = 0; k < 19; k++) *arr[k] = (double *)calloc(np, sizeof(double));
    S->vel = (v2 *)calloc((size_t)m * (n + 1), sizeof(v2));
    S->src = (v2 *)calloc((size_t)m * (n + 1), sizeof(v2));
    /* qs_multi constructor, qs_multi.cc:9-15 */
    S->Kq = p->K + p->mu / 3.0;
    S->qK = .25 * S->Kq * S->xsp * S->ysp;
    S->Kmu = S->Kq + p->mu;
    S->xsp2 = S->xsp * S->xsp; S->ysp2 = S->ysp * S->ysp;
    S->xyfac = S->xsp2 + S->ysp2;
    S->tmufac1 = S->Kmu * S->xsp2 + p->mu * S->ysp2;
    S->tmufac2 = p->mu * S->xsp2 + S->Kmu * S->ysp2;
    S->viscdt_prev = -1;
    stzo_set_tolerance(S, 0, 1e4);
    /* hierarchy, tgmg.in.cc:11-30 (x periodic, y not) */
    level *L = &S->lv[0];
    L->m = m; L->n = n + 1; L->mn = L->m * L->n;
    L->sm = (L->m + 1) >> 1; L->sn = (L->n + 2) >> 1;
    L->b = S->src; L->z = S->vel;
    L->r = (v2 *)calloc(L->mn, sizeof(v2));
    S->nl = 1;
    int am = L->sm, an = L->sn;
    /* coarsening stops where a periodic line would alias itself (m<3); the
     * reference collapses such levels instead (tgmg.in.cc:738-746) */
    while (am * an > 10 && am >= 3) {
        if (S->nl == MAXLEV + 1) { fprintf(stderr, "stz_oracle: too many levels\n"); abort(); }
        level *C = &S->lv[S->nl];
        C->m = am; C->n = an; C->mn = am * an;
        C->sm = (am + 1) >> 1; C->sn = (an + 2) >> 1;
        C->b = (v2 *)calloc(C->mn, sizeof(v2));
        C->z = (v2 *)calloc(C->mn, sizeof(v2));
        C->r = (v2 *)calloc(C->mn, sizeof(v2));
        C->st = (m2 *)calloc((size_t)10 * C->mn, sizeof(m2));
        am = C->sm; an = C->sn;
        S->nl++;
    }
    /* tgmg_predict defaults */
    S->mult = 16; S->decay = 32; S->max_thresh = 16 * 2048; S->extra_iters = 1;
    S->lim = S->mult * 8;
    return S;
}

void stzo_destroy(stzo_sim *S) {
    double *arr[19] = {S->u, S->v, S->p, S->q, S->s, S->tau, S->chi, S->X, S->Y, S->ddev,
                       S->cp, S->cq, S->cs, S->ctau, S->cchi, S->cX, S->cY, S->cu, S->cv};
    for (int k = 0; k < 19; k++) free(arr[k]);
    free(S->vel); free(S->src); free(S->lv[0].r);
    for (int l = 1; l < S->nl; l++) { free(S->lv[l].b); free(S->lv[l].z); free(S->lv[l].r); free(S->lv[l].st); }
    free(S);
}

void stzo_set_state(stzo_sim *S, const double *chi) {
    const int m = S->m, n = S->n;
    for (int j = -1; j <= n; j++)
        for (int i = 0; i < m; i++) {
            size_t c = CI(S, i, j);
            S->u[c] = S->v[c] = S->ddev[c] = 0;
            S->p[c] = S->q[c] = S->s[c] = S->tau[c] = 0;
            S->X[c] = S->P.ax + i * S->dx;
            S->Y[c] = S->P.ay + j * S->dy;
            if (j >= 0 && j < n) S->chi[c] = chi[(size_t)j * m + i];
        }
    for (int i = 0; i < m; i++) {
        S->chi[CI(S, i, -1)] = 2 * S->chi[CI(S, i, 0)] - S->chi[CI(S, i, 1)];
        S->chi[CI(S, i, n)] = 2 * S->chi[CI(S, i, n - 1)] - S->chi[CI(S, i, n - 2)];
    }
    memset(S->vel, 0, sizeof(v2) * (size_t)m * (n + 1));
    S->time = 0;
}

/* Resting state of every field but chi (zero velocity, stress and ddev,
 * identity reference map), rows -1..n, and a cleared solver array. */
static void rest_state(stzo_sim *S) {
    const int m = S->m, n = S->n;
    for (int j = -1; j <= n; j++)
        for (int i = 0; i < m; i++) {
            size_t c = CI(S, i, j);
            S->u[c] = S->v[c] = S->ddev[c] = 0;
            S->p[c] = S->q[c] = S->s[c] = S->tau[c] = 0;
            S->X[c] = S->P.ax + i * S->dx;
            S->Y[c] = S->P.ay + j * S->dy;
        }
    memset(S->vel, 0, sizeof(v2) * (size_t)m * (n + 1));
    S->time = 0;
}

/* shear_sim::init_fields, shear_sim.cc:60-114: chi cases 0 (a Gaussian
 * blip at the origin), 1 (a line at 30 degrees, wrapped), 2 (sixteen blips
 * along a sine wave), evaluated at the cell centres of rows -1..n. */
void stzo_init_fields(stzo_sim *S, int chi_case, double tem_base, double tem_delta) {
    const double pi = 3.1415926535897932384626433832795;
    const int m = S->m, n = S->n;
    const double chi0 = tem_base / S->P.TZ, chi1 = tem_delta / S->P.TZ;
    double sx[16], sy[16];
    for (int k = 0; k < 16; k++) {
        sx[k] = S->P.ax + S->lx * (k + 0.5) * 0.0625;
        sy[k] = -0.2 * sin(pi * 0.0625 * (2 * k + 1));
    }
    rest_state(S);
    for (int j = -1; j <= n; j++) {
        const double ys = S->P.ay + j * S->dy + 0.5 * S->dy;
        for (int i = 0; i < m; i++) {
            const double xs = S->P.ax + i * S->dx + 0.5 * S->dx;
            double e;
            if (chi_case == 0) {
                e = xs * xs + ys * ys;
            } else if (chi_case == 1) {
                const double ca = cos(30 * pi / 180.), sa = sin(30 * pi / 180.);
                double xr = ca * xs + sa * ys, yr = -sa * xs + ca * ys;
                xr = xr < -1 ? xr + 1 : (xr > 1 ? xr - 1 : 0);
                e = xr * xr + yr * yr;
            } else {
                e = 1e100;
                for (int k = 0; k < 16; k++) {
                    double xr = sx[k] - xs, yr = sy[k] - ys;
                    if (xr < -S->lx * 0.5) xr += S->lx;
                    if (xr > S->lx * 0.5) xr -= S->lx;
                    double r2 = xr * xr + yr * yr;
                    if (r2 < e) e = r2;
                }
            }
            S->chi[CI(S, i, j)] = chi0 + chi1 * exp(-200 * e);
        }
    }
}

/* shear_sim::initialize_chi_bicubic, shear_sim.cc:832-909: chi of rows
 * 0..n-1 is lo + sca times the bicubic Hermite interpolant of arr (mm x nn,
 * periodic in x) with centred-difference derivatives (one-sided on the first
 * and last rows); the ghost rows get the linear extrapolation of
 * set_boundaries. */
void stzo_chi_bicubic(stzo_sim *S, int mm, int nn, const double *arr, double lo, double sca) {
    const int m = S->m, n = S->n;
    const size_t cnt = (size_t)mm * nn;
    double *ax = malloc(sizeof(double) * cnt), *ay = malloc(sizeof(double) * cnt),
           *axy = malloc(sizeof(double) * cnt);
    for (int j = 0; j < nn; j++)
        for (int i = 0; i < mm; i++) {
            const int ir = i == mm - 1 ? 0 : i + 1, il = i == 0 ? mm - 1 : i - 1;
            ax[(size_t)j * mm + i] = 0.5 * (arr[(size_t)j * mm + ir] - arr[(size_t)j * mm + il]);
        }
    for (int j = 0; j < nn; j++)
        for (int i = 0; i < mm; i++) {
            const size_t c = (size_t)j * mm + i;
            if (j == 0) {
                ay[c] = arr[c + mm] - arr[c];
                axy[c] = ax[c + mm] - ax[c];
            } else if (j == nn - 1) {
                ay[c] = arr[c] - arr[c - mm];
                axy[c] = ax[c] - ax[c - mm];
            } else {
                ay[c] = 0.5 * (arr[c + mm] - arr[c - mm]);
                axy[c] = 0.5 * (ax[c + mm] - ax[c - mm]);
            }
        }
    rest_state(S);
    const double xsca = S->dx * mm / (S->P.bx - S->P.ax), ysca = S->dy * nn / (S->P.by - S->P.ay);
    for (int j = 0; j < n; j++) {
        double y = (j + 0.5) * ysca - 0.5;
        int jj = (int)y;
        if (jj < 0) jj = 0;
        else if (jj > nn - 2) jj = nn - 2;
        y -= jj;
        const double my = 1 - y;
        /* Hermite basis in y: derivative at 0, value at 0, value at 1, derivative at 1 */
        const double hy0 = y * my * my, hy1 = my * my * (1 + 2 * y), hy2 = y * y * (3 - 2 * y), hy3 = -y * y * my;
        for (int i = 0; i < m; i++) {
            double x = (i + 0.5) * xsca - 0.5;
            if (x < 0) x += mm;
            int ii = (int)x;
            if (ii >= mm) ii -= mm;
            const size_t c0 = (size_t)jj * mm + ii, c1 = (size_t)jj * mm + (ii == mm - 1 ? 0 : ii + 1);
            x -= ii;
            const double mx = 1 - x;
            const double hx0 = x * mx * mx, hx1 = mx * mx * (1 + 2 * x), hx2 = x * x * (3 - 2 * x), hx3 = -x * x * mx;
            const double r0 = axy[c0] * hx0 + ay[c0] * hx1 + ay[c1] * hx2 + axy[c1] * hx3;
            const double r1 = ax[c0] * hx0 + arr[c0] * hx1 + arr[c1] * hx2 + ax[c1] * hx3;
            const double r2 = ax[c0 + mm] * hx0 + arr[c0 + mm] * hx1 + arr[c1 + mm] * hx2 + ax[c1 + mm] * hx3;
            const double r3 = axy[c0 + mm] * hx0 + ay[c0 + mm] * hx1 + ay[c1 + mm] * hx2 + axy[c1 + mm] * hx3;
            S->chi[CI(S, i, j)] = lo + sca * (hy0 * r0 + hy1 * r1 + hy2 * r2 + hy3 * r3);
        }
    }
    for (int i = 0; i < m; i++) {
        S->chi[CI(S, i, -1)] = 2 * S->chi[CI(S, i, 0)] - S->chi[CI(S, i, 1)];
        S->chi[CI(S, i, n)] = 2 * S->chi[CI(S, i, n - 1)] - S->chi[CI(S, i, n - 2)];
    }
    free(ax); free(ay); free(axy);
}

/* shear_sim::l2_comparison, shear_sim.cc:460-502: dx dy times the sums of
 * squared differences of (u, v) and (X, Y) over node rows 0..n with weight
 * 1/2 on rows 0 and n, of the stresses (2 tau^2 + 2 s^2 + 3 p^2 + 6 q^2) and
 * of chi over the cells. */
void stzo_l2_comparison(stzo_sim *A, stzo_sim *B, double *l2) {
    const int m = A->m, n = A->n;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int j = 0; j <= n; j++) {
        double c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        for (int i = 0; i < m; i++) {
            const size_t c = CI(A, i, j);
            const double du = A->u[c] - B->u[c], dv = A->v[c] - B->v[c];
            const double dX = A->X[c] - B->X[c], dY = A->Y[c] - B->Y[c];
            c0 += du * du + dv * dv;
            c3 += dX * dX + dY * dY;
            if (j < n) {
                const double dp = A->p[c] - B->p[c], dq = A->q[c] - B->q[c], ds = A->s[c] - B->s[c],
                             dt = A->tau[c] - B->tau[c], dc = A->chi[c] - B->chi[c];
                c1 += 2 * (dt * dt + ds * ds) + 3 * dp * dp + 6 * dq * dq;
                c2 += dc * dc;
            }
        }
        const double w = (j == 0 || j == n) ? 0.5 : 1.0;
        a0 += w * c0;
        a3 += w * c3;
        a1 += c1;
        a2 += c2;
    }
    const double fac = A->dx * A->dy;
    l2[0] = a0 * fac;
    l2[1] = a1 * fac;
    l2[2] = a2 * fac;
    l2[3] = a3 * fac;
}

void stzo_set_tolerance(stzo_sim *S, int mode, double value) {
    S->tol_mode = mode;
    if (mode == 0) {
        /* tgmg_accuracy, tgmg.hh:41-45 */
        double a = DBL_EPSILON * value * (2 * (S->tmufac1 + S->tmufac2));
        S->acc = a * a;
    } else {
        S->rtol = value;
    }
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* step_forward_quasistatic, shear_sim.cc:280-291 */
long stzo_steps(stzo_sim *S, double dt, int nsteps, double *eps_pl, double *seconds) {
    long c0 = S->vcount;
    double t = 0;
    for (int k = 0; k < nsteps; k++) {
        double a = now_s();
        S->time += dt;
        advection_step(S, dt);
        if (!projection_step(S, dt)) { if (seconds) *seconds = t; return -1; }
        t += now_s() - a;
        if (eps_pl)
            for (int j = 0; j < S->n; j++)
                for (int i = 0; i < S->m; i++)
                    eps_pl[(size_t)j * S->m + i] += S->ddev[CI(S, i, j)] / (2 * S->P.mu);
    }
    if (seconds) *seconds = t;
    return S->vcount - c0;
}

/* shear_sim::step_forward, shear_sim.cc:185-276, nsteps times; eps_pl
 * accumulates the raw stress drop / (2 mu) */
void stzo_steps_direct(stzo_sim *S, double dt, int nsteps, double *eps_pl) {
    const size_t mn = (size_t)S->m * S->n;
    double *raw = eps_pl ? (double *)malloc(mn * sizeof(double)) : NULL;
    for (int k = 0; k < nsteps; k++) {
        S->time += dt;
        direct_step(S, dt, raw);
        set_boundaries(S);
        if (eps_pl)
            for (size_t c = 0; c < mn; c++) eps_pl[c] += raw[c] / (2 * S->P.mu);
    }
    free(raw);
}

/* The frame loop of shear_sim::solve (shear_sim.cc:120-140) without output:
 * steps of dt while they stay short of target (relative margin 1e-8), then
 * one step of the remaining time.  Returns the number of steps. */
long stzo_advance_direct(stzo_sim *S, double dt, double target, double *eps_pl) {
    long k = 0;
    while (S->time + dt * (1 + 1e-8) < target) {
        stzo_steps_direct(S, dt, 1, eps_pl);
        k++;
    }
    stzo_steps_direct(S, target - S->time, 1, eps_pl);
    return k + 1;
}

double stzo_time(stzo_sim *S) { return S->time; }

void stzo_get(stzo_sim *S, int field, double *out) {
    const int m = S->m, n = S->n;
    const double *src;
    int node = field == 0 || field == 1 || field == 7 || field == 8;
    switch (field) {
        case 0: src = S->u; break; case 1: src = S->v; break; case 2: src = S->p; break;
        case 3: src = S->q; break; case 4: src = S->s; break; case 5: src = S->tau; break;
        case 6: src = S->chi; break; case 7: src = S->X; break; case 8: src = S->Y; break;
        default: src = S->ddev; break;
    }
    if (node) memcpy(out, src + CI(S, 0, 0), sizeof(double) * (size_t)m * (n + 1));
    else memcpy(out, src, sizeof(double) * (size_t)m * (n + 2));
}

/* Overwrites a stored field (ids of stzo_get; not u, v): cell fields
 * with their ghost rows, X and Y on node rows 0..n.  Used to start both
 * sides of a parity run from the same prepared state. */
void stzo_set(stzo_sim *S, int field, const double *in) {
    const int m = S->m, n = S->n;
    double *dst;
    switch (field) {
        case 2: dst = S->p; break; case 3: dst = S->q; break; case 4: dst = S->s; break;
        case 5: dst = S->tau; break; case 6: dst = S->chi; break; case 7: dst = S->X; break;
        case 8: dst = S->Y; break; case 9: dst = S->ddev; break;
        default: return;
    }
    if (field == 7 || field == 8) memcpy(dst + CI(S, 0, 0), in, sizeof(double) * (size_t)m * (n + 1));
    else memcpy(dst, in, sizeof(double) * (size_t)m * (n + 2));
}

void stzo_get_vel(stzo_sim *S, double *out) {
    memcpy(out, S->vel, sizeof(v2) * (size_t)S->m * (S->n + 1));
}

int stzo_mg_levels(stzo_sim *S, double dt, int *dims) {
    qs_init(S, S->P.viscosity / dt);
    for (int l = 1; l < S->nl; l++) { dims[2 * (l - 1)] = S->lv[l].m; dims[2 * (l - 1) + 1] = S->lv[l].n; }
    return S->nl - 1;
}

void stzo_mg_stencil(stzo_sim *S, int l, double *out) {
    memcpy(out, S->lv[l + 1].st, sizeof(m2) * 10 * (size_t)S->lv[l + 1].mn);
}

int stzo_mg_solve(stzo_sim *S, double dt, const double *src, double *vel, int *ncycles) {
    qs_init(S, S->P.viscosity / dt);
    size_t mn = (size_t)S->m * (S->n + 1);
    memcpy(S->src, src, sizeof(v2) * mn);
    memcpy(S->vel, vel, sizeof(v2) * mn);
    long c0 = S->vcount;
    int ok = solve_adaptive(S);
    if (ncycles) *ncycles = (int)(S->vcount - c0);
    memcpy(vel, S->vel, sizeof(v2) * mn);
    return ok;
}

void stzo_mg_vcycle(stzo_sim *S, double dt, const double *src, double *vel) {
    qs_init(S, S->P.viscosity / dt);
    size_t mn = (size_t)S->m * (S->n + 1);
    memcpy(S->src, src, sizeof(v2) * mn);
    memcpy(S->vel, vel, sizeof(v2) * mn);
    v_cycle(S);
    memcpy(vel, S->vel, sizeof(v2) * mn);
}

double stzo_mg_l2_error(stzo_sim *S) { return mds(S, 0) / S->lv[0].mn; }

/* Sum of squared residuals of the quasi-static system (mds, tgmg.in.cc:55-64)
 * for the given source and velocity, and the sum of squared sources. */
void stzo_mg_residual_sqnorms(stzo_sim *S, double dt, const double *src, const double *vel, double *out) {
    qs_init(S, S->P.viscosity / dt);
    size_t mn = (size_t)S->m * (S->n + 1);
    memcpy(S->src, src, sizeof(v2) * mn);
    memcpy(S->vel, vel, sizeof(v2) * mn);
    out[0] = mds(S, 0);
    double b2 = 0;
    for (size_t k = 0; k < 2 * mn; k++) b2 += src[k] * src[k];
    out[1] = b2;
}

/* ---------------------------------------------------------------------- */
/* Random chi (initialize_random, shear_sim.cc:915-998).  The reference draws
 * its white noise from libc rand(); here every noise point draws from its own
 * splitmix64 stream keyed by (seed, index), then the polar Box-Muller method
 * as box_muller (shear_sim.cc:988-998).  The truncated Gaussian smoothing and
 * its normalisation follow gaussian_normal_factor (shear_sim.cc:915-925);
 * the 2D kernel is applied as two 1D passes. */

static unsigned long long splitmix64(unsigned long long *st) {
    unsigned long long z = (*st += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double unit_draw(unsigned long long *st) { return (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0); }
static double noise_at(unsigned long long seed, unsigned long long idx) {
    unsigned long long st = seed * 0xD1342543DE82EF95ULL + idx * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
    double x, y, r;
    do {
        x = 2 * unit_draw(&st) - 1;
        y = 2 * unit_draw(&st) - 1;
        r = x * x + y * y;
    } while (r == 0.0 || r > 1.0);
    return x * sqrt(-2.0 * log(r) / r);
}

void stzo_random_chi(int m, int n, double l, double tem_avg, double tem_std, double TZ,
                     unsigned long long seed, double *out) {
    int cut = (int)(l * 5.), nx = n + 2 * cut;
    double llinv = 0.5 / (l * l);
    double vfac = 1;
    for (int j = 1; j < cut; j++) {
        double q = exp(-j * j * llinv);
        for (int k = 0; k <= j; k++) {
            double q2 = q * exp(-k * k * llinv);
            vfac += (k == 0 || k == j ? 4 : 8) * q2 * q2;
        }
    }
    double chi0 = tem_avg / TZ, chi1 = tem_std / (sqrt(vfac) * TZ);
    double *g = (double *)malloc(sizeof(double) * (2 * cut + 1));
    for (int d = -cut; d <= cut; d++) g[d + cut] = exp(-llinv * d * d);
    double *noise = (double *)malloc(sizeof(double) * (size_t)m * nx);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)m * nx);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nx; r++)
        for (int i = 0; i < m; i++) noise[(size_t)r * m + i] = noise_at(seed, (unsigned long long)r * m + i);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nx; r++)
        for (int i = 0; i < m; i++) {
            double a = 0;
            for (int d = -cut; d <= cut; d++) {
                int ii = ((i + d) % m + m) % m;
                a += noise[(size_t)r * m + ii] * g[d + cut];
            }
            tmp[(size_t)r * m + i] = a;
        }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double a = 0;
            for (int d = -cut; d <= cut; d++) a += tmp[(size_t)(j + cut + d) * m + i] * g[d + cut];
            out[(size_t)j * m + i] = chi0 + a * chi1;
        }
    free(g); free(noise); free(tmp);
}

int stzo_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Threads of the following parallel regions (the CPU baseline's
 * one-thread figure). */
void stzo_set_threads(int k) {
#ifdef _OPENMP
    omp_set_num_threads(k > 0 ? k : 1);
#else
    (void)k;
#endif
}
