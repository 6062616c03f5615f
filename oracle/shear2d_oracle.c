/*
 * shear2d_oracle.c -- CPU restatement of the reference's case1 particle step:
 * circles carried through a shear flow between two moving walls, periodic in
 * x (MPI/Micro_particles/fortran/case1/mpi_complete), FP64.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  One rank of the
 * MPI code with its compile-time variants as flags: stationaryFrame or
 * movingFrame, quadratic or linear interpolated bounce-back and refill.  Each
 * routine cites the subroutine it restates; statement and expression order are
 * kept, so with -ffp-contract=off the results equal the reference's statements
 * bit for bit (pinned by tests/golden/shear2d_*.npz, which execute them).
 *
 * Periodic x: the reference reads x-neighbours outside 1..nx from ghost
 * columns that its MPI exchanges fill with the periodic partner's values
 * (message_particle.F90); here such reads wrap around.  The solid mask keeps
 * the reference's plain circle test on its ghost columns 0 and nx+1 (no
 * periodic images), so, as in the reference, circles are meant to stay clear
 * of the periodic boundary.
 *
 * Layout, as the reference's arrays (freeall.F90:1-19):
 *   f(0:8, -2:nx+3, -2:ny+3), f_post(0:8, -1:nx+2, -1:ny+2),
 *   obst(0:nx+1, 0:ny+1), rho/u/v(1:nx, 1:ny), x fastest.
 */
#include "lbm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const int sx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int sy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int sr[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6}; /* commondata.F90:46-50 (r(0) unused) */

struct orc_shear {
    orc_shear_params p;
    double snu, sq;
    double w[9];
    double *f, *fp, *rho, *u, *v;
    int *ob, *obn;
    double *xc, *yc, *xco, *yco, *uc, *vc, *uco, *vco, *om, *omo, *fx, *fy, *tq;
    double rho_avg;
    long long itc;
};

#define NX (s->p.nx)
#define NY (s->p.ny)
static int wx(const orc_shear* s, int i) { return i < 1 ? i + NX : (i > NX ? i - NX : i); }
static double* Fa(orc_shear* s, int a, int i, int j) {
    i = wx(s, i);
    return &s->f[a + 9 * ((size_t)(i + 2) + (size_t)(NX + 6) * (size_t)(j + 2))];
}
static double* FPa(orc_shear* s, int a, int i, int j) {
    i = wx(s, i);
    return &s->fp[a + 9 * ((size_t)(i + 1) + (size_t)(NX + 4) * (size_t)(j + 1))];
}
#define F(a, i, j) (*Fa(s, a, i, j))
#define FP(a, i, j) (*FPa(s, a, i, j))
#define OB(i, j) s->ob[(size_t)(i) + (size_t)(NX + 2) * (size_t)(j)]
#define OBN(i, j) s->obn[(size_t)(i) + (size_t)(NX + 2) * (size_t)(j)]
#define S(arr, i, j) s->arr[(size_t)((i) - 1) + (size_t)NX * (size_t)((j) - 1)]

/* x**2.0d0: gfortran evaluates a real power of 2 as one product */
static double p2(double x) { return x * x; }

/* the circle test of initial.F90:79-82, particle_bounceback.F90:53-55,
 * particle_force.F90:40-42 and particle_update.F90:43-45 */
static int in_circle(const orc_shear* s, double x, double y, double xc, double yc) {
    return (p2(x - xc) + p2(y - yc)) <= p2(s->p.radius);
}

orc_shear* orc_shear_create(const orc_shear_params* p, const double* centers) {
    orc_shear* s = (orc_shear*)calloc(1, sizeof *s);
    s->p = *p;
    s->snu = 1.0 / p->tauf; /* commondata.F90:32 */
    s->sq = 8.0 * (2.0 * p->tauf - 1.0) / (8.0 * p->tauf - 1.0);
    s->w[0] = 4.0 / 9.0;
    for (int a = 1; a <= 4; a++) s->w[a] = 1.0 / 9.0;
    for (int a = 5; a <= 8; a++) s->w[a] = 1.0 / 36.0;
    const size_t nf = 9 * (size_t)(p->nx + 6) * (p->ny + 6), nfp = 9 * (size_t)(p->nx + 4) * (p->ny + 4);
    const size_t nc = (size_t)p->nx * p->ny, no = (size_t)(p->nx + 2) * (p->ny + 2);
    s->f = (double*)calloc(nf, 8);
    s->fp = (double*)calloc(nfp, 8);
    s->rho = (double*)calloc(nc, 8);
    s->u = (double*)calloc(nc, 8);
    s->v = (double*)calloc(nc, 8);
    s->ob = (int*)calloc(no, sizeof(int));
    s->obn = (int*)calloc(no, sizeof(int));
    double** arrs[] = {&s->xc, &s->yc, &s->xco, &s->yco, &s->uc, &s->vc, &s->uco,
                       &s->vco, &s->om, &s->omo, &s->fx, &s->fy, &s->tq};
    for (int q = 0; q < 13; q++) *arrs[q] = (double*)calloc(p->np > 0 ? p->np : 1, 8);
    /* initial.F90:37-155 */
    for (int c = 0; c < p->np; c++) {
        s->xc[c] = centers[2 * c];
        s->yc[c] = centers[2 * c + 1];
        s->uc[c] = p->moving_frame ? 0.0 : p->u0;
        s->vc[c] = 0.0;
        s->om[c] = 0.0;
    }
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) S(rho, i, j) = p->rho0;
    for (int j = 0; j <= NY + 1; j++)
        for (int i = 0; i <= NX + 1; i++)
            for (int c = 0; c < p->np; c++)
                if (in_circle(s, (double)i, (double)j, s->xc[c], s->yc[c])) OB(i, j) = 1;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            if (OB(i, j) == 1) S(rho, i, j) = p->rho_solid;
    const double ub = p->moving_frame ? -p->uwall - p->u0 : -p->uwall;
    const double ut = p->moving_frame ? p->uwall - p->u0 : p->uwall;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            S(u, i, j) = p->moving_frame ? 0.0 : p->u0;
            S(v, i, j) = 0.0;
        }
    for (int i = 1; i <= NX; i++) {
        S(u, i, 1) = ub;
        S(u, i, NY) = ut;
    }
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            if (OB(i, j) == 0) {
                const double uu = S(u, i, j), vv = S(v, i, j);
                const double us2 = uu * uu + vv * vv;
                for (int a = 0; a < 9; a++) {
                    const double un = uu * sx[a] + vv * sy[a];
                    F(a, i, j) = s->w[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
                }
            }
    return s;
}

void orc_shear_destroy(orc_shear* s) {
    if (!s) return;
    void* ps[] = {s->f, s->fp, s->rho, s->u, s->v, s->ob, s->obn, s->xc, s->yc, s->xco, s->yco,
                  s->uc, s->vc, s->uco, s->vco, s->om, s->omo, s->fx, s->fy, s->tq};
    for (size_t q = 0; q < sizeof ps / sizeof ps[0]; q++) free(ps[q]);
    free(s);
}

/* fluid.F90:1-72 (collision), fluid nodes only */
static void collision(orc_shear* s) {
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            if (OB(i, j) != 0) continue;
            double f[9], m[9], meq[9], sv[9], mp[9];
            for (int a = 0; a < 9; a++) f[a] = F(a, i, j);
            m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
            m[1] = -4.0 * f[0] - f[1] - f[2] - f[3] - f[4] + 2.0 * (f[5] + f[6] + f[7] + f[8]);
            m[2] = 4.0 * f[0] - 2.0 * (f[1] + f[2] + f[3] + f[4]) + f[5] + f[6] + f[7] + f[8];
            m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
            m[4] = -2.0 * f[1] + 2.0 * f[3] + f[5] - f[6] - f[7] + f[8];
            m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
            m[6] = -2.0 * f[2] + 2.0 * f[4] + f[5] + f[6] - f[7] - f[8];
            m[7] = f[1] - f[2] + f[3] - f[4];
            m[8] = f[5] - f[6] + f[7] - f[8];
            const double r = S(rho, i, j), uu = S(u, i, j), vv = S(v, i, j);
            meq[0] = r;
            meq[1] = r * (-2.0 + 3.0 * (uu * uu + vv * vv));
            meq[2] = r * (1.0 - 3.0 * (uu * uu + vv * vv));
            meq[3] = r * uu;
            meq[4] = -r * uu;
            meq[5] = r * vv;
            meq[6] = -r * vv;
            meq[7] = r * (uu * uu - vv * vv);
            meq[8] = r * (uu * vv);
            sv[0] = 0.0; sv[1] = s->snu; sv[2] = s->snu; sv[3] = 0.0; sv[4] = s->sq;
            sv[5] = 0.0; sv[6] = s->sq; sv[7] = s->snu; sv[8] = s->snu;
            for (int a = 0; a < 9; a++) mp[a] = m[a] - sv[a] * (m[a] - meq[a]);
            FP(0, i, j) = (mp[0] - mp[1] + mp[2]) / 9.0;
            FP(1, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[3] / 6.0 - mp[4] / 6.0 + mp[7] * 0.25;
            FP(2, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[5] / 6.0 - mp[6] / 6.0 - mp[7] * 0.25;
            FP(3, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[3] / 6.0 + mp[4] / 6.0 + mp[7] * 0.25;
            FP(4, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[5] / 6.0 + mp[6] / 6.0 - mp[7] * 0.25;
            FP(5, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 +
                          mp[5] / 6.0 + mp[6] / 12.0 + mp[8] * 0.25;
            FP(6, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 +
                          mp[5] / 6.0 + mp[6] / 12.0 - mp[8] * 0.25;
            FP(7, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 -
                          mp[5] / 6.0 - mp[6] / 12.0 + mp[8] * 0.25;
            FP(8, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 -
                          mp[5] / 6.0 - mp[6] / 12.0 - mp[8] * 0.25;
        }
}

/* fluid.F90:75-119 (streaming): pull from fluid sources, x wrapped */
static void streaming(orc_shear* s) {
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            for (int a = 0; a < 9; a++) {
                int ip = i - sx[a];
                const int jp = j - sy[a];
                if (ip == 0) ip = NX;
                if (ip == NX + 1) ip = 1;
                if (OB(ip, jp) == 0) F(a, i, j) = FP(a, ip, jp);
            }
}

/* fluid.F90:122-172 (bounceback): the two moving walls */
static void bounceback(orc_shear* s) {
    const orc_shear_params* p = &s->p;
    for (int i = 1; i <= NX; i++) {
        F(2, i, 1) = FP(4, i, 1);
        if (p->moving_frame) {
            F(5, i, 1) = FP(7, i, 1) + (-p->uwall - p->u0) / 6.0;
            F(6, i, 1) = FP(8, i, 1) - (-p->uwall - p->u0) / 6.0;
        } else {
            F(5, i, 1) = FP(7, i, 1) + (-p->uwall) / 6.0;
            F(6, i, 1) = FP(8, i, 1) - (-p->uwall) / 6.0;
        }
    }
    for (int i = 1; i <= NX; i++) {
        F(4, i, NY) = FP(2, i, NY);
        if (p->moving_frame) {
            F(7, i, NY) = FP(5, i, NY) - (p->uwall - p->u0) / 6.0;
            F(8, i, NY) = FP(6, i, NY) + (p->uwall - p->u0) / 6.0;
        } else {
            F(7, i, NY) = FP(5, i, NY) - (p->uwall) / 6.0;
            F(8, i, NY) = FP(6, i, NY) + (p->uwall) / 6.0;
        }
    }
}

/* particle_bounceback.F90:115-155 (calQ, bisection); 0 = ok */
static int calq(const orc_shear* s, int c, double i, double j, int a, double* x0, double* y0,
                double* q) {
    const double epsR = (double)1e-9f; /* default-real literal (:123) */
    double qq = 0.5, qt = 0.5;
    double px = i + qt * (double)sx[a], py = j + qt * (double)sy[a];
    const double xc = s->xc[c], yc = s->yc[c], R = s->p.radius;
    int guard = 0;
    while (fabs(sqrt(p2(px - xc) + p2(py - yc)) - R) >= epsR) {
        if (++guard > 200) return 2;
        if (sqrt(p2(px - xc) + p2(py - yc)) > R) {
            qt = qt / 2.0;
            px = px + qt * (double)sx[a];
            py = py + qt * (double)sy[a];
            qq = qq + qt;
        } else if (sqrt(p2(px - xc) + p2(py - yc)) < R) {
            qt = qt / 2.0;
            px = px - qt * (double)sx[a];
            py = py - qt * (double)sy[a];
            qq = qq - qt;
        } else {
            return 2;
        }
    }
    if (qq > 1.0 || qq < 0.0) return 2;
    *x0 = px;
    *y0 = py;
    *q = qq;
    return 0;
}

/* fluid average of rho over mask (particle_bounceback.F90:15-35,
 * particle_update.F90:72-87) */
static double rho_average(orc_shear* s, const int* mask) {
    double acc = 0.0;
    int n = 0;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            if (mask[(size_t)i + (size_t)(NX + 2) * j] == 0) {
                acc = acc + S(rho, i, j);
                n = n + 1;
            }
    return acc / (double)n;
}

/* particle_bounceback.F90:1-111; returns 0, 1 (no owner) or 2 (q) */
static int bounceback_particle(orc_shear* s) {
    s->rho_avg = rho_average(s, s->ob);
    const double ra = s->rho_avg;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            if (OB(i, j) != 0) continue;
            for (int a = 0; a < 9; a++) {
                const int ip = i + sx[a], jp = j + sy[a];
                if (OB(ip, jp) != 1) continue;
                int flag = 0;
                for (int c = 0; c < s->p.np; c++) {
                    if (!in_circle(s, (double)ip, (double)jp, s->xc[c], s->yc[c])) continue;
                    flag = 1;
                    double x0, y0, q;
                    if (calq(s, c, (double)i, (double)j, a, &x0, &y0, &q)) return 2;
                    const double t1 = -(y0 - s->yc[c]) * s->om[c];
                    const double t2 = (x0 - s->xc[c]) * s->om[c];
                    const int r = sr[a];
                    const double eu = sx[r] * (s->uc[c] + t1) + sy[r] * (s->vc[c] + t2);
                    if (s->p.linear) {
                        if (q < 0.5) {
                            F(r, i, j) = 2.0 * q * FP(a, i, j) + (1.0 - 2.0 * q) * FP(a, i - sx[a], j - sy[a]) +
                                         6.0 * s->w[a] * ra * eu;
                        } else if (q >= 0.5) {
                            F(r, i, j) = 0.5 / q * FP(a, i, j) + (1.0 - 0.50 / q) * FP(r, i, j) +
                                         3.0 * s->w[a] * ra / q * eu;
                        }
                    } else {
                        if (q < 0.5) {
                            F(r, i, j) = q * (1.0 + 2.0 * q) * FP(a, i, j) +
                                         (1.0 - 4.0 * q * q) * FP(a, i - sx[a], j - sy[a]) -
                                         q * (1.0 - 2.0 * q) * FP(a, i - 2 * sx[a], j - 2 * sy[a]) +
                                         6.0 * s->w[a] * ra * eu;
                        } else if (q >= 0.5) {
                            F(r, i, j) = FP(a, i, j) / q / (1.0 + 2.0 * q) + FP(r, i, j) * (2.0 * q - 1.0) / q -
                                         FP(r, i - sx[a], j - sy[a]) * (2.0 * q - 1.0) / (2.0 * q + 1.0) +
                                         6.0 * s->w[a] * ra / q / (1.0 + 2.0 * q) * eu;
                        }
                    }
                }
                if (!flag) return 1;
            }
        }
    return 0;
}

/* fluid.F90:175-193 (macro) */
static void macro(orc_shear* s) {
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            if (OB(i, j) != 0) continue;
            double g[9];
            for (int a = 0; a < 9; a++) g[a] = F(a, i, j);
            const double r = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8];
            S(rho, i, j) = r;
            S(u, i, j) = (g[1] - g[3] + g[5] - g[6] - g[7] + g[8]) / r;
            S(v, i, j) = (g[2] - g[4] + g[5] + g[6] - g[7] - g[8]) / r;
        }
}

/* particle_force.F90:1-104 (calForce): momentum exchange only */
static int cal_force(orc_shear* s) {
    const int np = s->p.np;
    for (int c = 0; c < np; c++) {
        s->fx[c] = 0.0;
        s->fy[c] = 0.0;
        s->tq[c] = 0.0;
    }
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            if (OB(i, j) != 0) continue;
            for (int a = 1; a < 9; a++) {
                const int ip = i + sx[a], jp = j + sy[a];
                if (OB(ip, jp) != 1) continue;
                int flag = 0;
                for (int c = 0; c < np; c++) {
                    if (!in_circle(s, (double)ip, (double)jp, s->xc[c], s->yc[c])) continue;
                    flag = 1;
                    double x0, y0, q;
                    if (calq(s, c, (double)i, (double)j, a, &x0, &y0, &q)) return 2;
                    const double t1 = -(y0 - s->yc[c]) * s->om[c];
                    const double t2 = (x0 - s->xc[c]) * s->om[c];
                    const int r = sr[a];
                    const double tfx = (sx[a] - s->uc[c] - t1) * FP(a, i, j) - (sx[r] - s->uc[c] - t1) * F(r, i, j);
                    const double tfy = (sy[a] - s->vc[c] - t2) * FP(a, i, j) - (sy[r] - s->vc[c] - t2) * F(r, i, j);
                    const double tt = (x0 - s->xc[c]) * tfy - (y0 - s->yc[c]) * tfx;
                    s->fx[c] = s->fx[c] + tfx;
                    s->fy[c] = s->fy[c] + tfy;
                    s->tq[c] = s->tq[c] + tt;
                }
                if (!flag) return 1;
            }
        }
    for (int c = 0; c < np; c++) { /* :93-101 */
        s->xco[c] = s->xc[c];
        s->yco[c] = s->yc[c];
        s->uco[c] = s->uc[c];
        s->vco[c] = s->vc[c];
        s->omo[c] = s->om[c];
    }
    return 0;
}

/* particle_update.F90:1-174 (updateCenter): prescribed motion, mask, refill;
 * returns 0, 1 (no owner) or 5 (no refill direction) */
static int update_center(orc_shear* s) {
    const orc_shear_params* p = &s->p;
    for (int c = 0; c < p->np; c++) {
        s->uc[c] = p->moving_frame ? 0.0 : p->u0;
        s->vc[c] = 0.0;
        s->om[c] = 0.0;
        s->xc[c] = s->xco[c] + s->uco[c];
        s->yc[c] = s->yco[c] + s->vco[c];
    }
    for (int j = 0; j <= NY + 1; j++)
        for (int i = 0; i <= NX + 1; i++) {
            OBN(i, j) = 0;
            for (int c = 0; c < p->np; c++)
                if (in_circle(s, (double)i, (double)j, s->xc[c], s->yc[c])) OBN(i, j) = 1;
        }
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            if (OBN(i, j) == 1) {
                S(rho, i, j) = p->rho_solid;
                S(u, i, j) = 0.0;
                S(v, i, j) = 0.0;
            }
    s->rho_avg = rho_average(s, s->obn);
    const double ra = s->rho_avg;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            if (!(OB(i, j) == 1 && OBN(i, j) == 0)) continue;
            int flag = 0;
            for (int c = 0; c < p->np; c++) {
                if (!in_circle(s, (double)i, (double)j, s->xco[c], s->yco[c])) continue;
                flag = 1;
                double out = 0.0;
                int ec = 0;
                for (int a = 1; a < 9; a++) {
                    const double t = ((i - s->xc[c]) * sx[a] + (j - s->yc[c]) * sy[a]) /
                                     sqrt(p2(i - s->xc[c]) + p2(j - s->yc[c]));
                    if (t > out) {
                        out = t;
                        ec = a;
                    }
                }
                if (ec == 0) return 5;
                const int e0 = sx[ec], e1 = sy[ec];
                for (int a = 0; a < 9; a++) {
                    if (p->linear)
                        F(a, i, j) = 2.0 * F(a, i + e0, j + e1) - F(a, i + 2 * e0, j + 2 * e1);
                    else
                        F(a, i, j) = 3.0 * F(a, i + e0, j + e1) - 3.0 * F(a, i + 2 * e0, j + 2 * e1) +
                                     F(a, i + 3 * e0, j + 3 * e1);
                }
                double G[9], m[9];
                for (int a = 0; a < 9; a++) G[a] = F(a, i, j);
                m[0] = G[0] + G[1] + G[2] + G[3] + G[4] + G[5] + G[6] + G[7] + G[8];
                m[1] = -4.0 * G[0] - G[1] - G[2] - G[3] - G[4] + 2.0 * G[5] + 2.0 * G[6] + 2.0 * G[7] +
                       2.0 * G[8];
                m[2] = 4.0 * G[0] - 2.0 * G[1] - 2.0 * G[2] - 2.0 * G[3] - 2.0 * G[4] + G[5] + G[6] +
                       G[7] + G[8];
                m[3] = ra * s->uc[0]; /* Uc(1): the first circle, as written (:130) */
                m[4] = -2.0 * G[1] + 2.0 * G[3] + G[5] - G[6] - G[7] + G[8];
                m[5] = ra * s->vc[0];
                m[6] = -2.0 * G[2] + 2.0 * G[4] + G[5] + G[6] - G[7] - G[8];
                m[7] = G[1] - G[2] + G[3] - G[4];
                m[8] = G[5] - G[6] + G[7] - G[8];
                G[0] = (m[0] - m[1] + m[2]) / 9.0;
                G[1] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[3] / 6.0 - m[4] / 6.0 + m[7] * 0.25;
                G[2] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[5] / 6.0 - m[6] / 6.0 - m[7] * 0.25;
                G[3] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[3] / 6.0 + m[4] / 6.0 + m[7] * 0.25;
                G[4] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[5] / 6.0 + m[6] / 6.0 - m[7] * 0.25;
                G[5] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 + m[5] / 6.0 +
                       m[6] / 12.0 + m[8] * 0.25;
                G[6] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 + m[5] / 6.0 +
                       m[6] / 12.0 - m[8] * 0.25;
                G[7] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 - m[5] / 6.0 -
                       m[6] / 12.0 + m[8] * 0.25;
                G[8] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 - m[5] / 6.0 -
                       m[6] / 12.0 - m[8] * 0.25;
                for (int a = 0; a < 9; a++) F(a, i, j) = G[a];
                const double r = G[0] + G[1] + G[2] + G[3] + G[4] + G[5] + G[6] + G[7] + G[8];
                S(rho, i, j) = r;
                S(u, i, j) = (G[1] - G[3] + G[5] - G[6] - G[7] + G[8]) / r;
                S(v, i, j) = (G[2] - G[4] + G[5] + G[6] - G[7] - G[8]) / r;
            }
            if (!flag) return 1;
        }
    memcpy(s->ob, s->obn, sizeof(int) * (size_t)(NX + 2) * (NY + 2));
    return 0;
}

/* main.F90:34-67: collision, (exchange), streaming, bounceback, (exchange),
 * bounceback_particle, macro, calForce, (exchange), updateCenter */
int orc_shear_step(orc_shear* s, int nsteps) {
    for (int n = 0; n < nsteps; n++) {
        int rc;
        collision(s);
        streaming(s);
        bounceback(s);
        if ((rc = bounceback_particle(s))) return rc;
        macro(s);
        if ((rc = cal_force(s))) return rc;
        s->itc++;
        if ((rc = update_center(s))) return rc;
    }
    return 0;
}

void orc_shear_get(const orc_shear* s, double* f, double* rho, double* u, double* v, int* obst,
                   double* xc, double* uc, double* force, double* torque, double* rho_avg) {
    orc_shear* t = (orc_shear*)s;
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            const size_t q = (size_t)(i - 1) + (size_t)NX * (j - 1);
            for (int a = 0; a < 9; a++) f[9 * q + a] = *Fa(t, a, i, j);
            rho[q] = s->rho[q];
            u[q] = s->u[q];
            v[q] = s->v[q];
            obst[q] = s->ob[(size_t)i + (size_t)(NX + 2) * j];
        }
    for (int c = 0; c < s->p.np; c++) {
        xc[2 * c] = s->xc[c];
        xc[2 * c + 1] = s->yc[c];
        uc[2 * c] = s->uc[c];
        uc[2 * c + 1] = s->vc[c];
        force[2 * c] = s->fx[c];
        force[2 * c + 1] = s->fy[c];
        torque[c] = s->tq[c];
    }
    *rho_avg = s->rho_avg;
}
