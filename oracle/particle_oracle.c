/*
 * particle_oracle.c -- CPU restatement of MGLC's moving-particle step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA particle path).
 *
 * dim = 2: a literal restatement of MPI/Micro_particles/fortran/case4/
 *          mpi_particle (D2Q9 MRT, circular particles, quadratic
 *          interpolated bounce-back, Wen 2014 momentum exchange, springs,
 *          explicit update, refill), single rank, in the order of
 *          main.F90:35-73.  Pinned against fixtures executed from the
 *          reference's own statements (tests/golden/gen_golden.py).
 * dim = 3: the same algorithm generalised to D3Q19 and spheres (the
 *          reference has no 3-D particle code): the D3Q19 forced MRT of
 *          bouyancy3d_mpi.F90:641-864 with a constant body force, periodic x
 *          (case1 pattern), no-slip y/z walls, torque r x F, I = 2/5 M R^2.
 *
 * Arrays carry 3 ghost layers per spatial axis, Fortran 1-based cell
 * coordinates (node i sits at x = i, as on one rank where
 * i_start_global = 0).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "lbm_oracle.h"

#define PI_ (4.0 * atan(1.0))

static const int ex9[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int ey9[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int r9[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
static const int ex19[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int ey19[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int ez19[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int r19[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

struct orc_particles {
    orc_pp p;
    int Q, X, Y, Z; /* padded extents */
    const int *ex, *ey, *ez, *r;
    int ez0[9];
    double omega[19];
    double snu, sq;
    double *f, *fp;
    int *obst, *obst_new;
    double *rho, *u, *v, *w, *up, *vp, *wp;
    double *xc, *uc, *om;          /* np*3 */
    double *xc_old, *uc_old, *om_old;
    double *force, *torque;        /* np*3: wallTotalForce, totalTorque */
    double *radius;                /* np */
    double rho_avg;
    long itc;
};

static size_t IX(const orc_particles* s, int i, int j, int k) {
    if (s->p.periodic_x) {
        while (i < 1) i += s->p.nx;
        while (i > s->p.nx) i -= s->p.nx;
    }
    return (size_t)(i + 2) + (size_t)s->X * ((size_t)(j + 2) + (size_t)s->Y * (size_t)(s->p.dim == 3 ? k + 2 : 0));
}
#define F_(a, i, j, k) s->f[(size_t)s->Q * IX(s, i, j, k) + (a)]
#define FP_(a, i, j, k) s->fp[(size_t)s->Q * IX(s, i, j, k) + (a)]
#define OB_(i, j, k) s->obst[IX(s, i, j, k)]
#define ON_(i, j, k) s->obst_new[IX(s, i, j, k)]
#define SC_(arr, i, j, k) s->arr[IX(s, i, j, k)]

/* signed separation along x with the periodic image (case1 pattern) */
/* One shift by L suffices while centres stay in [0.5, nx + 0.5); a larger
 * |d| (a centre that jumped, which update_center reports) takes the closed
 * form d - L rint(d/L), and a non-finite d is returned as is. */
static double dxp(const orc_particles* s, double a, double b) {
    double d = a - b;
    if (s->p.periodic_x && isfinite(d)) {
        double L = (double)s->p.nx, h = 0.5 * L;
        if (d > h) d -= L;
        else if (d < -h) d += L;
        if (d > h || d < -h) d -= L * rint(d / L);
    }
    return d;
}
static double sq_(double x) { return x * x; }

/* inside particle c: ((x-xc)^2 + (y-yc)^2 [+ (z-zc)^2]) <= R^2 (particle_bounceback.F90:50-52) */
static int inside(const orc_particles* s, int c, double x, double y, double z, const double* centers) {
    double d = sq_(dxp(s, x, centers[3 * c])) + sq_(y - centers[3 * c + 1]);
    if (s->p.dim == 3) d = d + sq_(z - centers[3 * c + 2]);
    return d <= sq_(s->radius[c]);
}

/* ---------------------------------------------------------------- MRT ---- */
/* D2Q9 MRT (case4 fluid.F90:14-64) for one cell */
static void mrt9(const double* f, double rho, double u, double v, double Snu, double Sq, double* fp) {
    double m[9], meq[9], s[9], mp[9];
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
    m[1] = -4.0 * f[0] - f[1] - f[2] - f[3] - f[4] + 2.0 * f[5] + 2.0 * f[6] + 2.0 * f[7] + 2.0 * f[8];
    m[2] = 4.0 * f[0] - 2.0 * f[1] - 2.0 * f[2] - 2.0 * f[3] - 2.0 * f[4] + f[5] + f[6] + f[7] + f[8];
    m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
    m[4] = -2.0 * f[1] + 2.0 * f[3] + f[5] - f[6] - f[7] + f[8];
    m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    m[6] = -2.0 * f[2] + 2.0 * f[4] + f[5] + f[6] - f[7] - f[8];
    m[7] = f[1] - f[2] + f[3] - f[4];
    m[8] = f[5] - f[6] + f[7] - f[8];
    meq[0] = rho;
    meq[1] = rho * (-2.0 + 3.0 * (u * u + v * v));
    meq[2] = rho * (1.0 - 3.0 * (u * u + v * v));
    meq[3] = rho * u;
    meq[4] = -meq[3];
    meq[5] = rho * v;
    meq[6] = -meq[5];
    meq[7] = rho * (u * u - v * v);
    meq[8] = rho * (u * v);
    s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq; s[5] = 0.0; s[6] = Sq;
    s[7] = Snu; s[8] = Snu;
    for (int a = 0; a < 9; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]);
    fp[0] = (mp[0] - mp[1] + mp[2]) / 9.0;
    fp[1] = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[3] / 6.0 - mp[4] / 6.0 + mp[7] * 0.25;
    fp[2] = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[5] / 6.0 - mp[6] / 6.0 - mp[7] * 0.25;
    fp[3] = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[3] / 6.0 + mp[4] / 6.0 + mp[7] * 0.25;
    fp[4] = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[5] / 6.0 + mp[6] / 6.0 - mp[7] * 0.25;
    fp[5] = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 + mp[5] / 6.0 +
            mp[6] / 12.0 + mp[8] * 0.25;
    fp[6] = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 + mp[5] / 6.0 +
            mp[6] / 12.0 - mp[8] * 0.25;
    fp[7] = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 - mp[5] / 6.0 -
            mp[6] / 12.0 + mp[8] * 0.25;
    fp[8] = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 - mp[5] / 6.0 -
            mp[6] / 12.0 - mp[8] * 0.25;
}

/* D3Q19 forward moments (bouyancy3d_mpi.F90:652-692) */
static void moments19(const double* f, double* m) {
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] +
           f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    m[1] = -30.0 * f[0] - 11.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6]) +
           8.0 * (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] +
                  f[17] + f[18]);
    m[2] = 12.0 * f[0] - 4.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6]) + f[7] + f[8] + f[9] +
           f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    m[3] = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[4] = -4.0 * (f[1] - f[2]) + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[5] = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[6] = -4.0 * (f[3] - f[4]) + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[7] = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[8] = -4.0 * (f[5] - f[6]) + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[9] = 2.0 * (f[1] + f[2]) - f[3] - f[4] - f[5] - f[6] + f[7] + f[8] + f[9] + f[10] + f[11] +
           f[12] + f[13] + f[14] - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[10] = -4.0 * (f[1] + f[2]) + 2.0 * (f[3] + f[4] + f[5] + f[6]) + f[7] + f[8] + f[9] + f[10] +
            f[11] + f[12] + f[13] + f[14] - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[11] = f[3] + f[4] - f[5] - f[6] + f[7] + f[8] + f[9] + f[10] - (f[11] + f[12] + f[13] + f[14]);
    m[12] = -2.0 * (f[3] + f[4] - f[5] - f[6]) + (f[7] + f[8] + f[9] + f[10]) -
            (f[11] + f[12] + f[13] + f[14]);
    m[13] = f[7] - f[8] - f[9] + f[10];
    m[14] = f[15] - f[16] - f[17] + f[18];
    m[15] = f[11] - f[12] - f[13] + f[14];
    m[16] = f[7] - f[8] + f[9] - f[10] - f[11] + f[12] - f[13] + f[14];
    m[17] = -f[7] - f[8] + f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    m[18] = f[11] + f[12] - f[13] - f[14] - f[15] - f[16] + f[17] + f[18];
}

/* D3Q19 inverse transform (bouyancy3d_mpi.F90:779-855) */
static void inverse19(const double* mp, double* fp) {
    fp[0] = mp[0] / 19.0 - 5.0 / 399.0 * mp[1] + mp[2] / 21.0;
    fp[1] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[3] - mp[4]) * 0.1 + (mp[9] - mp[10]) / 18.0;
    fp[2] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[3] - mp[4]) * 0.1 + (mp[9] - mp[10]) / 18.0;
    fp[3] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[5] - mp[6]) * 0.1 - (mp[9] - mp[10]) / 36.0 + (mp[11] - mp[12]) / 12.0;
    fp[4] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[5] - mp[6]) * 0.1 - (mp[9] - mp[10]) / 36.0 + (mp[11] - mp[12]) / 12.0;
    fp[5] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[7] - mp[8]) * 0.1 - (mp[9] - mp[10]) / 36.0 - (mp[11] - mp[12]) / 12.0;
    fp[6] = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[7] - mp[8]) * 0.1 - (mp[9] - mp[10]) / 36.0 - (mp[11] - mp[12]) / 12.0;
    fp[7] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + 0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[5] + mp[6]) + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 + mp[13] * 0.25 + (mp[16] - mp[17]) * 0.125;
    fp[8] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - 0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[5] - mp[6]) + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 - mp[13] * 0.25 - (mp[16] + mp[17]) * 0.125;
    fp[9] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + 0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[5] - mp[6]) + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 - mp[13] * 0.25 + (mp[16] + mp[17]) * 0.125;
    fp[10] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - 0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[5] + mp[6]) + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 + mp[13] * 0.25 - (mp[16] - mp[17]) * 0.125;
    fp[11] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + 0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[7] + mp[8]) + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 + 0.25 * mp[15] - 0.1250 * (mp[16] - mp[18]);
    fp[12] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - 0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[7] - mp[8]) + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 - 0.25 * mp[15] + 0.125 * (mp[16] + mp[18]);
    fp[13] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + 0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[7] - mp[8]) + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 - 0.25 * mp[15] - 0.125 * (mp[16] + mp[18]);
    fp[14] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - 0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[7] + mp[8]) + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 + 0.25 * mp[15] + 0.125 * (mp[16] - mp[18]);
    fp[15] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + (4.0 * mp[5] + mp[6] + 4.0 * mp[7] + mp[8]) * 0.025 - (mp[9] + mp[10] * 0.5) / 18.0 + 0.25 * mp[14] + 0.125 * (mp[17] - mp[18]);
    fp[16] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - (4.0 * mp[5] + mp[6] - 4.0 * mp[7] - mp[8]) * 0.025 - (mp[9] + mp[10] * 0.5) / 18.0 - 0.25 * mp[14] - 0.125 * (mp[17] + mp[18]);
    fp[17] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + (4.0 * mp[5] + mp[6] - 4.0 * mp[7] - mp[8]) * 0.025 - (mp[9] + mp[10] * 0.5) / 18.0 - 0.25 * mp[14] + 0.125 * (mp[17] + mp[18]);
    fp[18] = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - (4.0 * mp[5] + mp[6] + 4.0 * mp[7] + mp[8]) * 0.025 - (mp[9] + mp[10] * 0.5) / 18.0 + 0.25 * mp[14] - 0.125 * (mp[17] - mp[18]);
}

/* D3Q19 forced MRT for one cell: bouyancy3d_mpi.F90:694-778 with F = rho*a */
static void mrt19(const double* f, double r, double uu, double vv, double ww, double fx, double fy,
                  double fz, double Snu, double Sq, double* fp) {
    double m[19], meq[19], s[19], mp[19], src[19];
    moments19(f, m);
    meq[0] = r;
    meq[1] = -11.0 * r + 19.0 * r * (uu * uu + vv * vv + ww * ww);
    meq[2] = 3.0 * r - 11.0 / 2.0 * r * (uu * uu + vv * vv + ww * ww);
    meq[3] = r * uu;
    meq[4] = -2.0 / 3.0 * meq[3];
    meq[5] = r * vv;
    meq[6] = -2.0 / 3.0 * meq[5];
    meq[7] = r * ww;
    meq[8] = -2.0 / 3.0 * meq[7];
    meq[9] = r * (2.0 * uu * uu - vv * vv - ww * ww);
    meq[10] = -0.5 * meq[9];
    meq[11] = r * (vv * vv - ww * ww);
    meq[12] = -0.5 * meq[11];
    meq[13] = r * (uu * vv);
    meq[14] = r * (vv * ww);
    meq[15] = r * (ww * uu);
    meq[16] = 0.0; meq[17] = 0.0; meq[18] = 0.0;
    s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq; s[5] = 0.0; s[6] = Sq; s[7] = 0.0;
    s[8] = Sq; s[9] = Snu; s[10] = Snu; s[11] = Snu; s[12] = Snu; s[13] = Snu; s[14] = Snu;
    s[15] = Snu; s[16] = Sq; s[17] = Sq; s[18] = Sq;
    src[0] = 0.0;
    src[1] = 38.0 * (uu * fx + vv * fy + ww * fz);
    src[2] = -11.0 * (uu * fx + vv * fy + ww * fz);
    src[3] = fx;
    src[4] = -2.0 / 3.0 * fx;
    src[5] = fy;
    src[6] = -2.0 / 3.0 * fy;
    src[7] = fz;
    src[8] = -2.0 / 3.0 * fz;
    src[9] = 4.0 * uu * fx - 2.0 * vv * fy - 2.0 * ww * fz;
    src[10] = -2.0 * uu * fx + vv * fy + ww * fz;
    src[11] = 2.0 * vv * fy - 2.0 * ww * fz;
    src[12] = -vv * fy + ww * fz;
    src[13] = uu * fy + vv * fx;
    src[14] = vv * fz + ww * fy;
    src[15] = uu * fz + ww * fx;
    src[16] = 0.0; src[17] = 0.0; src[18] = 0.0;
    for (int a = 0; a < 19; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]) + (1.0 - 0.5 * s[a]) * src[a];
    inverse19(mp, fp);
}

/* ------------------------------------------------------------ lifetime --- */
orc_particles* orc_pt_create(const orc_pp* p, const double* centers) {
    orc_particles* s = (orc_particles*)calloc(1, sizeof *s);
    s->p = *p;
    if (p->dim == 2) {
        s->Q = 9;
        s->ex = ex9; s->ey = ey9; s->ez = s->ez0; s->r = r9;
        s->omega[0] = 4.0 / 9.0;
        for (int a = 1; a <= 4; a++) s->omega[a] = 1.0 / 9.0;
        for (int a = 5; a <= 8; a++) s->omega[a] = 1.0 / 36.0;
    } else {
        s->Q = 19;
        s->ex = ex19; s->ey = ey19; s->ez = ez19; s->r = r19;
        s->omega[0] = 1.0 / 3.0;
        for (int a = 1; a <= 6; a++) s->omega[a] = 1.0 / 18.0;
        for (int a = 7; a <= 18; a++) s->omega[a] = 1.0 / 36.0;
    }
    s->X = p->nx + 6;
    s->Y = p->ny + 6;
    s->Z = p->dim == 3 ? p->nz + 6 : 1;
    /* commondata.F90:33-34 */
    s->snu = 1.0 / p->tauf;
    s->sq = 8.0 * (2.0 * p->tauf - 1.0) / (8.0 * p->tauf - 1.0);
    size_t nc = (size_t)s->X * s->Y * s->Z;
    s->f = (double*)calloc(nc * s->Q, sizeof(double));
    s->fp = (double*)calloc(nc * s->Q, sizeof(double));
    s->obst = (int*)calloc(nc, sizeof(int));
    s->obst_new = (int*)calloc(nc, sizeof(int));
    double** fl[] = {&s->rho, &s->u, &s->v, &s->w, &s->up, &s->vp, &s->wp};
    for (int q = 0; q < 7; q++) *fl[q] = (double*)calloc(nc, sizeof(double));
    int np = p->np;
    double** pa[] = {&s->xc, &s->uc, &s->om, &s->xc_old, &s->uc_old, &s->om_old, &s->force, &s->torque};
    for (int q = 0; q < 8; q++) *pa[q] = (double*)calloc((size_t)np * 3, sizeof(double));
    s->radius = (double*)calloc((size_t)np, sizeof(double));
    /* initial.F90:78-188 with the centres given by the caller */
    for (int c = 0; c < np; c++) {
        for (int d = 0; d < 3; d++) s->xc[3 * c + d] = centers[3 * c + d];
        s->radius[c] = p->radius;
    }
    memcpy(s->xc_old, s->xc, sizeof(double) * 3 * np);
    const int kz0 = p->dim == 3 ? 0 : 1, kz1 = p->dim == 3 ? p->nz + 1 : 1;
    for (int k = kz0; k <= kz1; k++)
        for (int j = 0; j <= p->ny + 1; j++)
            for (int i = 0; i <= p->nx + 1; i++)
                for (int c = 0; c < np; c++)
                    if (inside(s, c, (double)i, (double)j, (double)k, s->xc)) OB_(i, j, k) = 1;
    const int k1 = p->dim == 3 ? p->nz : 1;
    for (int k = 1; k <= k1; k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                SC_(rho, i, j, k) = OB_(i, j, k) == 1 ? p->rho_solid : p->rho0;
                SC_(u, i, j, k) = 0.0;
                SC_(v, i, j, k) = 0.0;
                SC_(w, i, j, k) = 0.0;
            }
    /* f = omega*(1 + 3 un + 4.5 un^2 - 1.5 us2) on fluid nodes, u = 0 */
    for (int k = 1; k <= k1; k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (OB_(i, j, k) != 0) continue;
                double uu = SC_(u, i, j, k), vv = SC_(v, i, j, k), ww = SC_(w, i, j, k);
                double us2 = p->dim == 3 ? uu * uu + vv * vv + ww * ww : uu * uu + vv * vv;
                for (int a = 0; a < s->Q; a++) {
                    double un = p->dim == 3 ? uu * s->ex[a] + vv * s->ey[a] + ww * s->ez[a]
                                            : uu * s->ex[a] + vv * s->ey[a];
                    F_(a, i, j, k) = s->omega[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
                }
            }
    /* ghost points: omega*rho0 (initial.F90:157-188); the 2-D reference fills
     * layers -1..n+2, the 3-D form all three */
    const int gl = p->dim == 2 ? -1 : -2, gh = p->dim == 2 ? 2 : 3;
    for (int k = (p->dim == 3 ? -2 : 1); k <= (p->dim == 3 ? p->nz + 3 : 1); k++)
        for (int j = gl; j <= p->ny + gh; j++)
            for (int i = gl; i <= p->nx + gh; i++) {
                int interior = i >= 1 && i <= p->nx && j >= 1 && j <= p->ny &&
                               (p->dim == 2 || (k >= 1 && k <= p->nz));
                if (interior) continue;
                size_t ix = (size_t)(i + 2) + (size_t)s->X * ((size_t)(j + 2) + (size_t)s->Y * (size_t)(p->dim == 3 ? k + 2 : 0));
                for (int a = 0; a < s->Q; a++) {
                    s->f[(size_t)s->Q * ix + a] = s->omega[a] * p->rho0;
                    s->fp[(size_t)s->Q * ix + a] = s->omega[a] * p->rho0;
                }
            }
    return s;
}

void orc_pt_destroy(orc_particles* s) {
    if (!s) return;
    void* ptrs[] = {s->f, s->fp, s->obst, s->obst_new, s->rho, s->u, s->v, s->w, s->up, s->vp,
                    s->wp, s->xc, s->uc, s->om, s->xc_old, s->uc_old, s->om_old, s->force,
                    s->torque, s->radius};
    for (unsigned q = 0; q < sizeof ptrs / sizeof ptrs[0]; q++) free(ptrs[q]);
    free(s);
}

/* -------------------------------------------------------------- fluid ---- */
static int kmax(const orc_particles* s) { return s->p.dim == 3 ? s->p.nz : 1; }

/* fluid.F90:1-72 (2-D) / forced D3Q19 MRT (3-D); solid nodes skipped */
static void collision(orc_particles* s) {
    const orc_pp* p = &s->p;
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (OB_(i, j, k) != 0) continue;
                double fl[19], out[19];
                for (int a = 0; a < s->Q; a++) fl[a] = F_(a, i, j, k);
                double r = SC_(rho, i, j, k);
                if (p->dim == 2) {
                    mrt9(fl, r, SC_(u, i, j, k), SC_(v, i, j, k), s->snu, s->sq, out);
                } else {
                    mrt19(fl, r, SC_(u, i, j, k), SC_(v, i, j, k), SC_(w, i, j, k),
                          r * p->body_force[0], r * p->body_force[1], r * p->body_force[2], s->snu,
                          s->sq, out);
                }
                for (int a = 0; a < s->Q; a++) FP_(a, i, j, k) = out[a];
            }
}

/* fluid.F90:97-108: pull from fluid sources only */
static void streaming(orc_particles* s) {
    const orc_pp* p = &s->p;
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++)
                for (int a = 0; a < s->Q; a++) {
                    int ip = i - s->ex[a], jp = j - s->ey[a], kp = k - s->ez[a];
                    if (OB_(ip, jp, kp) == 0) F_(a, i, j, k) = FP_(a, ip, jp, kp);
                }
}

/* fluid.F90:115-161 (2-D: four walls); 3-D: y and z walls (and x walls
 * unless periodic), halfway bounce-back of every population entering */
static void bounceback_walls(orc_particles* s) {
    const orc_pp* p = &s->p;
    if (p->dim == 2) {
        for (int j = 1; j <= p->ny; j++) {
            F_(1, 1, j, 1) = FP_(3, 1, j, 1);
            F_(5, 1, j, 1) = FP_(7, 1, j, 1);
            F_(8, 1, j, 1) = FP_(6, 1, j, 1);
        }
        for (int j = 1; j <= p->ny; j++) {
            F_(3, p->nx, j, 1) = FP_(1, p->nx, j, 1);
            F_(6, p->nx, j, 1) = FP_(8, p->nx, j, 1);
            F_(7, p->nx, j, 1) = FP_(5, p->nx, j, 1);
        }
        for (int i = 1; i <= p->nx; i++) {
            F_(2, i, 1, 1) = FP_(4, i, 1, 1);
            F_(5, i, 1, 1) = FP_(7, i, 1, 1);
            F_(6, i, 1, 1) = FP_(8, i, 1, 1);
        }
        for (int i = 1; i <= p->nx; i++) {
            F_(4, i, p->ny, 1) = FP_(2, i, p->ny, 1);
            F_(7, i, p->ny, 1) = FP_(5, i, p->ny, 1);
            F_(8, i, p->ny, 1) = FP_(6, i, p->ny, 1);
        }
        return;
    }
    for (int k = 1; k <= p->nz; k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++)
                for (int a = 1; a < 19; a++) {
                    int ip = i - s->ex[a], jp = j - s->ey[a], kp = k - s->ez[a];
                    int out = jp < 1 || jp > p->ny || kp < 1 || kp > p->nz;
                    if (!p->periodic_x) out = out || ip < 1 || ip > p->nx;
                    if (out) F_(a, i, j, k) = FP_(s->r[a], i, j, k);
                }
}

/* fluid.F90:164-184 (+ half-force shift in 3-D, thermal macro form) */
static void macro(orc_particles* s) {
    const orc_pp* p = &s->p;
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (OB_(i, j, k) != 0) continue;
                if (p->dim == 2) {
#define G(a) F_(a, i, j, 1)
                    double r = G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6) + G(7) + G(8);
                    SC_(rho, i, j, k) = r;
                    SC_(u, i, j, k) = (G(1) - G(3) + G(5) - G(6) - G(7) + G(8)) / r;
                    SC_(v, i, j, k) = (G(2) - G(4) + G(5) + G(6) - G(7) - G(8)) / r;
#undef G
                } else {
#define G(a) F_(a, i, j, k)
                    double r = G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6) + G(7) + G(8) + G(9) +
                               G(10) + G(11) + G(12) + G(13) + G(14) + G(15) + G(16) + G(17) + G(18);
                    SC_(rho, i, j, k) = r;
                    SC_(u, i, j, k) = (G(1) - G(2) + G(7) - G(8) + G(9) - G(10) + G(11) - G(12) +
                                       G(13) - G(14) + 0.5 * (r * p->body_force[0])) / r;
                    SC_(v, i, j, k) = (G(3) - G(4) + G(7) + G(8) - G(9) - G(10) + G(15) - G(16) +
                                       G(17) - G(18) + 0.5 * (r * p->body_force[1])) / r;
                    SC_(w, i, j, k) = (G(5) - G(6) + G(11) + G(12) - G(13) - G(14) + G(15) +
                                       G(16) - G(17) - G(18) + 0.5 * (r * p->body_force[2])) / r;
#undef G
                }
            }
}

/* ----------------------------------------------------------- boundary ---- */
/* calQ (particle_bounceback.F90:101-141): bisection along e_alpha from the
 * fluid node for the wall point; calQ2 (:144-185): the ray-sphere root */
static int calq(const orc_particles* s, int c, double x, double y, double z, int a, double* x0,
                double* y0, double* z0, double* q) {
    const double xc = s->xc[3 * c], yc = s->xc[3 * c + 1], zc = s->xc[3 * c + 2], R = s->radius[c];
    const int dim = s->p.dim;
    /* unwrap the node next to the particle's periodic image */
    if (s->p.periodic_x) x = xc + dxp(s, x, xc);
    if (s->p.qmode == 1) {
        double ea = s->ex[a], eb = s->ey[a], ec = dim == 3 ? s->ez[a] : 0.0;
        double ca = ea * ea + eb * eb + ec * ec;
        double cb = 2.0 * (ea * (x - xc) + eb * (y - yc) + (dim == 3 ? ec * (z - zc) : 0.0));
        double cc = (x - xc) * (x - xc) + (y - yc) * (y - yc) + (dim == 3 ? (z - zc) * (z - zc) : 0.0) - R * R;
        double delta = cb * cb - 4.0 * ca * cc;
        if (delta < 0) return 2;
        *q = (-cb - sqrt(delta)) / (2.0 * ca);
        *x0 = x + *q * ea;
        *y0 = y + *q * eb;
        *z0 = z + *q * ec;
    } else {
        const double epsR = (double)1e-9f; /* default-real literal 1e-9 (particle_bounceback.F90:106) */
        double qq = 0.5, qt = 0.5;
        double px = x + qt * (double)s->ex[a], py = y + qt * (double)s->ey[a];
        double pz = z + (dim == 3 ? qt * (double)s->ez[a] : 0.0);
#define DIST() sqrt((px - xc) * (px - xc) + (py - yc) * (py - yc) + (dim == 3 ? (pz - zc) * (pz - zc) : 0.0))
        int guard = 0;
        while (fabs(DIST() - R) >= epsR) {
            if (++guard > 200) return 2;
            if (DIST() > R) {
                qt = qt / 2.0;
                px = px + qt * (double)s->ex[a];
                py = py + qt * (double)s->ey[a];
                if (dim == 3) pz = pz + qt * (double)s->ez[a];
                qq = qq + qt;
            } else if (DIST() < R) {
                qt = qt / 2.0;
                px = px - qt * (double)s->ex[a];
                py = py - qt * (double)s->ey[a];
                if (dim == 3) pz = pz - qt * (double)s->ez[a];
                qq = qq - qt;
            } else {
                return 2;
            }
        }
#undef DIST
        *q = qq;
        *x0 = px;
        *y0 = py;
        *z0 = pz;
    }
    if (*q > 1.0 || *q < 0.0) return 2;
    return 0;
}

/* rotational wall velocity Omega x (x0 - X_c) at the wall point; 2-D:
 * temp1 = -(y0-yc)*Omega, temp2 = (x0-xc)*Omega (particle_bounceback.F90:59-60) */
static void wall_rot(const orc_particles* s, int c, double x0, double y0, double z0, double* rot) {
    const double* X = s->xc + 3 * c;
    const double* O = s->om + 3 * c;
    if (s->p.dim == 2) {
        rot[0] = -(y0 - X[1]) * O[2];
        rot[1] = (x0 - X[0]) * O[2];
        rot[2] = 0.0;
        return;
    }
    double rx = x0 - X[0], ry = y0 - X[1], rz = z0 - X[2];
    rot[0] = O[1] * rz - O[2] * ry;
    rot[1] = O[2] * rx - O[0] * rz;
    rot[2] = O[0] * ry - O[1] * rx;
}

/* rho average over fluid nodes (particle_bounceback.F90:15-35) */
static double rho_average(orc_particles* s, const int* mask) {
    const orc_pp* p = &s->p;
    double acc = 0.0;
    long n = 0;
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++)
                if (mask[IX(s, i, j, k)] == 0) {
                    acc = acc + SC_(rho, i, j, k);
                    n = n + 1;
                }
    return acc / (double)n;
}

/* particle_bounceback.F90:37-97 -- quadratic interpolated bounce-back */
static int bounceback_particle(orc_particles* s) {
    const orc_pp* p = &s->p;
    s->rho_avg = rho_average(s, s->obst);
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (OB_(i, j, k) != 0) continue;
                for (int a = 0; a < s->Q; a++) {
                    int ip = i + s->ex[a], jp = j + s->ey[a], kp = k + s->ez[a];
                    if (OB_(ip, jp, kp) != 1) continue;
                    int found = 0;
                    for (int c = 0; c < p->np; c++) {
                        if (!inside(s, c, (double)ip, (double)jp, (double)kp, s->xc)) continue;
                        found = 1;
                        double x0, y0, z0, q, rot[3];
                        if (calq(s, c, (double)i, (double)j, (double)k, a, &x0, &y0, &z0, &q)) return 2;
                        wall_rot(s, c, x0, y0, z0, rot);
                        const int ra = s->r[a];
                        const double* U = s->uc + 3 * c;
                        double eu = s->ex[ra] * (U[0] + rot[0]) + s->ey[ra] * (U[1] + rot[1]);
                        if (p->dim == 3) eu = eu + s->ez[ra] * (U[2] + rot[2]);
                        const int ex = s->ex[a], ey = s->ey[a], ez = s->ez[a];
                        /* 3-D generalisation: an interpolation node inside a
                         * solid (a gap below two lattice units) has no
                         * post-collision value of this step; the scheme falls
                         * back to the reference's linear IBB (case1/mpi_complete/
                         * particle_bounceback.F90:66-76), or to simple
                         * bounce-back when the linear form lacks its node too.
                         * Nodes outside the domain are ghosts (omega*rho0) and
                         * count as available.  The 2-D mode keeps the
                         * reference's reads of solid f_post. */
                        const int sol1 = p->dim == 3 && OB_(i - ex, j - ey, k - ez) != 0;
                        const int sol2 = p->dim == 3 && OB_(i - 2 * ex, j - 2 * ey, k - 2 * ez) != 0;
                        if (q < 0.5 && !sol1 && !sol2) {
                            F_(ra, i, j, k) = q * (1.0 + 2.0 * q) * FP_(a, i, j, k) +
                                              (1.0 - 4.0 * q * q) * FP_(a, i - ex, j - ey, k - ez) -
                                              q * (1.0 - 2.0 * q) * FP_(a, i - 2 * ex, j - 2 * ey, k - 2 * ez) +
                                              6.0 * s->omega[a] * s->rho_avg * eu;
                        } else if (q < 0.5 && !sol1) {
                            F_(ra, i, j, k) = 2.0 * q * FP_(a, i, j, k) +
                                              (1.0 - 2.0 * q) * FP_(a, i - ex, j - ey, k - ez) +
                                              6.0 * s->omega[a] * s->rho_avg * eu;
                        } else if (q < 0.5) {
                            F_(ra, i, j, k) = FP_(a, i, j, k) + 6.0 * s->omega[a] * s->rho_avg * eu;
                        } else if (!sol1) {
                            F_(ra, i, j, k) = FP_(a, i, j, k) / q / (1.0 + 2.0 * q) +
                                              FP_(ra, i, j, k) * (2.0 * q - 1.0) / q -
                                              FP_(ra, i - ex, j - ey, k - ez) * (2.0 * q - 1.0) / (2.0 * q + 1.0) +
                                              6.0 * s->omega[a] * s->rho_avg / q / (1.0 + 2.0 * q) * eu;
                        } else {
                            F_(ra, i, j, k) = 0.5 / q * FP_(a, i, j, k) +
                                              (1.0 - 0.5 / q) * FP_(ra, i, j, k) +
                                              3.0 * s->omega[a] * s->rho_avg / q * eu;
                        }
                    }
                    if (!found) return 1;
                }
            }
    return 0;
}

/* particle_force.F90:35-190 */
static int cal_force(orc_particles* s) {
    const orc_pp* p = &s->p;
    const int np = p->np;
    double* fsum = (double*)calloc((size_t)np * 3, sizeof(double));
    double* tsum = (double*)calloc((size_t)np * 3, sizeof(double));
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (OB_(i, j, k) != 0) continue;
                for (int a = 1; a < s->Q; a++) {
                    int ip = i + s->ex[a], jp = j + s->ey[a], kp = k + s->ez[a];
                    if (OB_(ip, jp, kp) != 1) continue;
                    int found = 0;
                    for (int c = 0; c < np; c++) {
                        if (!inside(s, c, (double)ip, (double)jp, (double)kp, s->xc)) continue;
                        found = 1;
                        double x0, y0, z0, q, rot[3];
                        if (calq(s, c, (double)i, (double)j, (double)k, a, &x0, &y0, &z0, &q)) {
                            free(fsum); free(tsum);
                            return 2;
                        }
                        wall_rot(s, c, x0, y0, z0, rot);
                        const int ra = s->r[a];
                        const double* U = s->uc + 3 * c;
                        /* Wen et al. 2014 Galilean-invariant momentum exchange (:59-62) */
                        double Fx = (s->ex[a] - U[0] - rot[0]) * FP_(a, i, j, k) - (s->ex[ra] - U[0] - rot[0]) * F_(ra, i, j, k);
                        double Fy = (s->ey[a] - U[1] - rot[1]) * FP_(a, i, j, k) - (s->ey[ra] - U[1] - rot[1]) * F_(ra, i, j, k);
                        double Fz = 0.0;
                        double rx = (x0 - s->xc[3 * c]), ry = (y0 - s->xc[3 * c + 1]);
                        if (p->dim == 2) {
                            rx = x0 - s->xc[3 * c];
                            double T = rx * Fy - ry * Fx;
                            fsum[3 * c] = fsum[3 * c] + Fx;
                            fsum[3 * c + 1] = fsum[3 * c + 1] + Fy;
                            tsum[3 * c + 2] = tsum[3 * c + 2] + T;
                        } else {
                            Fz = (s->ez[a] - U[2] - rot[2]) * FP_(a, i, j, k) - (s->ez[ra] - U[2] - rot[2]) * F_(ra, i, j, k);
                            double rz = z0 - s->xc[3 * c + 2];
                            fsum[3 * c] = fsum[3 * c] + Fx;
                            fsum[3 * c + 1] = fsum[3 * c + 1] + Fy;
                            fsum[3 * c + 2] = fsum[3 * c + 2] + Fz;
                            tsum[3 * c] = tsum[3 * c] + (ry * Fz - rz * Fy);
                            tsum[3 * c + 1] = tsum[3 * c + 1] + (rz * Fx - rx * Fz);
                            tsum[3 * c + 2] = tsum[3 * c + 2] + (rx * Fy - ry * Fx);
                        }
                    }
                    if (!found) {
                        free(fsum); free(tsum);
                        return 1;
                    }
                }
            }
    const double R0 = p->radius;
    const double vol = p->dim == 2 ? PI_ * R0 * R0 : 4.0 / 3.0 * PI_ * R0 * R0 * R0;
    /* 2-D: the reference's scalar gravity pulls along -y */
    const double gmag = p->dim == 2 ? fabs(p->gravity[1])
                                    : sqrt(p->gravity[0] * p->gravity[0] + p->gravity[1] * p->gravity[1] + p->gravity[2] * p->gravity[2]);
    for (int c = 0; c < np; c++) {
        double fij[3] = {0.0, 0.0, 0.0}, fw[3] = {0.0, 0.0, 0.0};
        const double Rc = s->radius[c];
        /* particle-particle springs (:100-125) */
        double scale_p = p->dim == 2 ? PI_ * (Rc * Rc) * (p->rho_solid - s->rho_avg) * gmag / p->stiff_particle
                                     : p->spring_scale_particle;
        for (int c2 = 0; c2 < np; c2++) {
            if (c2 == c) continue;
            double d0 = dxp(s, s->xc[3 * c], s->xc[3 * c2]);
            double d1 = s->xc[3 * c + 1] - s->xc[3 * c2 + 1];
            double d2 = p->dim == 3 ? s->xc[3 * c + 2] - s->xc[3 * c2 + 2] : 0.0;
            double dij = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            const double R2 = s->radius[c2], thr = p->threshold_particle;
            if (dij >= Rc + R2 + thr) {
            } else if (dij < Rc + R2 + thr && dij >= Rc + R2) {
                double t = (dij - Rc - R2 - thr) / thr;
                fij[0] = fij[0] + scale_p * (t * t) * d0 / dij;
                fij[1] = fij[1] + scale_p * (t * t) * d1 / dij;
                fij[2] = fij[2] + scale_p * (t * t) * d2 / dij;
            } else {
                free(fsum); free(tsum);
                return 3;
            }
        }
        /* particle-wall springs (:128-178): 2-D bottom, left, right; 3-D both
         * walls of every non-periodic axis */
        double scale_w = p->dim == 2 ? PI_ * (Rc * Rc) * (p->rho_solid - p->rho0) * gmag / p->stiff_wall
                                     : p->spring_scale_wall;
        const double thw = p->threshold_wall;
        for (int ax = 0; ax < (p->dim == 3 ? 3 : 2); ax++) {
            int n_ax = ax == 0 ? p->nx : (ax == 1 ? p->ny : p->nz);
            int low = 1, high = 1;
            if (ax == 0 && p->periodic_x) low = high = 0;
            if (p->dim == 2 && ax == 1) high = 0; /* case4 has no top-wall spring */
            const double cpos = s->xc[3 * c + ax];
            if (low) {
                double dw = cpos - Rc - 1.0;
                if (dw < 0) { free(fsum); free(tsum); return 4; }
                if (dw < thw) fw[ax] = fw[ax] + scale_w * ((dw - thw) / thw) * ((dw - thw) / thw);
            }
            if (high) {
                double dw = (double)n_ax - cpos - Rc;
                if (dw < 0) { free(fsum); free(tsum); return 4; }
                if (dw < thw) fw[ax] = fw[ax] - scale_w * ((dw - thw) / thw) * ((dw - thw) / thw);
            }
        }
        /* totals (:184-190): fluid force + springs + (rho_s - rho_avg) V g [+ rho_avg V a_body] */
        for (int d = 0; d < 3; d++) {
            double tot = fsum[3 * c + d] + (p->rho_solid - s->rho_avg) * vol * p->gravity[d] + fij[d] + fw[d];
            if (p->dim == 3) tot = tot + s->rho_avg * vol * p->body_force[d];
            if (p->dim == 2 && d == 0) tot = fsum[3 * c] + fij[0] + fw[0];
            if (p->dim == 2 && d == 1) tot = fsum[3 * c + 1] - (p->rho_solid - s->rho_avg) * PI_ * (R0 * R0) * gmag + fij[1] + fw[1];
            if (p->dim == 2 && d == 2) tot = 0.0;
            s->force[3 * c + d] = tot;
            s->torque[3 * c + d] = tsum[3 * c + d];
        }
    }
    free(fsum);
    free(tsum);
    return 0;
}


/* 3-D refill, two phases (see update_center) */
static int refill3(orc_particles* s) {
    const orc_pp* p = &s->p;
    const int np = p->np;
    size_t cap = 1024, nref = 0;
    size_t* cells = (size_t*)malloc(cap * sizeof(size_t));
    double* vals = (double*)malloc(cap * 23 * sizeof(double));
    for (int k = 1; k <= p->nz; k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (!(OB_(i, j, k) == 1 && ON_(i, j, k) == 0)) continue;
                int c = -1;
                for (int cc = 0; cc < np; cc++)
                    if (inside(s, cc, (double)i, (double)j, (double)k, s->xc_old)) { c = cc; break; }
                if (c < 0) { free(cells); free(vals); return 1; }
                double rx = dxp(s, (double)i, s->xc[3 * c]);
                double ry = (double)j - s->xc[3 * c + 1];
                double rz = (double)k - s->xc[3 * c + 2];
                double out = 0.0;
                int ec = 0;
                for (int a = 1; a < 19; a++) {
                    double t = (rx * s->ex[a] + ry * s->ey[a] + rz * s->ez[a]) / sqrt(rx * rx + ry * ry + rz * rz);
                    if (t > out) { out = t; ec = a; }
                }
                if (ec == 0) { free(cells); free(vals); return 5; }
                const int e0 = s->ex[ec], e1 = s->ey[ec], e2 = s->ez[ec];
                double fl[19], m[19], rot[3];
                for (int a = 0; a < 19; a++)
                    fl[a] = 3.0 * F_(a, i + e0, j + e1, k + e2) - 3.0 * F_(a, i + 2 * e0, j + 2 * e1, k + 2 * e2) +
                            F_(a, i + 3 * e0, j + 3 * e1, k + 3 * e2);
                moments19(fl, m);
                wall_rot(s, c, s->xc[3 * c] + rx, (double)j, (double)k, rot);
                const double ra = s->rho_avg;
                m[3] = ra * (s->uc[3 * c] + rot[0]);
                m[5] = ra * (s->uc[3 * c + 1] + rot[1]);
                m[7] = ra * (s->uc[3 * c + 2] + rot[2]);
                inverse19(m, fl);
                if (nref == cap) {
                    cap *= 2;
                    cells = (size_t*)realloc(cells, cap * sizeof(size_t));
                    vals = (double*)realloc(vals, cap * 23 * sizeof(double));
                }
                cells[nref] = IX(s, i, j, k);
                double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
                for (int a = 0; a < 19; a++) {
                    vals[nref * 23 + a] = fl[a];
                    r = r + fl[a];
                    jx = jx + fl[a] * s->ex[a];
                    jy = jy + fl[a] * s->ey[a];
                    jz = jz + fl[a] * s->ez[a];
                }
                vals[nref * 23 + 19] = r;
                vals[nref * 23 + 20] = (jx + 0.5 * (r * p->body_force[0])) / r;
                vals[nref * 23 + 21] = (jy + 0.5 * (r * p->body_force[1])) / r;
                vals[nref * 23 + 22] = (jz + 0.5 * (r * p->body_force[2])) / r;
                nref++;
            }
    for (size_t q = 0; q < nref; q++) {
        size_t ix = cells[q];
        for (int a = 0; a < 19; a++) s->f[(size_t)19 * ix + a] = vals[q * 23 + a];
        s->rho[ix] = vals[q * 23 + 19];
        s->u[ix] = vals[q * 23 + 20];
        s->v[ix] = vals[q * 23 + 21];
        s->w[ix] = vals[q * 23 + 22];
    }
    free(cells);
    free(vals);
    return 0;
}

/* particle_update.F90:26-206 */
static int update_center(orc_particles* s) {
    const orc_pp* p = &s->p;
    const int np = p->np;
    memcpy(s->xc_old, s->xc, sizeof(double) * 3 * np);
    memcpy(s->uc_old, s->uc, sizeof(double) * 3 * np);
    memcpy(s->om_old, s->om, sizeof(double) * 3 * np);
    const double R0 = p->radius;
    for (int c = 0; c < np; c++) {
        if (p->dim == 2) {
            double ax = s->force[3 * c] / PI_ / (R0 * R0) / p->rho_solid;
            double ay = s->force[3 * c + 1] / PI_ / (R0 * R0) / p->rho_solid;
            double aom = s->torque[3 * c + 2] / (0.5 * p->rho_solid * PI_ * (s->radius[c] * s->radius[c] * s->radius[c] * s->radius[c]));
            s->uc[3 * c] = s->uc_old[3 * c] + ax;
            s->uc[3 * c + 1] = s->uc_old[3 * c + 1] + ay;
            s->om[3 * c + 2] = s->om_old[3 * c + 2] + aom;
            s->xc[3 * c] = s->xc_old[3 * c] + s->uc_old[3 * c] + 0.5 * ax;
            s->xc[3 * c + 1] = s->xc_old[3 * c + 1] + s->uc_old[3 * c + 1] + 0.5 * ay;
        } else {
            const double M = p->rho_solid * 4.0 / 3.0 * PI_ * R0 * R0 * R0;
            const double I = 0.4 * M * s->radius[c] * s->radius[c];
            for (int d = 0; d < 3; d++) {
                double a = s->force[3 * c + d] / M;
                s->uc[3 * c + d] = s->uc_old[3 * c + d] + a;
                s->om[3 * c + d] = s->om_old[3 * c + d] + s->torque[3 * c + d] / I;
                s->xc[3 * c + d] = s->xc_old[3 * c + d] + s->uc_old[3 * c + d] + 0.5 * a;
                if (!isfinite(s->xc[3 * c + d]) || !isfinite(s->uc[3 * c + d]) || !isfinite(s->om[3 * c + d]))
                    return 7;
            }
            if (p->periodic_x) {
                double L = (double)p->nx;
                /* one wrap per step holds only for moves below half the period */
                if (!(fabs(s->xc[3 * c] - s->xc_old[3 * c]) < 0.5 * L)) return 7;
                if (s->xc[3 * c] >= L + 0.5) s->xc[3 * c] -= L;
                if (s->xc[3 * c] < 0.5) s->xc[3 * c] += L;
            }
        }
    }
    /* new mask (:80-93), including the first ghost layer */
    const int kz0 = p->dim == 3 ? 0 : 1, kz1 = p->dim == 3 ? p->nz + 1 : 1;
    for (int k = kz0; k <= kz1; k++)
        for (int j = 0; j <= p->ny + 1; j++)
            for (int i = 0; i <= p->nx + 1; i++) {
                ON_(i, j, k) = 0;
                for (int c = 0; c < np; c++)
                    if (inside(s, c, (double)i, (double)j, (double)k, s->xc)) ON_(i, j, k) = 1;
            }
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++)
                if (ON_(i, j, k) == 1) {
                    SC_(rho, i, j, k) = p->rho_solid;
                    SC_(u, i, j, k) = 0.0;
                    SC_(v, i, j, k) = 0.0;
                    SC_(w, i, j, k) = 0.0;
                }
    s->rho_avg = rho_average(s, s->obst_new);
    /* refill nodes that left a particle (:134-193).  2-D: the reference's
     * sequential loop.  3-D: two phases -- every refilled node is computed
     * from the populations as they were before any refill of this step, then
     * all are written -- so the result does not depend on the sweep order;
     * u carries the half-force shift like macro(). */
    if (p->dim == 3) {
        int rc3 = refill3(s);
        if (rc3) return rc3;
        memcpy(s->obst, s->obst_new, sizeof(int) * (size_t)s->X * s->Y * s->Z);
        return 0;
    }
    /* refill nodes that left a particle (:134-193) */
    for (int k = 1; k <= kmax(s); k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++) {
                if (!(OB_(i, j, k) == 1 && ON_(i, j, k) == 0)) continue;
                int found = 0;
                for (int c = 0; c < np; c++) {
                    if (!inside(s, c, (double)i, (double)j, (double)k, s->xc_old)) continue;
                    found = 1;
                    double rx = dxp(s, (double)i, s->xc[3 * c]);
                    double ry = (double)j - s->xc[3 * c + 1];
                    double rz = p->dim == 3 ? (double)k - s->xc[3 * c + 2] : 0.0;
                    double out = 0.0;
                    int ec = 0;
                    for (int a = 1; a < s->Q; a++) {
                        double t;
                        if (p->dim == 2)
                            t = ((i - s->xc[3 * c]) * s->ex[a] + (j - s->xc[3 * c + 1]) * s->ey[a]) /
                                sqrt((i - s->xc[3 * c]) * (i - s->xc[3 * c]) + (j - s->xc[3 * c + 1]) * (j - s->xc[3 * c + 1]));
                        else
                            t = (rx * s->ex[a] + ry * s->ey[a] + rz * s->ez[a]) / sqrt(rx * rx + ry * ry + rz * rz);
                        if (t > out) {
                            out = t;
                            ec = a;
                        }
                    }
                    if (ec == 0) return 5;
                    const int e0 = s->ex[ec], e1 = s->ey[ec], e2 = s->ez[ec];
                    for (int a = 0; a < s->Q; a++)
                        F_(a, i, j, k) = 3.0 * F_(a, i + e0, j + e1, k + e2) -
                                         3.0 * F_(a, i + 2 * e0, j + 2 * e1, k + 2 * e2) +
                                         F_(a, i + 3 * e0, j + 3 * e1, k + 3 * e2);
                    const double ra = s->rho_avg;
                    if (p->dim == 2) {
                        double m[9];
#define G(a) F_(a, i, j, 1)
                        m[0] = G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6) + G(7) + G(8);
                        m[1] = -4.0 * G(0) - G(1) - G(2) - G(3) - G(4) + 2.0 * G(5) + 2.0 * G(6) + 2.0 * G(7) + 2.0 * G(8);
                        m[2] = 4.0 * G(0) - 2.0 * G(1) - 2.0 * G(2) - 2.0 * G(3) - 2.0 * G(4) + G(5) + G(6) + G(7) + G(8);
                        m[3] = ra * (s->uc[3 * c] - (j - s->xc[3 * c + 1]) * s->om[3 * c + 2]);
                        m[4] = -2.0 * G(1) + 2.0 * G(3) + G(5) - G(6) - G(7) + G(8);
                        m[5] = ra * (s->uc[3 * c + 1] + (i - s->xc[3 * c]) * s->om[3 * c + 2]);
                        m[6] = -2.0 * G(2) + 2.0 * G(4) + G(5) + G(6) - G(7) - G(8);
                        m[7] = G(1) - G(2) + G(3) - G(4);
                        m[8] = G(5) - G(6) + G(7) - G(8);
                        G(0) = (m[0] - m[1] + m[2]) / 9.0;
                        G(1) = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[3] / 6.0 - m[4] / 6.0 + m[7] * 0.25;
                        G(2) = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[5] / 6.0 - m[6] / 6.0 - m[7] * 0.25;
                        G(3) = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[3] / 6.0 + m[4] / 6.0 + m[7] * 0.25;
                        G(4) = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[5] / 6.0 + m[6] / 6.0 - m[7] * 0.25;
                        G(5) = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 + m[5] / 6.0 + m[6] / 12.0 + m[8] * 0.25;
                        G(6) = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 + m[5] / 6.0 + m[6] / 12.0 - m[8] * 0.25;
                        G(7) = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 - m[5] / 6.0 - m[6] / 12.0 + m[8] * 0.25;
                        G(8) = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 - m[5] / 6.0 - m[6] / 12.0 - m[8] * 0.25;
                        double r = G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6) + G(7) + G(8);
                        SC_(rho, i, j, k) = r;
                        SC_(u, i, j, k) = (G(1) - G(3) + G(5) - G(6) - G(7) + G(8)) / r;
                        SC_(v, i, j, k) = (G(2) - G(4) + G(5) + G(6) - G(7) - G(8)) / r;
#undef G
                    } else {
                        double fl[19], m[19], rot[3];
                        for (int a = 0; a < 19; a++) fl[a] = F_(a, i, j, k);
                        moments19(fl, m);
                        wall_rot(s, c, s->xc[3 * c] + rx, (double)j, (double)k, rot);
                        m[3] = ra * (s->uc[3 * c] + rot[0]);
                        m[5] = ra * (s->uc[3 * c + 1] + rot[1]);
                        m[7] = ra * (s->uc[3 * c + 2] + rot[2]);
                        inverse19(m, fl);
                        double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
                        for (int a = 0; a < 19; a++) {
                            F_(a, i, j, k) = fl[a];
                            r = r + fl[a];
                            jx = jx + fl[a] * s->ex[a];
                            jy = jy + fl[a] * s->ey[a];
                            jz = jz + fl[a] * s->ez[a];
                        }
                        SC_(rho, i, j, k) = r;
                        SC_(u, i, j, k) = jx / r;
                        SC_(v, i, j, k) = jy / r;
                        SC_(w, i, j, k) = jz / r;
                    }
                }
                if (!found) return 1;
            }
    memcpy(s->obst, s->obst_new, sizeof(int) * (size_t)s->X * s->Y * s->Z);
    return 0;
}

/* main.F90:35-73: collision, streaming, bounceback, bounceback_particle,
 * macro, calForce, itc++, updateCenter */
int orc_pt_step(orc_particles* s, int nsteps) {
    for (int n = 0; n < nsteps; n++) {
        collision(s);
        streaming(s);
        bounceback_walls(s);
        int rc = bounceback_particle(s);
        if (rc) return rc;
        macro(s);
        if ((rc = cal_force(s))) return rc;
        s->itc++;
        if ((rc = update_center(s))) return rc;
    }
    return 0;
}

void orc_pt_get(const orc_particles* s, double* f, double* f_post, double* rho, double* u, double* v,
                double* w, int* obst, double* xc, double* uc, double* om, double* force,
                double* torque, double* rho_avg) {
    const orc_pp* p = &s->p;
    const int nz = kmax(s);
    size_t c = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= p->ny; j++)
            for (int i = 1; i <= p->nx; i++, c++) {
                for (int a = 0; a < s->Q; a++) {
                    if (f) f[c * s->Q + a] = F_(a, i, j, k);
                    if (f_post) f_post[c * s->Q + a] = FP_(a, i, j, k);
                }
                if (rho) rho[c] = SC_(rho, i, j, k);
                if (u) u[c] = SC_(u, i, j, k);
                if (v) v[c] = SC_(v, i, j, k);
                if (w) w[c] = SC_(w, i, j, k);
                if (obst) obst[c] = OB_(i, j, k);
            }
    size_t b = sizeof(double) * 3 * (size_t)p->np;
    if (xc) memcpy(xc, s->xc, b);
    if (uc) memcpy(uc, s->uc, b);
    if (om) memcpy(om, s->om, b);
    if (force) memcpy(force, s->force, b);
    if (torque) memcpy(torque, s->torque, b);
    if (rho_avg) *rho_avg = s->rho_avg;
}
