/*
 * lbm_oracle.c -- CPU restatement of the MGLC reference LBM step (FP64).
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Each function
 * cites the reference routine it restates; expression order is kept so that,
 * compiled with -ffp-contract=off, results match the reference's source
 * semantics bit for bit.  Paths are relative to the MGLC repository root.
 */
#include "lbm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q19 velocity set and weights: mpi_3d_blocked/commondata.f90:29-40 */
static const int ex[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int ez[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

/* 1-based Fortran indexing helpers */
#define IDX3(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
#define FQ(arr, Q, a, i, j, k) arr[(size_t)(a) + (size_t)(Q) * IDX3(i, j, k)]
#define FPQ(arr, Q, a, i, j, k) \
    arr[(size_t)(a) + (size_t)(Q) * ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (size_t)(k)))]

#define f_(a, i, j, k) FQ(f, 19, a, i, j, k)
#define fp_(a, i, j, k) FPQ(f_post, 19, a, i, j, k)
#define g_(a, i, j, k) FQ(g, 7, a, i, j, k)
#define gp_(a, i, j, k) FPQ(g_post, 7, a, i, j, k)
#define S_(arr, i, j, k) arr[IDX3(i, j, k)]

static int g_nthreads = 1;
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static) num_threads(g_nthreads)")
#else
#define OMP_FOR
#endif

/* ========================================================================== */
/* Lid-driven cavity                                                          */
/* ========================================================================== */

/* commondata.f90:9,42 : tauf=U0*dble(total_nx)/Reynolds*3.0d0+0.5d0 */
void orc_lid_params(int total_nx, double reynolds, double u0, double* tauf, double* snu,
                    double* sq) {
    double t = u0 * (double)total_nx / reynolds * 3.0 + 0.5;
    *tauf = t;
    *snu = 1.0 / t;
    *sq = 8.0 * (2.0 * t - 1.0) / (8.0 * t - 1.0);
}

/* initial.f90:46-73 (top layer u=U0 at :55-61 when top_layer_u0 != 0) */
void orc_lid_initial(int nx, int ny, int nz, double u0, double rho0, int top_layer_u0,
                     double* f, double* rho, double* u, double* v, double* w) {
    static const double omega[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                                     1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                     1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                     1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                S_(rho, i, j, k) = rho0;
                S_(u, i, j, k) = 0.0;
                S_(v, i, j, k) = 0.0;
                S_(w, i, j, k) = 0.0;
            }
    if (top_layer_u0)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) S_(u, i, j, nz) = u0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double uu = S_(u, i, j, k), vv = S_(v, i, j, k), ww = S_(w, i, j, k);
                double us2 = uu * uu + vv * vv + ww * ww;
                for (int a = 0; a < 19; a++) {
                    double un = uu * ex[a] + vv * ey[a] + ww * ez[a];
                    f_(a, i, j, k) =
                        S_(rho, i, j, k) * omega[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
                }
            }
}

/* collision.f90:15-202 -- MRT collision, literal expression order.
 * Note meq(12) carries no factor rho in the reference (collision.f90:85). */
void orc_lid_collision(int nx, int ny, int nz, double Snu, double Sq, const double* f,
                       const double* rho, const double* u, const double* v, const double* w,
                       double* f_post) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double m[19], meq[19], s[19], mp[19];
#define F(a) f_(a, i, j, k)
                m[0] = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8) + F(9) + F(10) +
                       F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
                m[1] = -30.0 * F(0) - 11.0 * (F(1) + F(2) + F(3) + F(4) + F(5) + F(6)) +
                       8.0 * (F(7) + F(8) + F(9) + F(10) + F(11) + F(12)) +
                       8.0 * (F(13) + F(14) + F(15) + F(16) + F(17) + F(18));
                m[2] = 12.0 * F(0) - 4.0 * (F(1) + F(2) + F(3) + F(4) + F(5) + F(6)) + F(7) + F(8) +
                       F(9) + F(10) + F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
                m[3] = F(1) - F(2) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) - F(14);
                m[4] = -4.0 * (F(1) - F(2)) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) -
                       F(14);
                m[5] = F(3) - F(4) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) - F(18);
                m[6] = -4.0 * (F(3) - F(4)) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) -
                       F(18);
                m[7] = F(5) - F(6) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) - F(17) - F(18);
                m[8] = -4.0 * (F(5) - F(6)) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) -
                       F(17) - F(18);
                m[9] = 2.0 * (F(1) + F(2)) - F(3) - F(4) - F(5) - F(6) + F(7) + F(8) + F(9) + F(10) +
                       F(11) + F(12) + F(13) + F(14) - 2.0 * (F(15) + F(16) + F(17) + F(18));
                m[10] = -4.0 * (F(1) + F(2)) + 2.0 * (F(3) + F(4) + F(5) + F(6)) + F(7) + F(8) +
                        F(9) + F(10) + F(11) + F(12) + F(13) + F(14) -
                        2.0 * (F(15) + F(16) + F(17) + F(18));
                m[11] = F(3) + F(4) - F(5) - F(6) + F(7) + F(8) + F(9) + F(10) - F(11) - F(12) -
                        F(13) - F(14);
                m[12] = -2.0 * (F(3) + F(4) - F(5) - F(6)) + F(7) + F(8) + F(9) + F(10) - F(11) -
                        F(12) - F(13) - F(14);
                m[13] = F(7) - F(8) - F(9) + F(10);
                m[14] = F(15) - F(16) - F(17) + F(18);
                m[15] = F(11) - F(12) - F(13) + F(14);
                m[16] = F(7) - F(8) + F(9) - F(10) - F(11) + F(12) - F(13) + F(14);
                m[17] = -F(7) - F(8) + F(9) + F(10) + F(15) - F(16) + F(17) - F(18);
                m[18] = F(11) + F(12) - F(13) - F(14) - F(15) - F(16) + F(17) + F(18);
#undef F
                double r = S_(rho, i, j, k), uu = S_(u, i, j, k), vv = S_(v, i, j, k),
                       ww = S_(w, i, j, k);
                meq[0] = r;
                meq[1] = r * (-11.0 + 19.0 * (uu * uu + vv * vv + ww * ww));
                meq[2] = r * (3.0 - 11.0 / 2.0 * (uu * uu + vv * vv + ww * ww));
                meq[3] = r * uu;
                meq[4] = -2.0 / 3.0 * r * uu;
                meq[5] = r * vv;
                meq[6] = -2.0 / 3.0 * r * vv;
                meq[7] = r * ww;
                meq[8] = -2.0 / 3.0 * r * ww;
                meq[9] = r * (2.0 * uu * uu - vv * vv - ww * ww);
                meq[10] = -1.0 / 2.0 * r * (2.0 * uu * uu - vv * vv - ww * ww);
                meq[11] = r * (vv * vv - ww * ww);
                meq[12] = -1.0 / 2.0 * (vv * vv - ww * ww);
                meq[13] = r * uu * vv;
                meq[14] = r * vv * ww;
                meq[15] = r * uu * ww;
                meq[16] = 0.0;
                meq[17] = 0.0;
                meq[18] = 0.0;
                s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq; s[5] = 0.0;
                s[6] = Sq; s[7] = 0.0; s[8] = Sq; s[9] = Snu; s[10] = Snu; s[11] = Snu;
                s[12] = Snu; s[13] = Snu; s[14] = Snu; s[15] = Snu; s[16] = Sq; s[17] = Sq;
                s[18] = Sq;
                for (int a = 0; a < 19; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]);
#define P(a) fp_(a, i, j, k)
                P(0) = mp[0] / 19.0 - 5.0 / 399.0 * mp[1] + mp[2] / 21.0;
                P(1) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + mp[3] / 10.0 -
                       mp[4] / 10.0 + mp[9] / 18.0 - mp[10] / 18.0;
                P(2) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - mp[3] / 10.0 +
                       mp[4] / 10.0 + mp[9] / 18.0 - mp[10] / 18.0;
                P(3) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + mp[5] / 10.0 -
                       mp[6] / 10.0 - mp[9] / 36.0 + mp[10] / 36.0 + mp[11] / 12.0 - mp[12] / 12.0;
                P(4) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - mp[5] / 10.0 +
                       mp[6] / 10.0 - mp[9] / 36.0 + mp[10] / 36.0 + mp[11] / 12.0 - mp[12] / 12.0;
                P(5) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + mp[7] / 10.0 -
                       mp[8] / 10.0 - mp[9] / 36.0 + mp[10] / 36.0 - mp[11] / 12.0 + mp[12] / 12.0;
                P(6) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - mp[7] / 10.0 +
                       mp[8] / 10.0 - mp[9] / 36.0 + mp[10] / 36.0 - mp[11] / 12.0 + mp[12] / 12.0;
                P(7) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[3] / 10.0 +
                       mp[4] / 40.0 + mp[5] / 10.0 + mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 +
                       mp[11] / 12.0 + mp[12] / 24.0 + mp[13] / 4.0 + mp[16] / 8.0 - mp[17] / 8.0;
                P(8) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[3] / 10.0 -
                       mp[4] / 40.0 + mp[5] / 10.0 + mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 +
                       mp[11] / 12.0 + mp[12] / 24.0 - mp[13] / 4.0 - mp[16] / 8.0 - mp[17] / 8.0;
                P(9) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[3] / 10.0 +
                       mp[4] / 40.0 - mp[5] / 10.0 - mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 +
                       mp[11] / 12.0 + mp[12] / 24.0 - mp[13] / 4.0 + mp[16] / 8.0 + mp[17] / 8.0;
                P(10) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[3] / 10.0 -
                        mp[4] / 40.0 - mp[5] / 10.0 - mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 +
                        mp[11] / 12.0 + mp[12] / 24.0 + mp[13] / 4.0 - mp[16] / 8.0 + mp[17] / 8.0;
                P(11) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[3] / 10.0 +
                        mp[4] / 40.0 + mp[7] / 10.0 + mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 -
                        mp[11] / 12.0 - mp[12] / 24.0 + mp[15] / 4.0 - mp[16] / 8.0 + mp[18] / 8.0;
                P(12) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[3] / 10.0 -
                        mp[4] / 40.0 + mp[7] / 10.0 + mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 -
                        mp[11] / 12.0 - mp[12] / 24.0 - mp[15] / 4.0 + mp[16] / 8.0 + mp[18] / 8.0;
                P(13) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[3] / 10.0 +
                        mp[4] / 40.0 - mp[7] / 10.0 - mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 -
                        mp[11] / 12.0 - mp[12] / 24.0 - mp[15] / 4.0 - mp[16] / 8.0 - mp[18] / 8.0;
                P(14) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[3] / 10.0 -
                        mp[4] / 40.0 - mp[7] / 10.0 - mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 -
                        mp[11] / 12.0 - mp[12] / 24.0 + mp[15] / 4.0 + mp[16] / 8.0 - mp[18] / 8.0;
                P(15) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[5] / 10.0 +
                        mp[6] / 40.0 + mp[7] / 10.0 + mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 +
                        mp[14] / 4.0 + mp[17] / 8.0 - mp[18] / 8.0;
                P(16) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[5] / 10.0 -
                        mp[6] / 40.0 + mp[7] / 10.0 + mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 -
                        mp[14] / 4.0 - mp[17] / 8.0 - mp[18] / 8.0;
                P(17) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 + mp[5] / 10.0 +
                        mp[6] / 40.0 - mp[7] / 10.0 - mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 -
                        mp[14] / 4.0 + mp[17] / 8.0 + mp[18] / 8.0;
                P(18) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 - mp[5] / 10.0 -
                        mp[6] / 40.0 - mp[7] / 10.0 - mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 +
                        mp[14] / 4.0 - mp[17] / 8.0 + mp[18] / 8.0;
#undef P
            }
}

/* streaming.f90:8-20 -- pull from the haloed post-collision array */
void orc_lid_streaming(int nx, int ny, int nz, double* f, const double* f_post) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++)
                for (int a = 0; a < 19; a++) f_(a, i, j, k) = fp_(a, i - ex[a], j - ey[a], k - ez[a]);
}

/* bounce_back.f90:6-83 (single rank: every face is a wall).  Faces are
 * written x, then y, then z, so the lid terms win on the top edges. */
void orc_lid_bounceback(int nx, int ny, int nz, double U0, double* f, const double* f_post,
                        const double* rho) {
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            f_(1, 1, j, k) = fp_(2, 1, j, k);
            f_(7, 1, j, k) = fp_(10, 1, j, k);
            f_(9, 1, j, k) = fp_(8, 1, j, k);
            f_(11, 1, j, k) = fp_(14, 1, j, k);
            f_(13, 1, j, k) = fp_(12, 1, j, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            f_(2, nx, j, k) = fp_(1, nx, j, k);
            f_(10, nx, j, k) = fp_(7, nx, j, k);
            f_(8, nx, j, k) = fp_(9, nx, j, k);
            f_(14, nx, j, k) = fp_(11, nx, j, k);
            f_(12, nx, j, k) = fp_(13, nx, j, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            f_(3, i, 1, k) = fp_(4, i, 1, k);
            f_(7, i, 1, k) = fp_(10, i, 1, k);
            f_(8, i, 1, k) = fp_(9, i, 1, k);
            f_(15, i, 1, k) = fp_(18, i, 1, k);
            f_(17, i, 1, k) = fp_(16, i, 1, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            f_(4, i, ny, k) = fp_(3, i, ny, k);
            f_(10, i, ny, k) = fp_(7, i, ny, k);
            f_(9, i, ny, k) = fp_(8, i, ny, k);
            f_(18, i, ny, k) = fp_(15, i, ny, k);
            f_(16, i, ny, k) = fp_(17, i, ny, k);
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            f_(5, i, j, 1) = fp_(6, i, j, 1);
            f_(11, i, j, 1) = fp_(14, i, j, 1);
            f_(12, i, j, 1) = fp_(13, i, j, 1);
            f_(15, i, j, 1) = fp_(18, i, j, 1);
            f_(16, i, j, 1) = fp_(17, i, j, 1);
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            f_(6, i, j, nz) = fp_(5, i, j, nz);
            f_(14, i, j, nz) = fp_(11, i, j, nz) - S_(rho, i, j, nz) / 6.0 * (U0);
            f_(13, i, j, nz) = fp_(12, i, j, nz) - S_(rho, i, j, nz) / 6.0 * (-U0);
            f_(18, i, j, nz) = fp_(15, i, j, nz);
            f_(17, i, j, nz) = fp_(16, i, j, nz);
        }
}

/* macro.f90:6-25 -- sequential accumulation over alpha from zero */
void orc_lid_macro(int nx, int ny, int nz, const double* f, double* rho, double* u, double* v,
                   double* w) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double r = 0.0, uu = 0.0, vv = 0.0, ww = 0.0;
                for (int a = 0; a < 19; a++) {
                    double fa = f_(a, i, j, k);
                    r = r + fa;
                    uu = uu + fa * ex[a];
                    vv = vv + fa * ey[a];
                    ww = ww + fa * ez[a];
                }
                S_(rho, i, j, k) = r;
                S_(u, i, j, k) = uu / r;
                S_(v, i, j, k) = vv / r;
                S_(w, i, j, k) = ww / r;
            }
}

/* check.f90:12-30 -- w is excluded from the numerator (check.f90:15) */
double orc_lid_check(int nx, int ny, int nz, const double* u, const double* v, const double* w,
                     double* up, double* vp, double* wp) {
    double e1 = 0.0, e2 = 0.0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double uu = S_(u, i, j, k), vv = S_(v, i, j, k), ww = S_(w, i, j, k);
                double a = uu - S_(up, i, j, k), b = vv - S_(vp, i, j, k);
                e1 = e1 + a * a + b * b;
                e2 = e2 + uu * uu + vv * vv + ww * ww;
            }
    size_t n = (size_t)nx * ny * nz;
    memcpy(up, u, n * sizeof(double));
    memcpy(vp, v, n * sizeof(double));
    memcpy(wp, w, n * sizeof(double));
    return sqrt(e1) / sqrt(e2);
}

double orc_lid_run(int nx, int ny, int nz, double snu, double sq, double u0, int nsteps,
                   int check_every, int nthreads, double* f, double* f_post, double* rho,
                   double* u, double* v, double* w, double* up, double* vp, double* wp) {
    g_nthreads = nthreads > 0 ? nthreads : 1;
    double err = -1.0;
    for (int itc = 1; itc <= nsteps; itc++) {
        orc_lid_collision(nx, ny, nz, snu, sq, f, rho, u, v, w, f_post);
        orc_lid_streaming(nx, ny, nz, f, f_post);
        orc_lid_bounceback(nx, ny, nz, u0, f, f_post, rho);
        orc_lid_macro(nx, ny, nz, f, rho, u, v, w);
        if (check_every > 0 && itc % check_every == 0)
            err = orc_lid_check(nx, ny, nz, u, v, w, up, vp, wp);
    }
    g_nthreads = 1;
    return err;
}

/* ========================================================================== */
/* Buoyancy-driven cavity                                                     */
/* ========================================================================== */

/* bouyancy3d_mpi.F90:28-54,80-81 (parameters of module commondata) */
void orc_th_params(int total_nz, double rayleigh, double prandtl, double mach, double ekman,
                   orc_th_consts* c) {
    double tauf = 0.5 + mach * (double)total_nz * sqrt(3.0 * prandtl / rayleigh);
    double viscosity = (tauf - 0.5) / 3.0;
    double diffusivity = viscosity / prandtl;
    c->tauf = tauf;
    c->viscosity = viscosity;
    c->diffusivity = diffusivity;
    c->omega_rot = ekman > 0.0 ? viscosity / 2.0 / ekman / (double)(total_nz * total_nz) : 0.0;
    c->para_a = 42.0 * sqrt(3.0) * diffusivity - 6.0;
    double gbeta1 = rayleigh * viscosity * diffusivity / (double)total_nz;
    c->gbeta = gbeta1 / (double)(total_nz * total_nz);
    c->snu = 1.0 / tauf;
    c->sq = 8.0 * (2.0 * tauf - 1.0) / (8.0 * tauf - 1.0);
    c->qd = 3.0 - sqrt(3.0);
    c->qnu = 4.0 * sqrt(3.0) - 6.0;
}

/* bouyancy3d_mpi.F90:409-638 (loadInitField=0 branch) */
void orc_th_initial(int nx, int ny, int nz, const orc_th_consts* c, double t_hot, double t_cold,
                    int bc_y, int bc_z, double* f, double* g, double* rho, double* u, double* v,
                    double* w, double* T) {
    double omega[19], omegaT[7];
    omega[0] = 1.0 / 3.0;
    for (int a = 1; a <= 6; a++) omega[a] = 1.0 / 18.0;
    for (int a = 7; a <= 18; a++) omega[a] = 1.0 / 36.0;
    omegaT[0] = (1.0 - c->para_a) / 7.0;
    for (int a = 1; a <= 6; a++) omegaT[a] = (c->para_a + 6.0) / 42.0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                S_(rho, i, j, k) = 1.0;
                S_(u, i, j, k) = 0.0;
                S_(v, i, j, k) = 0.0;
                S_(w, i, j, k) = 0.0;
                S_(T, i, j, k) = 0.0;
            }
    if (bc_y) { /* LeftRightWallsConstT :517-535 */
        for (int k = 1; k <= nz; k++)
            for (int i = 1; i <= nx; i++) S_(T, i, 1, k) = t_hot;
        for (int k = 1; k <= nz; k++)
            for (int i = 1; i <= nx; i++) S_(T, i, ny, k) = t_cold;
    }
    if (bc_z) { /* TopBottomPlatesConstT :540-559 */
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) S_(T, i, j, 1) = t_hot;
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) S_(T, i, j, nz) = t_cold;
    }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double uu = S_(u, i, j, k), vv = S_(v, i, j, k), ww = S_(w, i, j, k);
                double us2 = uu * uu + vv * vv + ww * ww;
                for (int a = 0; a < 19; a++) {
                    double un = uu * ex[a] + vv * ey[a] + ww * ez[a];
                    f_(a, i, j, k) =
                        S_(rho, i, j, k) * omega[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
                }
                for (int a = 0; a < 7; a++) {
                    double unT = uu * ex[a] + vv * ey[a] + ww * ez[a];
                    g_(a, i, j, k) =
                        omegaT[a] * S_(T, i, j, k) * (1.0 + 21.0 / (6.0 + c->para_a) * unT);
                }
            }
}

/* bouyancy3d_mpi.F90:641-864 -- forced MRT collision; F stored in Fx,Fy,Fz */
void orc_th_collision(int nx, int ny, int nz, const orc_th_consts* c, double Tref,
                      const double* f, const double* rho, const double* u, const double* v,
                      const double* w, const double* T, double* f_post, double* Fx, double* Fy,
                      double* Fz) {
    const double Snu = c->snu, Sq = c->sq, omegaRatating = c->omega_rot, gBeta = c->gbeta;
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double m[19], meq[19], s[19], mp[19], src[19];
#define F(a) f_(a, i, j, k)
                m[0] = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8) + F(9) + F(10) +
                       F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
                m[1] = -30.0 * F(0) - 11.0 * (F(1) + F(2) + F(3) + F(4) + F(5) + F(6)) +
                       8.0 * (F(7) + F(8) + F(9) + F(10) + F(11) + F(12) + F(13) + F(14) + F(15) +
                              F(16) + F(17) + F(18));
                m[2] = 12.0 * F(0) - 4.0 * (F(1) + F(2) + F(3) + F(4) + F(5) + F(6)) + F(7) + F(8) +
                       F(9) + F(10) + F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
                m[3] = F(1) - F(2) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) - F(14);
                m[4] = -4.0 * (F(1) - F(2)) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) -
                       F(14);
                m[5] = F(3) - F(4) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) - F(18);
                m[6] = -4.0 * (F(3) - F(4)) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) -
                       F(18);
                m[7] = F(5) - F(6) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) - F(17) - F(18);
                m[8] = -4.0 * (F(5) - F(6)) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) -
                       F(17) - F(18);
                m[9] = 2.0 * (F(1) + F(2)) - F(3) - F(4) - F(5) - F(6) + F(7) + F(8) + F(9) + F(10) +
                       F(11) + F(12) + F(13) + F(14) - 2.0 * (F(15) + F(16) + F(17) + F(18));
                m[10] = -4.0 * (F(1) + F(2)) + 2.0 * (F(3) + F(4) + F(5) + F(6)) + F(7) + F(8) +
                        F(9) + F(10) + F(11) + F(12) + F(13) + F(14) -
                        2.0 * (F(15) + F(16) + F(17) + F(18));
                m[11] = F(3) + F(4) - F(5) - F(6) + F(7) + F(8) + F(9) + F(10) -
                        (F(11) + F(12) + F(13) + F(14));
                m[12] = -2.0 * (F(3) + F(4) - F(5) - F(6)) + (F(7) + F(8) + F(9) + F(10)) -
                        (F(11) + F(12) + F(13) + F(14));
                m[13] = F(7) - F(8) - F(9) + F(10);
                m[14] = F(15) - F(16) - F(17) + F(18);
                m[15] = F(11) - F(12) - F(13) + F(14);
                m[16] = F(7) - F(8) + F(9) - F(10) - F(11) + F(12) - F(13) + F(14);
                m[17] = -F(7) - F(8) + F(9) + F(10) + F(15) - F(16) + F(17) - F(18);
                m[18] = F(11) + F(12) - F(13) - F(14) - F(15) - F(16) + F(17) + F(18);
#undef F
                double r = S_(rho, i, j, k), uu = S_(u, i, j, k), vv = S_(v, i, j, k),
                       ww = S_(w, i, j, k);
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
                meq[16] = 0.0;
                meq[17] = 0.0;
                meq[18] = 0.0;
                s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq; s[5] = 0.0;
                s[6] = Sq; s[7] = 0.0; s[8] = Sq; s[9] = Snu; s[10] = Snu; s[11] = Snu;
                s[12] = Snu; s[13] = Snu; s[14] = Snu; s[15] = Snu; s[16] = Sq; s[17] = Sq;
                s[18] = Sq;
                double fx = -2.0 * r * vv * omegaRatating;
                double fy = 2.0 * r * uu * omegaRatating;
                double fz = r * gBeta * (S_(T, i, j, k) - Tref);
                S_(Fx, i, j, k) = fx;
                S_(Fy, i, j, k) = fy;
                S_(Fz, i, j, k) = fz;
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
                src[16] = 0.0;
                src[17] = 0.0;
                src[18] = 0.0;
                for (int a = 0; a < 19; a++)
                    mp[a] = m[a] - s[a] * (m[a] - meq[a]) + (1.0 - 0.5 * s[a]) * src[a];
#define P(a) fp_(a, i, j, k)
                P(0) = mp[0] / 19.0 - 5.0 / 399.0 * mp[1] + mp[2] / 21.0;
                P(1) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[3] - mp[4]) * 0.1 +
                       (mp[9] - mp[10]) / 18.0;
                P(2) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[3] - mp[4]) * 0.1 +
                       (mp[9] - mp[10]) / 18.0;
                P(3) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[5] - mp[6]) * 0.1 -
                       (mp[9] - mp[10]) / 36.0 + (mp[11] - mp[12]) / 12.0;
                P(4) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[5] - mp[6]) * 0.1 -
                       (mp[9] - mp[10]) / 36.0 + (mp[11] - mp[12]) / 12.0;
                P(5) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 + (mp[7] - mp[8]) * 0.1 -
                       (mp[9] - mp[10]) / 36.0 - (mp[11] - mp[12]) / 12.0;
                P(6) = mp[0] / 19.0 - 11.0 / 2394.0 * mp[1] - mp[2] / 63.0 - (mp[7] - mp[8]) * 0.1 -
                       (mp[9] - mp[10]) / 36.0 - (mp[11] - mp[12]) / 12.0;
                P(7) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                       0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[5] + mp[6]) + mp[9] / 36.0 +
                       mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 + mp[13] * 0.25 +
                       (mp[16] - mp[17]) * 0.125;
                P(8) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                       0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[5] - mp[6]) + mp[9] / 36.0 +
                       mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 - mp[13] * 0.25 -
                       (mp[16] + mp[17]) * 0.125;
                P(9) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                       0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[5] - mp[6]) + mp[9] / 36.0 +
                       mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 - mp[13] * 0.25 +
                       (mp[16] + mp[17]) * 0.125;
                P(10) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                        0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[5] + mp[6]) + mp[9] / 36.0 +
                        mp[10] / 72.0 + mp[11] / 12.0 + mp[12] / 24.0 + mp[13] * 0.25 -
                        (mp[16] - mp[17]) * 0.125;
                P(11) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                        0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[7] + mp[8]) + mp[9] / 36.0 +
                        mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 + 0.25 * mp[15] -
                        0.1250 * (mp[16] - mp[18]);
                P(12) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                        0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[7] - mp[8]) + mp[9] / 36.0 +
                        mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 - 0.25 * mp[15] +
                        0.125 * (mp[16] + mp[18]);
                P(13) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                        0.025 * (4.0 * mp[3] + mp[4] - 4.0 * mp[7] - mp[8]) + mp[9] / 36.0 +
                        mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 - 0.25 * mp[15] -
                        0.125 * (mp[16] + mp[18]);
                P(14) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                        0.025 * (4.0 * mp[3] + mp[4] + 4.0 * mp[7] + mp[8]) + mp[9] / 36.0 +
                        mp[10] / 72.0 - mp[11] / 12.0 - mp[12] / 24.0 + 0.25 * mp[15] +
                        0.125 * (mp[16] - mp[18]);
                P(15) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                        (4.0 * mp[5] + mp[6] + 4.0 * mp[7] + mp[8]) * 0.025 -
                        (mp[9] + mp[10] * 0.5) / 18.0 + 0.25 * mp[14] + 0.125 * (mp[17] - mp[18]);
                P(16) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                        (4.0 * mp[5] + mp[6] - 4.0 * mp[7] - mp[8]) * 0.025 -
                        (mp[9] + mp[10] * 0.5) / 18.0 - 0.25 * mp[14] - 0.125 * (mp[17] + mp[18]);
                P(17) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 +
                        (4.0 * mp[5] + mp[6] - 4.0 * mp[7] - mp[8]) * 0.025 -
                        (mp[9] + mp[10] * 0.5) / 18.0 - 0.25 * mp[14] + 0.125 * (mp[17] + mp[18]);
                P(18) = mp[0] / 19.0 + 4.0 / 1197.0 * mp[1] + mp[2] / 252.0 -
                        (4.0 * mp[5] + mp[6] + 4.0 * mp[7] + mp[8]) * 0.025 -
                        (mp[9] + mp[10] * 0.5) / 18.0 + 0.25 * mp[14] - 0.125 * (mp[17] - mp[18]);
#undef P
            }
}

/* bouyancy3d_mpi.F90:867-892 */
void orc_th_streaming(int nx, int ny, int nz, double* f, const double* f_post) {
    orc_lid_streaming(nx, ny, nz, f, f_post);
}

/* bouyancy3d_mpi.F90:895-983 (noslipWalls defined: all six faces) */
void orc_th_bounceback(int nx, int ny, int nz, double* f, const double* f_post) {
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            f_(1, 1, j, k) = fp_(2, 1, j, k);
            f_(7, 1, j, k) = fp_(10, 1, j, k);
            f_(9, 1, j, k) = fp_(8, 1, j, k);
            f_(11, 1, j, k) = fp_(14, 1, j, k);
            f_(13, 1, j, k) = fp_(12, 1, j, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            f_(2, nx, j, k) = fp_(1, nx, j, k);
            f_(8, nx, j, k) = fp_(9, nx, j, k);
            f_(10, nx, j, k) = fp_(7, nx, j, k);
            f_(12, nx, j, k) = fp_(13, nx, j, k);
            f_(14, nx, j, k) = fp_(11, nx, j, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            f_(3, i, 1, k) = fp_(4, i, 1, k);
            f_(7, i, 1, k) = fp_(10, i, 1, k);
            f_(8, i, 1, k) = fp_(9, i, 1, k);
            f_(15, i, 1, k) = fp_(18, i, 1, k);
            f_(17, i, 1, k) = fp_(16, i, 1, k);
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            f_(4, i, ny, k) = fp_(3, i, ny, k);
            f_(9, i, ny, k) = fp_(8, i, ny, k);
            f_(10, i, ny, k) = fp_(7, i, ny, k);
            f_(16, i, ny, k) = fp_(17, i, ny, k);
            f_(18, i, ny, k) = fp_(15, i, ny, k);
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            f_(5, i, j, 1) = fp_(6, i, j, 1);
            f_(11, i, j, 1) = fp_(14, i, j, 1);
            f_(12, i, j, 1) = fp_(13, i, j, 1);
            f_(15, i, j, 1) = fp_(18, i, j, 1);
            f_(16, i, j, 1) = fp_(17, i, j, 1);
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            f_(6, i, j, nz) = fp_(5, i, j, nz);
            f_(13, i, j, nz) = fp_(12, i, j, nz);
            f_(14, i, j, nz) = fp_(11, i, j, nz);
            f_(17, i, j, nz) = fp_(16, i, j, nz);
            f_(18, i, j, nz) = fp_(15, i, j, nz);
        }
}

/* bouyancy3d_mpi.F90:1014-1070 -- D3Q7 MRT */
void orc_th_collisionT(int nx, int ny, int nz, const orc_th_consts* c, const double* g,
                       const double* u, const double* v, const double* w, const double* T,
                       double* g_post) {
    const double paraA = c->para_a, Qd = c->qd, Qnu = c->qnu;
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double n[7], neq[7], q[7], np[7];
#define G(a) g_(a, i, j, k)
                n[0] = G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6);
                n[1] = G(1) - G(2);
                n[2] = G(3) - G(4);
                n[3] = G(5) - G(6);
                n[4] = -6.0 * G(0) + G(1) + G(2) + G(3) + G(4) + G(5) + G(6);
                n[5] = 2.0 * G(1) + 2.0 * G(2) - G(3) - G(4) - G(5) - G(6);
                n[6] = G(3) + G(4) - G(5) - G(6);
#undef G
                double t = S_(T, i, j, k);
                neq[0] = t;
                neq[1] = t * S_(u, i, j, k);
                neq[2] = t * S_(v, i, j, k);
                neq[3] = t * S_(w, i, j, k);
                neq[4] = t * paraA;
                neq[5] = 0.0;
                neq[6] = 0.0;
                q[0] = 0.0; q[1] = Qd; q[2] = Qd; q[3] = Qd; q[4] = Qnu; q[5] = Qnu; q[6] = Qnu;
                for (int a = 0; a < 7; a++) np[a] = n[a] - q[a] * (n[a] - neq[a]);
                gp_(0, i, j, k) = np[0] / 7.0 - np[4] / 7.0;
                gp_(1, i, j, k) = np[0] / 7.0 + 0.5 * np[1] + np[4] / 42.0 + np[5] / 6.0;
                gp_(2, i, j, k) = np[0] / 7.0 - 0.5 * np[1] + np[4] / 42.0 + np[5] / 6.0;
                gp_(3, i, j, k) =
                    np[0] / 7.0 + 0.5 * np[2] + np[4] / 42.0 - np[5] / 12.0 + 0.25 * np[6];
                gp_(4, i, j, k) =
                    np[0] / 7.0 - 0.5 * np[2] + np[4] / 42.0 - np[5] / 12.0 + 0.25 * np[6];
                gp_(5, i, j, k) =
                    np[0] / 7.0 + 0.5 * np[3] + np[4] / 42.0 - np[5] / 12.0 - 0.25 * np[6];
                gp_(6, i, j, k) =
                    np[0] / 7.0 - 0.5 * np[3] + np[4] / 42.0 - np[5] / 12.0 - 0.25 * np[6];
            }
}

/* bouyancy3d_mpi.F90:1073-1098 */
void orc_th_streamingT(int nx, int ny, int nz, double* g, const double* g_post) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++)
                for (int a = 0; a < 7; a++) g_(a, i, j, k) = gp_(a, i - ex[a], j - ey[a], k - ez[a]);
}

/* bouyancy3d_mpi.F90:1101-1210 -- face order: top/bottom, left/right, back/front */
void orc_th_bouncebackT(int nx, int ny, int nz, const orc_th_consts* c, double Thot,
                        double Tcold, int bc_y, int bc_z, double* g, const double* g_post) {
    const double paraA = c->para_a;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            if (bc_z) {
                g_(5, i, j, 1) = -gp_(6, i, j, 1) + (6.0 + paraA) / 21.0 * Thot;
            } else {
                g_(5, i, j, 1) = gp_(6, i, j, 1);
            }
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            if (bc_z) {
                g_(6, i, j, nz) = -gp_(5, i, j, nz) + (6.0 + paraA) / 21.0 * Tcold;
            } else {
                g_(6, i, j, nz) = gp_(5, i, j, nz);
            }
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            if (bc_y) {
                g_(3, i, 1, k) = -gp_(4, i, 1, k) + (6.0 + paraA) / 21.0 * Thot;
            } else {
                g_(3, i, 1, k) = gp_(4, i, 1, k);
            }
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            if (bc_y) {
                g_(4, i, ny, k) = -gp_(3, i, ny, k) + (6.0 + paraA) / 21.0 * Tcold;
            } else {
                g_(4, i, ny, k) = gp_(3, i, ny, k);
            }
        }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) g_(1, 1, j, k) = gp_(2, 1, j, k);
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) g_(2, nx, j, k) = gp_(1, nx, j, k);
}

/* bouyancy3d_mpi.F90:986-1010 */
void orc_th_macro(int nx, int ny, int nz, const double* f, const double* Fx, const double* Fy,
                  const double* Fz, double* rho, double* u, double* v, double* w) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
#define F(a) f_(a, i, j, k)
                double r = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8) + F(9) +
                           F(10) + F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
                S_(rho, i, j, k) = r;
                S_(u, i, j, k) = (F(1) - F(2) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) -
                                  F(14) + 0.5 * S_(Fx, i, j, k)) /
                                 r;
                S_(v, i, j, k) = (F(3) - F(4) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) -
                                  F(18) + 0.5 * S_(Fy, i, j, k)) /
                                 r;
                S_(w, i, j, k) = (F(5) - F(6) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) -
                                  F(17) - F(18) + 0.5 * S_(Fz, i, j, k)) /
                                 r;
#undef F
            }
}

/* bouyancy3d_mpi.F90:1215-1231 */
void orc_th_macroT(int nx, int ny, int nz, const double* g, double* T) {
    OMP_FOR
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++)
                S_(T, i, j, k) = g_(0, i, j, k) + g_(1, i, j, k) + g_(2, i, j, k) + g_(3, i, j, k) +
                                 g_(4, i, j, k) + g_(5, i, j, k) + g_(6, i, j, k);
}

/* bouyancy3d_mpi.F90:1234-1281 */
void orc_th_check(int nx, int ny, int nz, const double* u, const double* v, const double* w,
                  const double* T, double* up, double* vp, double* wp, double* Tp, double* error_u,
                  double* error_t) {
    double e1 = 0.0, e2 = 0.0, e5 = 0.0, e6 = 0.0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double uu = S_(u, i, j, k), vv = S_(v, i, j, k), ww = S_(w, i, j, k),
                       tt = S_(T, i, j, k);
                double a = uu - S_(up, i, j, k), b = vv - S_(vp, i, j, k), cc = ww - S_(wp, i, j, k);
                e1 = e1 + a * a + b * b + cc * cc;
                e2 = e2 + uu * uu + vv * vv + ww * ww;
                e5 = e5 + fabs(tt - S_(Tp, i, j, k));
                e6 = e6 + fabs(tt);
                S_(up, i, j, k) = uu;
                S_(vp, i, j, k) = vv;
                S_(wp, i, j, k) = ww;
                S_(Tp, i, j, k) = tt;
            }
    *error_u = sqrt(e1) / sqrt(e2);
    *error_t = e5 / e6;
}

void orc_th_run(int nx, int ny, int nz, const orc_th_consts* c, double t_ref, double t_hot,
                double t_cold, int bc_y, int bc_z, int nsteps, int nthreads, double* f,
                double* f_post, double* g, double* g_post, double* rho, double* u, double* v,
                double* w, double* T, double* Fx, double* Fy, double* Fz) {
    g_nthreads = nthreads > 0 ? nthreads : 1;
    for (int itc = 1; itc <= nsteps; itc++) {
        orc_th_collision(nx, ny, nz, c, t_ref, f, rho, u, v, w, T, f_post, Fx, Fy, Fz);
        orc_th_streaming(nx, ny, nz, f, f_post);
        orc_th_bounceback(nx, ny, nz, f, f_post);
        orc_th_collisionT(nx, ny, nz, c, g, u, v, w, T, g_post);
        orc_th_streamingT(nx, ny, nz, g, g_post);
        orc_th_bouncebackT(nx, ny, nz, c, t_hot, t_cold, bc_y, bc_z, g, g_post);
        orc_th_macro(nx, ny, nz, f, Fx, Fy, Fz, rho, u, v, w);
        orc_th_macroT(nx, ny, nz, g, T);
    }
    g_nthreads = 1;
}
