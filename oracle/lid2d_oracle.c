/*
 * lid2d_oracle.c -- CPU restatement of the reference's D2Q9 MRT lid-driven
 * cavity (MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked), FP64.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  One rank of the
 * blocked MPI code: every neighbour exchange is a no-op and all four walls
 * are domain walls.  Each function cites the routine it restates; expression
 * order is kept, so with -ffp-contract=off the results equal the reference's
 * statements bit for bit (pinned by tests/golden/lid2d_*.npz, which execute
 * those statements).
 *
 * Layout, as the reference's arrays:
 *   f(0:8, 1:nx, 1:ny)         -> f[a + 9*((i-1) + nx*(j-1))]
 *   f_post(0:8, 0:nx+1, 0:ny+1) -> f_post[a + 9*(i + (nx+2)*j)]
 *   rho/u/v/up/vp(1:nx, 1:ny)  -> [(i-1) + nx*(j-1)]
 */
#include "lbm_oracle.h"
#include <math.h>
#include <stddef.h>

/* D2Q9 velocity set: commondata.f90:26-27 */
static const int ex2[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int ey2[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

#define C2(i, j) ((size_t)((i) - 1) + (size_t)nx * (size_t)((j) - 1))
#define F2(a, i, j) f[(size_t)(a) + 9 * C2(i, j)]
#define FP2(a, i, j) f_post[(size_t)(a) + 9 * ((size_t)(i) + (size_t)(nx + 2) * (size_t)(j))]

static int l2_threads = 1;
#ifdef _OPENMP
#define OMP_FOR2 _Pragma("omp parallel for schedule(static) num_threads(l2_threads)")
#else
#define OMP_FOR2
#endif

/* commondata.f90:9,30: tauf=U0*dble(total_nx)/Reynolds*3.0d0+0.5d0,
 * Snu=1/tauf, Sq=8(2 tauf-1)/(8 tauf-1) */
void orc_lid2d_params(int total_nx, double reynolds, double u0, double* tauf, double* snu,
                      double* sq) {
    double t = u0 * (double)total_nx / reynolds * 3.0 + 0.5;
    *tauf = t;
    *snu = 1.0 / t;
    *sq = 8.0 * (2.0 * t - 1.0) / (8.0 * t - 1.0);
}

/* initial.f90:40-68: rho = rho0, u = v = 0 except u = U0 on the top row,
 * f = equilibrium of those fields. */
void orc_lid2d_initial(int nx, int ny, double u0, double rho0, double* f, double* rho,
                       double* u, double* v) {
    double omega[9];
    omega[0] = 4.0 / 9.0;
    for (int a = 1; a <= 4; a++) omega[a] = 1.0 / 9.0;
    for (int a = 5; a <= 8; a++) omega[a] = 1.0 / 36.0;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            rho[C2(i, j)] = rho0;
            u[C2(i, j)] = 0.0;
            v[C2(i, j)] = 0.0;
        }
    for (int i = 1; i <= nx; i++) u[C2(i, ny)] = u0;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            double uu = u[C2(i, j)], vv = v[C2(i, j)];
            double us2 = uu * uu + vv * vv;
            for (int a = 0; a < 9; a++) {
                double un = uu * ex2[a] + vv * ey2[a];
                F2(a, i, j) = rho[C2(i, j)] * omega[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
            }
        }
}

/* evolution.f90:1-71 (collision): MRT with s = (0, Snu, Snu, 0, Sq, 0, Sq, Snu, Snu). */
void orc_lid2d_collision(int nx, int ny, double Snu, double Sq, const double* f,
                         const double* rho, const double* u, const double* v, double* f_post) {
    OMP_FOR2
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            double m[9], meq[9], s[9], mp[9];
#define F(a) F2(a, i, j)
            m[0] = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8);
            m[1] = -4.0 * F(0) - F(1) - F(2) - F(3) - F(4) + 2.0 * (F(5) + F(6) + F(7) + F(8));
            m[2] = 4.0 * F(0) - 2.0 * (F(1) + F(2) + F(3) + F(4)) + F(5) + F(6) + F(7) + F(8);
            m[3] = F(1) - F(3) + F(5) - F(6) - F(7) + F(8);
            m[4] = -2.0 * F(1) + 2.0 * F(3) + F(5) - F(6) - F(7) + F(8);
            m[5] = F(2) - F(4) + F(5) + F(6) - F(7) - F(8);
            m[6] = -2.0 * F(2) + 2.0 * F(4) + F(5) + F(6) - F(7) - F(8);
            m[7] = F(1) - F(2) + F(3) - F(4);
            m[8] = F(5) - F(6) + F(7) - F(8);
#undef F
            const double r = rho[C2(i, j)], uu = u[C2(i, j)], vv = v[C2(i, j)];
            meq[0] = r;
            meq[1] = r * (-2.0 + 3.0 * (uu * uu + vv * vv));
            meq[2] = r * (1.0 - 3.0 * (uu * uu + vv * vv));
            meq[3] = r * uu;
            meq[4] = -r * uu;
            meq[5] = r * vv;
            meq[6] = -r * vv;
            meq[7] = r * (uu * uu - vv * vv);
            meq[8] = r * (uu * vv);
            s[0] = 0.0;
            s[1] = Snu;
            s[2] = Snu;
            s[3] = 0.0;
            s[4] = Sq;
            s[5] = 0.0;
            s[6] = Sq;
            s[7] = Snu;
            s[8] = Snu;
            for (int a = 0; a < 9; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]);
            FP2(0, i, j) = (mp[0] - mp[1] + mp[2]) / 9.0;
            FP2(1, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[3] / 6.0 - mp[4] / 6.0 +
                           mp[7] * 0.25;
            FP2(2, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[5] / 6.0 - mp[6] / 6.0 -
                           mp[7] * 0.25;
            FP2(3, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[3] / 6.0 + mp[4] / 6.0 +
                           mp[7] * 0.25;
            FP2(4, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[5] / 6.0 + mp[6] / 6.0 -
                           mp[7] * 0.25;
            FP2(5, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 +
                           mp[5] / 6.0 + mp[6] / 12.0 + mp[8] * 0.25;
            FP2(6, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 +
                           mp[5] / 6.0 + mp[6] / 12.0 - mp[8] * 0.25;
            FP2(7, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 -
                           mp[5] / 6.0 - mp[6] / 12.0 + mp[8] * 0.25;
            FP2(8, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 -
                           mp[5] / 6.0 - mp[6] / 12.0 - mp[8] * 0.25;
        }
}

/* evolution.f90:75-94 (streaming): pull from f_post, halo included.  The
 * halo entries are never written; every value read from them is replaced by
 * bounceback() below, so the halo is only read, never used. */
void orc_lid2d_streaming(int nx, int ny, double* f, const double* f_post) {
    OMP_FOR2
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++)
            for (int a = 0; a < 9; a++) F2(a, i, j) = FP2(a, i - ex2[a], j - ey2[a]);
}

/* bounceback.f90:1-45: halfway bounce-back on the four walls, the lid term
 * -rho*Uwall/6 on the top row; the top loop runs last and so wins at the two
 * top corners. */
void orc_lid2d_bounceback(int nx, int ny, double uwall, double* f, const double* f_post,
                          const double* rho) {
    for (int j = 1; j <= ny; j++) {
        F2(1, 1, j) = FP2(3, 1, j);
        F2(5, 1, j) = FP2(7, 1, j);
        F2(8, 1, j) = FP2(6, 1, j);
    }
    for (int j = 1; j <= ny; j++) {
        F2(3, nx, j) = FP2(1, nx, j);
        F2(6, nx, j) = FP2(8, nx, j);
        F2(7, nx, j) = FP2(5, nx, j);
    }
    for (int i = 1; i <= nx; i++) {
        F2(2, i, 1) = FP2(4, i, 1);
        F2(5, i, 1) = FP2(7, i, 1);
        F2(6, i, 1) = FP2(8, i, 1);
    }
    for (int i = 1; i <= nx; i++) {
        F2(4, i, ny) = FP2(2, i, ny);
        F2(7, i, ny) = FP2(5, i, ny) - rho[C2(i, ny)] * (uwall) / 6.0;
        F2(8, i, ny) = FP2(6, i, ny) - rho[C2(i, ny)] * (-uwall) / 6.0;
    }
}

/* evolution.f90:98-112 (macro) */
void orc_lid2d_macro(int nx, int ny, const double* f, double* rho, double* u, double* v) {
    OMP_FOR2
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            const size_t c = C2(i, j);
            rho[c] = F2(0, i, j) + F2(1, i, j) + F2(2, i, j) + F2(3, i, j) + F2(4, i, j) +
                     F2(5, i, j) + F2(6, i, j) + F2(7, i, j) + F2(8, i, j);
            u[c] = (F2(1, i, j) - F2(3, i, j) + F2(5, i, j) - F2(6, i, j) - F2(7, i, j) +
                    F2(8, i, j)) / rho[c];
            v[c] = (F2(2, i, j) - F2(4, i, j) + F2(5, i, j) + F2(6, i, j) - F2(7, i, j) -
                    F2(8, i, j)) / rho[c];
        }
}

/* evolution.f90:115-150 (check): sums in (j, i) order, then up = u, vp = v. */
double orc_lid2d_check(int nx, int ny, const double* u, const double* v, double* up,
                       double* vp) {
    double e1 = 0.0, e2 = 0.0;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            const size_t c = C2(i, j);
            e1 = e1 + (u[c] - up[c]) * (u[c] - up[c]) + (v[c] - vp[c]) * (v[c] - vp[c]);
            e2 = e2 + u[c] * u[c] + v[c] * v[c];
        }
    for (size_t c = 0; c < (size_t)nx * ny; c++) {
        up[c] = u[c];
        vp[c] = v[c];
    }
    return sqrt(e1) / sqrt(e2);
}

/* nsteps of main.f90:69-89: collision, (message_passing), streaming,
 * bounceback, macro; check() every check_every steps (0 = never).  Returns
 * the last errorU, or -1 when no check ran. */
double orc_lid2d_run(int nx, int ny, double snu, double sq, double u0, int nsteps,
                     int check_every, int nthreads, double* f, double* f_post, double* rho,
                     double* u, double* v, double* up, double* vp) {
    l2_threads = nthreads > 0 ? nthreads : 1;
    double err = -1.0;
    for (int itc = 1; itc <= nsteps; itc++) {
        orc_lid2d_collision(nx, ny, snu, sq, f, rho, u, v, f_post);
        orc_lid2d_streaming(nx, ny, f, f_post);
        orc_lid2d_bounceback(nx, ny, u0, f, f_post, rho);
        orc_lid2d_macro(nx, ny, f, rho, u, v);
        if (check_every > 0 && itc % check_every == 0) err = orc_lid2d_check(nx, ny, u, v, up, vp);
    }
    return err;
}
