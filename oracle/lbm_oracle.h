/*
 * lbm_oracle.h -- CPU restatement of the MGLC reference lattice-Boltzmann step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only the test suite, the smoke check and the CPU-baseline leg of bench.py
 * may load it.  The product (libmglc_gb300.so) never links or calls it.
 *
 * Layout follows the reference exactly: Fortran column-major arrays with the
 * population index fastest,
 *   f(0:Q-1, 1:nx, 1:ny, 1:nz)                   -> f[a + Q*((i-1) + nx*((j-1) + ny*(k-1)))]
 *   f_post(0:Q-1, 0:nx+1, 0:ny+1, 0:nz+1)        -> halo array, (nx+2)(ny+2)(nz+2)*Q doubles
 *   rho/u/v/w/T(1:nx, 1:ny, 1:nz)                -> [ (i-1) + nx*((j-1) + ny*(k-1)) ]
 * Arithmetic follows the reference's expression order; build with
 * -O2 -ffp-contract=off (no FMA contraction, no reassociation).
 *
 * Parity pin: tests/golden/gen_golden.py executes the reference's own Fortran
 * statements through a mechanical Fortran-subset interpreter and stores the
 * results; the oracle reproduces those fixtures bit for bit.
 */
#ifndef MGLC_LBM_ORACLE_H
#define MGLC_LBM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* ---- lid-driven cavity (MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked) ---- */
void orc_lid_params(int total_nx, double reynolds, double u0,
                    double* tauf, double* snu, double* sq);
void orc_lid_initial(int nx, int ny, int nz, double u0, double rho0, int top_layer_u0,
                     double* f, double* rho, double* u, double* v, double* w);
void orc_lid_collision(int nx, int ny, int nz, double snu, double sq,
                       const double* f, const double* rho, const double* u,
                       const double* v, const double* w, double* f_post);
void orc_lid_streaming(int nx, int ny, int nz, double* f, const double* f_post);
void orc_lid_bounceback(int nx, int ny, int nz, double u0, double* f,
                        const double* f_post, const double* rho);
void orc_lid_macro(int nx, int ny, int nz, const double* f,
                   double* rho, double* u, double* v, double* w);
double orc_lid_check(int nx, int ny, int nz, const double* u, const double* v,
                     const double* w, double* up, double* vp, double* wp);
/* nsteps of: collision, streaming, bounceback, macro (main.f90:85-102).  A
 * residual check every check_every steps (0 = never) writes into up/vp/wp and
 * returns the last errorU (or -1 when no check ran).  nthreads > 1 uses
 * OpenMP over k for the cell-local sweeps (results are identical). */
double orc_lid_run(int nx, int ny, int nz, double snu, double sq, double u0,
                   int nsteps, int check_every, int nthreads,
                   double* f, double* f_post, double* rho, double* u, double* v, double* w,
                   double* up, double* vp, double* wp);

/* ---- D2Q9 lid-driven cavity (MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked),
 * lid2d_oracle.c.  f(0:8,1:nx,1:ny), f_post(0:8,0:nx+1,0:ny+1), fields (1:nx,1:ny). ---- */
void orc_lid2d_params(int total_nx, double reynolds, double u0, double* tauf, double* snu,
                      double* sq);
void orc_lid2d_initial(int nx, int ny, double u0, double rho0, double* f, double* rho,
                       double* u, double* v);
void orc_lid2d_collision(int nx, int ny, double snu, double sq, const double* f,
                         const double* rho, const double* u, const double* v, double* f_post);
void orc_lid2d_streaming(int nx, int ny, double* f, const double* f_post);
void orc_lid2d_bounceback(int nx, int ny, double uwall, double* f, const double* f_post,
                          const double* rho);
void orc_lid2d_macro(int nx, int ny, const double* f, double* rho, double* u, double* v);
double orc_lid2d_check(int nx, int ny, const double* u, const double* v, double* up,
                       double* vp);
double orc_lid2d_run(int nx, int ny, double snu, double sq, double u0, int nsteps,
                     int check_every, int nthreads, double* f, double* f_post, double* rho,
                     double* u, double* v, double* up, double* vp);

/* ---- buoyancy-driven cavity (MPI/Buoyancy_driven_cavity/fortran/3d/bouyancy3d_mpi.F90) ---- */
typedef struct {
    double tauf, viscosity, diffusivity, omega_rot, para_a, gbeta, snu, sq, qd, qnu;
} orc_th_consts;
/* ekman <= 0 turns the Coriolis force off (omega_rot = 0). */
void orc_th_params(int total_nz, double rayleigh, double prandtl, double mach,
                   double ekman, orc_th_consts* out);
/* bc_y / bc_z: 0 = adiabatic walls, 1 = constant-temperature walls (hot at the
 * low face, cold at the high face).  x faces are always adiabatic. */
void orc_th_initial(int nx, int ny, int nz, const orc_th_consts* c,
                    double t_hot, double t_cold, int bc_y, int bc_z,
                    double* f, double* g, double* rho, double* u, double* v, double* w,
                    double* T);
void orc_th_collision(int nx, int ny, int nz, const orc_th_consts* c, double t_ref,
                      const double* f, const double* rho, const double* u,
                      const double* v, const double* w, const double* T,
                      double* f_post, double* Fx, double* Fy, double* Fz);
void orc_th_streaming(int nx, int ny, int nz, double* f, const double* f_post);
void orc_th_bounceback(int nx, int ny, int nz, double* f, const double* f_post);
void orc_th_collisionT(int nx, int ny, int nz, const orc_th_consts* c,
                       const double* g, const double* u, const double* v,
                       const double* w, const double* T, double* g_post);
void orc_th_streamingT(int nx, int ny, int nz, double* g, const double* g_post);
void orc_th_bouncebackT(int nx, int ny, int nz, const orc_th_consts* c,
                        double t_hot, double t_cold, int bc_y, int bc_z,
                        double* g, const double* g_post);
void orc_th_macro(int nx, int ny, int nz, const double* f, const double* Fx,
                  const double* Fy, const double* Fz,
                  double* rho, double* u, double* v, double* w);
void orc_th_macroT(int nx, int ny, int nz, const double* g, double* T);
void orc_th_check(int nx, int ny, int nz, const double* u, const double* v,
                  const double* w, const double* T, double* up, double* vp,
                  double* wp, double* Tp, double* error_u, double* error_t);
/* nsteps in the order of bouyancy3d_mpi.F90:222-249. */
void orc_th_run(int nx, int ny, int nz, const orc_th_consts* c, double t_ref,
                double t_hot, double t_cold, int bc_y, int bc_z,
                int nsteps, int nthreads,
                double* f, double* f_post, double* g, double* g_post,
                double* rho, double* u, double* v, double* w, double* T,
                double* Fx, double* Fy, double* Fz);

/* ---- moving particles (MPI/Micro_particles/fortran/case4/mpi_particle) ---- */
typedef struct {
    int dim;        /* 2: literal D2Q9 case4; 3: D3Q19 spheres */
    int nx, ny, nz; /* nz = 1 in 2-D */
    int periodic_x; /* 3-D channel */
    int np;
    double tauf, rho0, rho_solid, radius;
    double gravity[3];    /* acceleration on the particles; 2-D reference: (0,-g,0) */
    double body_force[3]; /* fluid body-force acceleration (3-D, MRT source) */
    double threshold_wall, stiff_wall, threshold_particle, stiff_particle;
    double spring_scale_wall, spring_scale_particle; /* 3-D spring scales */
    int qmode; /* 0: bisection calQ (reference), 1: analytic calQ2 */
} orc_pp;
typedef struct orc_particles orc_particles;
orc_particles* orc_pt_create(const orc_pp* p, const double* centers /* np*3 */);
/* returns 0, or 1 no owning particle, 2 q out of range, 3 particle overlap,
 * 4 wall penetration, 5 no refill direction, 7 diverged (a centre, velocity
 * or spin not finite, or a periodic-x move of half the period or more) */
int orc_pt_step(orc_particles* s, int nsteps);
void orc_pt_get(const orc_particles* s, double* f, double* f_post, double* rho, double* u,
                double* v, double* w, int* obst, double* xc, double* uc, double* om,
                double* force, double* torque, double* rho_avg);
void orc_pt_destroy(orc_particles* s);

/* ---- circles in shear flow, periodic x (MPI/Micro_particles/fortran/case1/mpi_complete),
 * shear2d_oracle.c.  centers = np x (x, y); outputs (ny, nx) fields, np x 2 vectors. ---- */
typedef struct {
    int nx, ny, np;
    int moving_frame; /* 0: stationaryFrame (the shipped build), 1: movingFrame */
    int linear;       /* 0: quadratic IBB and refill (shipped), 1: linear */
    double tauf, rho0, rho_solid, radius;
    double u0;        /* carrier speed of the circles (stationary frame) */
    double uwall;     /* wall speeds -uwall (j = 1) and +uwall (j = ny) */
} orc_shear_params;
typedef struct orc_shear orc_shear;
orc_shear* orc_shear_create(const orc_shear_params* p, const double* centers);
/* returns 0, or 1 no owning circle, 2 q out of range, 5 no refill direction */
int orc_shear_step(orc_shear* s, int nsteps);
void orc_shear_get(const orc_shear* s, double* f, double* rho, double* u, double* v, int* obst,
                   double* xc, double* uc, double* force, double* torque, double* rho_avg);
void orc_shear_destroy(orc_shear* s);

#ifdef __cplusplus
}
#endif
#endif
