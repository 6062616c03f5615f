/*
 * mglc.h -- C-ABI of libmglc_gb300.so: the MGLC lattice-Boltzmann time step on
 * one GB300 GPU (sm_103a).
 *
 * The reference (cheryli/MGLC, Fortran 90 + MPI) has no library interface:
 * its hot path is a set of argument-less subroutines acting on module arrays,
 * called from `program main`'s loop.  Each entry point below replaces one of
 * those calls; the header comment of each names the reference routine (paths
 * relative to the MGLC repository root).  A Fortran host binds these through
 * iso_c_binding (fortran/mglc_iface.f90); C, C++ and Python (ctypes) call them
 * directly.
 *
 * Conventions
 *  - Every function returns an int status (MGLC_OK = 0).  On failure the
 *    context keeps a message readable with mglc_last_error().  Nothing exits
 *    or throws across the ABI.
 *  - Host arrays are caller-owned and use the reference's Fortran layout:
 *    populations f(0:18,1:nx,1:ny,1:nz) with the population index fastest,
 *    g(0:6,1:nx,1:ny,1:nz), and scalar fields rho(1:nx,1:ny,1:nz), x fastest.
 *    Device memory is owned by the context.
 *  - A context is bound to one CUDA stream; calls on one context are not
 *    thread-safe, different contexts may be driven from different threads.
 *    mglc_step() is asynchronous; getters synchronise the context's stream.
 */
#ifndef MGLC_GB300_H
#define MGLC_GB300_H
#ifdef __cplusplus
extern "C" {
#endif

#define MGLC_OK 0
#define MGLC_ERR_INVALID 1     /* bad argument or size */
#define MGLC_ERR_CUDA 2        /* CUDA runtime error */
#define MGLC_ERR_NOMEM 3       /* device allocation failed */
#define MGLC_ERR_STATE 4       /* call not valid for this context kind or state */
#define MGLC_ERR_NUMERIC 5     /* NaN or Inf found in the state */
#define MGLC_ERR_UNSUPPORTED 6 /* feature not built for this form */
#define MGLC_ERR_PARTICLE 7    /* particle overlap or wall penetration */

/* Storage / arithmetic form of the populations.
 *  FP64: FP64 storage and FP64 arithmetic -- the drop-in for the reference.
 *  FP32/FP16/BF16: populations stored as deviations f_i - w_i*rho0 in that
 *  type, FP32 arithmetic; FP64 kept for reductions (residual, totals).
 *  FX64 (lid-driven and heated cavities): FP64 storage; the collisions run in
 *  64-bit fixed point with 55 fractional bits (exact moment transforms, one
 *  rounding to FP64 per stored value), everything else as FP64.
 *  FP16S/BF16S: FP16/BF16 deviation storage written with stochastic rounding
 *  (unbiased; the storage error stays at its one-step level instead of
 *  accumulating over a transient).  The stored state then fluctuates at the
 *  16-bit resolution, so a steady state is not a fixed point: for runs to
 *  convergence (max|du|/U below ~1e-4) use FP16/BF16 (round to nearest). */
enum { MGLC_FP64 = 0, MGLC_FP32 = 1, MGLC_FP16 = 2, MGLC_BF16 = 3, MGLC_FX64 = 4,
       MGLC_FP16S = 5, MGLC_BF16S = 6 };

enum { MGLC_KIND_LID = 1, MGLC_KIND_THERMAL = 2, MGLC_KIND_PARTICLE = 3, MGLC_KIND_PARTICLE2D = 4,
       MGLC_KIND_LID2D = 5 };

typedef struct mglc_ctx mglc_ctx;

/* Lid-driven cavity parameters: MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked/commondata.f90:4-9
 * tauf = u0*total_nx/reynolds*3 + 0.5; lid moves along +x on the top z plane. */
typedef struct mglc_lid_params {
    int total_nx, total_ny, total_nz; /* lattice nodes per axis */
    double reynolds;                  /* Re, based on total_nx */
    double rho0;                      /* initial density (1.0) */
    double u0;                        /* lid velocity (lattice units) */
    int top_layer_u0; /* 1: initial u = u0 on the top layer (initial.f90:55-61); 0: u = 0 */
    int precision;    /* MGLC_FP64 ... MGLC_FX64 */
    int in_place;     /* 1: AA-pattern streaming on one population buffer (half the
                         memory; every precision; results identical to 0) */
} mglc_lid_params;

/* Buoyancy-driven cavity parameters:
 * MPI/Buoyancy_driven_cavity/fortran/3d/bouyancy3d_mpi.F90:28-54.
 * tauf = 0.5 + mach*total_nz*sqrt(3*prandtl/rayleigh); Boussinesq force
 * F_z = rho*gbeta*(T - t_ref); Coriolis F_x = -2 rho v Omega, F_y = 2 rho u Omega
 * with Omega = nu/2/ekman/total_nz^2 (ekman <= 0 turns rotation off). */
typedef struct mglc_thermal_params {
    int total_nx, total_ny, total_nz;
    double rayleigh, prandtl, mach;
    double t_hot, t_cold, t_ref;
    double ekman;
    int bc_y_const_t; /* 1: LeftRightWallsConstT (hot j=1, cold j=ny); 0: adiabatic */
    int bc_z_const_t; /* 1: TopBottomPlatesConstT (hot k=1, cold k=nz); 0: adiabatic */
    int precision;
    int in_place;     /* 1: AA-pattern streaming of f and g on one buffer each (every
                         precision; results identical to 0) */
} mglc_thermal_params;

/* Moving spheres in a D3Q19 flow: the 3-D generalisation of
 * MPI/Micro_particles/fortran/case4/mpi_particle (commondata.F90:26-60).
 * x is periodic or walled; y and z are no-slip walls. */
typedef struct mglc_particle_params {
    int total_nx, total_ny, total_nz;
    int periodic_x;            /* 1: periodic in x (channel); 0: walls on the x faces */
    double tauf;               /* relaxation time, 3*viscosity + 0.5 (commondata.F90:33) */
    double rho0, rho_solid;    /* fluid reference density, particle density */
    double radius;             /* sphere radius (lattice units) */
    double gravity[3];         /* acceleration on the particles: (rho_s - rho_avg) V g */
    double body_force[3];      /* fluid body-force acceleration; rho_avg V a acts on particles */
    double threshold_wall, threshold_particle;       /* spring ranges (particle_force.F90:100-178) */
    double spring_scale_wall, spring_scale_particle; /* spring force scales */
    int precision;             /* MGLC_FP64 or MGLC_FP32 (FP32: deviation storage, FP32 arithmetic) */
} mglc_particle_params;

/* Derived constants of a context (for logging and tests). */
typedef struct mglc_info {
    int kind, precision;
    int nx, ny, nz;
    long long itc;           /* time steps taken since initial()/load */
    double tauf, snu, sq;    /* flow relaxation */
    double viscosity, diffusivity, para_a, gbeta, omega_rot; /* thermal only */
    double bytes_per_cell_step; /* algorithmic HBM bytes of one fused step per cell */
    long long device_bytes;  /* device memory held by the context */
} mglc_info;

/* ---- lifetime ---------------------------------------------------------- */
/* Replaces the allocation part of initial.f90:35-44 (lid). */
int mglc_lid_create(const mglc_lid_params* p, mglc_ctx** out);
/* Replaces the allocation part of bouyancy3d_mpi.F90:476-496 (thermal). */
int mglc_thermal_create(const mglc_thermal_params* p, mglc_ctx** out);
/* Replaces allocate_all + the placement part of initial.F90:48-116 (particles);
 * centers = np x (x,y,z) in node coordinates (node i sits at x = i, 1-based). */
int mglc_particle_create(const mglc_particle_params* p, const double* centers, int np,
                         mglc_ctx** out);
/* D2Q9 moving circles: the reference's own 2-D case4 step
 * (MPI/Micro_particles/fortran/case4/mpi_particle, main.F90:35-73) with the
 * parameters of its commondata.F90: closed box (four halfway-bounce-back
 * walls), gravity along -y, springs with stiffness and threshold against
 * particles and the left, right and bottom walls.  FP64, every statement in
 * the reference's order (bitwise the reference's results).  centers = np x
 * (x, y), node i at x = i (1-based).  Verbs: mglc_initial, mglc_step,
 * mglc_get_f (9 per node), mglc_get_macros (w = 0), mglc_particle_state,
 * mglc_get_mask. */
typedef struct mglc_particle2d_params {
    int total_nx, total_ny;
    double tauf, rho0, rho_solid, radius;
    double gravity;                          /* magnitude, acting along -y */
    double threshold_wall, stiff_wall, threshold_particle, stiff_particle;
    int q_bisection;                         /* 1: calQ bisection (reference), 0: calQ2 */
} mglc_particle2d_params;
int mglc_particle2d_create(const mglc_particle2d_params* p, const double* centers, int np,
                           mglc_ctx** out);
/* D2Q9 circles carried through a shear flow: the reference's 2-D case1 step
 * (MPI/Micro_particles/fortran/case1/mpi_complete, main.F90:34-67;
 * commondata.F90:25-34 for the parameters).  Walls at j = 1 and j = ny move at
 * -uwall and +uwall, x is periodic; every circle moves at the prescribed
 * (u0, 0) with no rotation (stationaryFrame) or stays put while the walls move
 * at -uwall-u0 and uwall-u0 (movingFrame); momentum-exchange force and torque
 * are reported, no springs or gravity.  Quadratic (shipped) or linear
 * interpolated bounce-back and refill.  FP64 in the reference's statement
 * order: bitwise its results while circles stay clear of the periodic
 * boundary (the reference's solid mask has no periodic images).  The refill
 * uses the first circle's velocity for every circle, as the reference does.
 * Verbs as for mglc_particle2d_create. */
typedef struct mglc_shear2d_params {
    int total_nx, total_ny;
    double tauf, rho0, rho_solid, radius;
    double u0, uwall;
    int moving_frame;   /* 0: stationaryFrame (shipped), 1: movingFrame */
    int linear;         /* 0: quadratic (shipped), 1: linear */
} mglc_shear2d_params;
int mglc_shear2d_create(const mglc_shear2d_params* p, const double* centers, int np,
                        mglc_ctx** out);
/* D2Q9 MRT lid-driven cavity: the reference's 2-D code
 * (MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked; commondata.f90:4-30
 * for the parameters, tauf = u0*total_nx/reynolds*3 + 0.5).  Lid along +x on
 * the top row (j = ny), initial u = u0 on that row (initial.f90:47-51).  FP64,
 * every statement in the reference's order: bitwise the reference's fields and
 * check() residual.  Verbs: mglc_initial, mglc_load_state (f, and rho,u,v or
 * none), mglc_step, mglc_get_f (9 per node), mglc_get_macros(_device) (w = 0),
 * mglc_check (error_t = 0), mglc_totals. */
typedef struct mglc_lid2d_params {
    int total_nx, total_ny;
    double reynolds, rho0, u0;
    int precision; /* MGLC_FP64 */
} mglc_lid2d_params;
/* Replaces the allocation part of 2d_revised/mpi_blocked/initial.f90:32-38. */
int mglc_lid2d_create(const mglc_lid2d_params* p, mglc_ctx** out);
/* Frees the context's device memory and stream: the deallocate block at the end
 * of the reference's programs (mpi_3d_blocked/main.f90:122-130,
 * bouyancy3d_mpi.F90:303-318).  NULL is ignored. */
void mglc_destroy(mglc_ctx* ctx);
/* No counterpart (the reference writes a message and stops): the message of
 * the context's last failed call, valid until its next call. */
const char* mglc_last_error(const mglc_ctx* ctx);
/* No counterpart: bind the context to a caller-owned cudaStream_t (NULL = the
 * context's own stream). */
int mglc_set_stream(mglc_ctx* ctx, void* cuda_stream);
/* No counterpart: the derived constants the reference prints at start-up
 * (relaxation times, viscosity, ...) and the context's device memory. */
int mglc_get_info(const mglc_ctx* ctx, mglc_info* out);

/* ---- state ------------------------------------------------------------- */
/* Device-side initial(): lid initial.f90:46-73; thermal bouyancy3d_mpi.F90:497-629. */
int mglc_initial(mglc_ctx* ctx);
/* Load a state from host arrays in the reference layout (the reload path
 * bouyancy3d_mpi.F90:598-611).  g is used by thermal contexts only.  rho,u,v,w
 * (and T) are the macroscopic fields the next collision uses; pass NULL for
 * all of them to derive them from f (and g) with the reference macro.  Returns
 * once the host arrays have been read (they may be reused); the conversion to
 * the device layout may still be running on the context's stream. */
int mglc_load_state(mglc_ctx* ctx, const double* f, const double* g, const double* rho,
                    const double* u, const double* v, const double* w, const double* T);
/* Copy the post-stream populations f (and g) back in the reference layout. */
int mglc_get_f(mglc_ctx* ctx, double* f, double* g);

/* ---- the hot path ------------------------------------------------------ */
/* nsteps fused time steps.  Lid: collision + streaming + bounceback + macro
 * (main.f90:89-97).  Thermal: collision, streaming, bounceback, collisionT,
 * streamingT, bouncebackT, macro, macroT (bouyancy3d_mpi.F90:226-244).
 * Particles: collision, streaming, bounceback, bounceback_particle, macro,
 * calForce, updateCenter (case4 main.F90:37-71).  Asynchronous on the
 * context's stream, except for particle contexts, which synchronise at the
 * end to report MGLC_ERR_PARTICLE (overlap, wall penetration). */
int mglc_step(mglc_ctx* ctx, int nsteps);

/* macro() / macroT() output (lid macro.f90:6-25; thermal bouyancy3d_mpi.F90:
 * 986-1010 and 1215-1231): rho,u,v,w (and T) of the current state, host
 * arrays (x fastest).  Any pointer may be NULL.  Synchronises. */
int mglc_get_macros(mglc_ctx* ctx, double* rho, double* u, double* v, double* w, double* T);
/* check(): lid check.f90:12-30 (errorU over u,v only in the numerator);
 * thermal bouyancy3d_mpi.F90:1234-1281 (errorU over u,v,w; errorT).  Updates
 * the stored previous fields like the reference.  error_t may be NULL. */
int mglc_check(mglc_ctx* ctx, double* error_u, double* error_t);
/* No counterpart (a conservation check for tests and monitoring): totals in
 * FP64, mass = sum rho, energy = sum rho|u|^2/2, heat = sum T (thermal, else
 * 0).  Any pointer may be NULL. */
int mglc_totals(mglc_ctx* ctx, double* mass, double* energy, double* heat);

/* Particle centres, velocities, angular velocities, and the total force and
 * torque of the last step (particle_force.F90:184-190), each np x 3 doubles.
 * Any pointer may be NULL.  Synchronises. */
int mglc_particle_state(mglc_ctx* ctx, double* xc, double* uc, double* omega, double* force,
                        double* torque);
/* Owner of every node: -1 fluid, p >= 0 inside particle p (the reference's
 * obst, particle_update.F90:80-93, with the particle index).  Synchronises. */
int mglc_get_mask(mglc_ctx* ctx, int* owner);

/* Thermal statistics of the current state.  nu_vol and re_vol restate the
 * reference's calNuRe (mpi_blocked/RaNu.F90:13-47): Nu = <w T> nz/kappa + 1,
 * Re = sqrt(<|u|^2>) nz/nu.  nu_hot / nu_cold are wall Nusselt numbers at the
 * constant-temperature walls (no reference counterpart): -L/dT times the
 * wall-averaged temperature gradient, taken second order at the halfway wall.
 * Any pointer may be NULL.  Synchronises. */
int mglc_nusselt(mglc_ctx* ctx, double* nu_vol, double* re_vol, double* nu_hot, double* nu_cold);

/* ---- output, checkpoint/restart, statistics (host side) ------------------ */
/* Tecplot binary (.plt, "#!TDV101", one zone, point packing, 32-bit floats)
 * of the current fields: lid X Y Z U V W Pressure (= rho/3)
 * (mpi_3d_blocked/output.f90:175-296); heated X Y Z U V W T
 * (Buoyancy_driven_cavity/fortran/3d/seq/bouyancy3d.F90:1034-1164).  Node
 * coordinates x_i = i - 0.5.  Synchronises. */
int mglc_write_tecplot(mglc_ctx* ctx, const char* path);
/* The same writer on host arrays (x fastest); s = rho (thermal = 0) or T. */
int mglc_tecplot_write_fields(const char* path, int nx, int ny, int nz, const double* u,
                              const double* v, const double* w, const double* s, int thermal);
/* Centre-line profiles of getVelocity (output.f90:318-347): u(nx/2,ny/2,z)/U0
 * against z/nz, and x/nx against w(x,ny/2,nz/2)/U0, one pair per line. */
int mglc_write_profiles(mglc_ctx* ctx, const char* uz_path, const char* xw_path, double u0);
int mglc_profiles_write_fields(const char* uz_path, const char* xw_path, int nx, int ny, int nz,
                               const double* u, const double* w, double u0);
/* output_binary: Fortran unformatted sequential records, lid u, v, rho
 * (output.f90:350-367), heated u, v, w, T (bouyancy3d.F90:984-1008). */
int mglc_write_binary(mglc_ctx* ctx, const char* path);
/* backupData (bouyancy3d.F90:1011-1030): records u, v, w, T, f(0:18,...),
 * g(0:6,...) (lid contexts: u, v, w, f).  Records follow gfortran's layout:
 * 4-byte markers, subrecords of at most 2^31-9 bytes. */
int mglc_backup_save(mglc_ctx* ctx, const char* path);
/* Reload (bouyancy3d.F90:367-379): f, g and u, v, w, T from the file with
 * rho = 1 (:289); the next step collides with those fields, as the reference
 * does after a reload. */
int mglc_backup_load(mglc_ctx* ctx, const char* path);
/* The record writer/reader on host arrays; T and g may be NULL (omitted).
 * max_subrecord: subrecord payload limit in bytes, 0 = 2^31-9 (gfortran). */
int mglc_backup_write_fields(const char* path, int nx, int ny, int nz, const double* u,
                             const double* v, const double* w, const double* T, const double* f,
                             const double* g, long long max_subrecord);
int mglc_backup_read_fields(const char* path, int nx, int ny, int nz, double* u, double* v,
                            double* w, double* T, double* f, double* g);

/* calNuRe statistics (bouyancy3d.F90:1185-1321), one sample per time unit:
 * running means of Nu and Re, statistical stationarity (means change < 1%
 * over 100 samples, tested every 100) and convergence (first- and last-half
 * means of the stationary window within 1%, tested every 200 samples; with
 * flow reversal, not before flow_reversal_time samples after stationarity). */
typedef struct mglc_nure_monitor mglc_nure_monitor;
typedef struct mglc_nure_status {
    int time;                       /* samples so far (dimensionlessTime) */
    double nu, re, nu_mean, re_mean;
    int stationary, stationary_time, converged;
    double nu_half_change, re_half_change; /* relative change tested now, else -1 */
    double nu_mean_change, re_mean_change; /* relative change tested now, else -1 */
} mglc_nure_status;
int mglc_nure_create(int flow_reversal, int flow_reversal_time, mglc_nure_monitor** out);
void mglc_nure_destroy(mglc_nure_monitor* m);
/* add one sample (Nu, Re); out may be NULL */
int mglc_nure_push(mglc_nure_monitor* m, double nu, double re, mglc_nure_status* out);
/* sample a heated context (mglc_nusselt's Nu and Re on the device) and push */
int mglc_nure_sample(mglc_nure_monitor* m, mglc_ctx* ctx, mglc_nure_status* out);

/* ---- device-resident variants (no host copies) --------------------------- */
/* Same as mglc_get_macros but into device buffers of nx*ny*nz doubles. */
int mglc_get_macros_device(mglc_ctx* ctx, double* rho, double* u, double* v, double* w,
                           double* T);

/* ---- solve server: continuous batching of cavity solves ------------------- */
/* No counterpart in the reference (each reference run is one solve).  A
 * server keeps many lid-driven and heated-cavity solves resident in a device
 * arena of hbm_budget_bytes, admits arriving requests as slots and memory
 * free up, advances all active solves together in one persistent tile-queue
 * kernel per step (K steps per CUDA-graph replay), and retires each solve when
 * max|u - u_prev|/U over the last K steps falls below tol or at max_steps.
 * Lid solves: U = 0.1 on the top z plane, u = 0 initially.  Heated solves:
 * Pr = 0.71, Ma = 0.1, walls at y = 1 / ny with T = +0.5 / -0.5, U = the
 * free-fall velocity sqrt(g beta n). */
typedef struct mglc_server mglc_server;
typedef struct mglc_server_params {
    long long hbm_budget_bytes; /* device arena for resident solves */
    int max_active;             /* solve slots (<= 256) */
    int precision;              /* MGLC_FP16, MGLC_BF16, MGLC_FP16S, MGLC_BF16S or MGLC_FP32 storage of f */
    int steps_per_iteration;    /* K (even): steps between admission/retirement points */
    double tol;                 /* convergence threshold of max|du|/U */
    long long max_steps;        /* step cap of one solve */
    int autotune;               /* 1: time tile shapes on the first run and keep the fastest */
    int keep_results;           /* 1: keep rho,u,v,w(,T) of each retired solve on the host */
    int in_place;               /* 1: AA-pattern streaming, one population buffer per solve
                                   (about twice the solves per budget; identical results) */
} mglc_server_params;
typedef struct mglc_request {
    int kind;         /* MGLC_KIND_LID or MGLC_KIND_THERMAL */
    int n;            /* cubic grid, n^3 nodes */
    double reynolds;  /* lid: Re based on n */
    double rayleigh;  /* heated: Ra */
    double arrival_s; /* arrival time, seconds after the first mglc_server_run */
} mglc_request;
typedef struct mglc_request_result {
    long long id;
    int kind, n;
    long long steps;
    double residual;
    double arrival_s, admit_s, finish_s; /* seconds after the first mglc_server_run */
    int converged;
} mglc_request_result;
typedef struct mglc_server_stats {
    long long iterations, steps_total, cell_updates;
    double wall_s, busy_s;
    int tile_threads, tile_rows, ctas_per_sm; /* the tile shape in use */
    long long peak_device_bytes;
    int peak_active;
} mglc_server_stats;
int mglc_server_create(const mglc_server_params* p, mglc_server** out);
void mglc_server_destroy(mglc_server* s);
const char* mglc_server_last_error(const mglc_server* s);
int mglc_server_submit(mglc_server* s, const mglc_request* r, long long* id);
/* Serve until every submitted request has retired (or time_limit_s passes). */
int mglc_server_run(mglc_server* s, double time_limit_s);
int mglc_server_results(mglc_server* s, mglc_request_result* out, int max, int* count);
/* rho, u, v, w (and T) planes of a retired request, n^3 floats each. */
int mglc_server_get_field(mglc_server* s, long long id, float* out);
int mglc_server_get_stats(mglc_server* s, mglc_server_stats* out);

/* ---- no-allocation variant ----------------------------------------------- */
/* No counterpart in the reference.  The residual of check() (errorU, and errorT
 * when T and Tp are given) over caller-owned DEVICE arrays of n cells, for
 * callers that cannot allocate device memory: hosts whose device memory is
 * owned by another runtime's fixed pool, or latency-critical loops that must
 * not pay cudaMalloc's implicit synchronisation.  Allocates nothing: the
 * reduction's partial sums live in a static device array (512 KiB + 32 B per
 * GPU, held until exit).  n is limited to 67,108,864 cells; larger n returns
 * MGLC_ERR_INVALID.  with_w = 0 is the lid residual (w left out of the
 * numerator), 1 the thermal one.  up, vp, wp (and Tp) receive the current
 * fields like the reference's check().  All calls share the static array:
 * calls that overlap on the GPU race.  The first call in each CUDA context on
 * a device looks up the array's address (cached under the context's unique
 * id); make that first call before any stream capture.  Synchronises
 * cuda_stream (NULL = legacy default stream).  The ratios are written as
 * computed; when either is not finite (a non-finite field, or sum |u|^2 or
 * sum |T| equal to zero) the call returns MGLC_ERR_NUMERIC.  On failure a
 * message is written to errbuf (may be NULL). */
int mglc_residual_noalloc(long long n, const double* u, const double* v, const double* w,
                          const double* T, double* up, double* vp, double* wp, double* Tp,
                          int with_w, void* cuda_stream, double* error_u, double* error_t,
                          char* errbuf, int errbuf_len);

/* ---- sequential sums ------------------------------------------------------ */
/* No counterpart in the reference's interface: the primitive behind the 2-D
 * particle step's density averages (the rhoAvg loops of case4
 * seq_piece/particle_bounceback.F90:14-26 and particle_update.F90:80-92, run
 * single-threaded), exposed so it can be tested on its own.
 * *sum = x[t0] + x[t1] + ... over the t with keep[t] != 0, in increasing t,
 * rounded after every addition exactly as that loop rounds it, computed in
 * parallel on the GPU; *count = the number of kept addends.  x and keep are
 * HOST arrays of n entries.  Synchronises the device. */
int mglc_sequential_sum(const double* x, const int* keep, int n, double* sum, long long* count);

#ifdef __cplusplus
}
#endif
#endif
