// particles2d.cuh -- the D2Q9 moving-circle step of the reference's case4
// (MPI/Micro_particles/fortran/case4/mpi_particle) on the GPU, host side.
//
// This variant reproduces the reference's own 2-D algorithm statement by
// statement: bisection or analytic q, quadratic interpolated bounce-back
// reading the persistent post-collision array (solid nodes keep their last
// values), Wen 2014 momentum exchange, the case4 springs and gravity, the
// explicit update and the sequential refill.  All arithmetic is FP64 without
// contraction, in the reference's expression order, so results are bitwise
// those of the reference statements.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace mglc {

enum { P2_SETTLING = 0, P2_SHEAR = 1 };

struct P2Params {
    int nx, ny, np;
    int q_bisection;  // 1: calQ (bisection), 0: calQ2 (ray-circle root)
    double tauf, rho0, rho_solid, radius, gravity;  // gravity: magnitude along -y
    double threshold_wall, stiff_wall, threshold_particle, stiff_particle;
    double snu, sq, pi;
    // P2_SHEAR (case1/mpi_complete): circles carried at u0 through the shear
    // between walls moving at -/+uwall, periodic x, no springs or gravity
    int variant;       // P2_SETTLING (case4) or P2_SHEAR (case1)
    int moving_frame;  // case1 movingFrame (1) or stationaryFrame (0)
    int linear;        // case1 linear (1) or quadratic (0) bounce-back and refill
    double u0, uwall;
};

struct P2Ctx;  // device state (k_particle2d.cu)

int p2d_create(const P2Params& p, const double* centers_xy, P2Ctx** out, std::string& err);
void p2d_destroy(P2Ctx* c);
int p2d_set_stream(P2Ctx* c, cudaStream_t s);
int p2d_initial(P2Ctx* c, std::string& err);
// returns MGLC_OK or MGLC_ERR_PARTICLE (err holds the reason)
int p2d_step(P2Ctx* c, int nsteps, std::string& err);
int p2d_get_f(P2Ctx* c, double* f, std::string& err);  // (ny, nx, 9), population fastest
int p2d_get_macros(P2Ctx* c, double* rho, double* u, double* v, double* w, std::string& err);
int p2d_state(P2Ctx* c, double* xc, double* uc, double* omega, double* force, double* torque,
              std::string& err);  // np x 3 each (z components 0)
int p2d_mask(P2Ctx* c, int* owner, std::string& err);  // -1 fluid, else first owning circle
long long p2d_itc(const P2Ctx* c);
double p2d_rho_avg(P2Ctx* c);
long long p2d_device_bytes(const P2Ctx* c);

}  // namespace mglc
