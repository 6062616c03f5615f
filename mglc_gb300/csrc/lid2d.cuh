// lid2d.cuh -- the D2Q9 MRT lid-driven cavity of the reference's 2-D code
// (MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked) on the GPU, host side.
//
// One fused kernel per time step: macro (of the previous step), collision,
// streaming and the wall bounce-back with the moving-lid term.  FP64 in the
// reference's expression order, compiled without FMA contraction, so the
// fields are bitwise those of the reference's statements.
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace mglc {

struct L2Params {
    int nx, ny;
    double tauf, snu, sq, u0, rho0;
};

struct L2Ctx;  // device state (k_lid2d.cu)

int l2d_create(const L2Params& p, L2Ctx** out, std::string& err);
void l2d_destroy(L2Ctx* c);
int l2d_set_stream(L2Ctx* c, cudaStream_t s);
int l2d_initial(L2Ctx* c, std::string& err);
// f: (ny, nx, 9) population fastest; rho/u/v: (ny, nx) or all NULL (derived from f)
int l2d_load(L2Ctx* c, const double* f, const double* rho, const double* u, const double* v,
             std::string& err);
int l2d_step(L2Ctx* c, int nsteps, std::string& err);
int l2d_get_f(L2Ctx* c, double* f, std::string& err);
int l2d_get_macros(L2Ctx* c, double* rho, double* u, double* v, double* w, std::string& err);
// device pointers of (ny, nx) FP64 arrays (any may be NULL; w is zeroed); synchronises
int l2d_get_macros_device(L2Ctx* c, double* rho, double* u, double* v, double* w,
                          std::string& err);
int l2d_check(L2Ctx* c, double* error_u, std::string& err);
long long l2d_itc(const L2Ctx* c);
long long l2d_device_bytes(const L2Ctx* c);

}  // namespace mglc
