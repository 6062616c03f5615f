// kernels.cuh -- launcher declarations shared by the C-ABI layer and the
// kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "lbm_common.cuh"

namespace mglc {

// Storage forms of the populations (mirrors MGLC_FP64 ... in mglc.h).
// FORM_FX64: FP64 storage (the FP64 layout everywhere) with the Q55
// fixed-point lid collision of fixed64.cuh
enum Form { FORM_FP64 = 0, FORM_FP32 = 1, FORM_FP16 = 2, FORM_BF16 = 3, FORM_FX64 = 4 };

inline size_t form_bytes(int form) { return form == FORM_FP64 ? 8 : form == FORM_FP32 ? 4 : 2; }

struct Geom {
    int nx, ny, nz;
    long long plane;  // elements between population planes (= nx*ny*nz)
};

// Arguments of one fused lid step.
struct LidStepArgs {
    Geom g;
    MrtCoef<double> cd;
    double u0, rho0;
    float scale, inv_scale;  // deviation storage scale (FP16); 1 otherwise
    unsigned seed;           // step index: stochastic rounding of 16-bit stores
    int sr;                  // 1: stochastic rounding of 16-bit stores
    // macroscopic fields used by the first step after initial()/load (the
    // reference's collision reads the stored rho,u,v,w)
    const double *rho, *u, *v, *w;
};

struct ThermalStepArgs {
    Geom g;
    MrtCoef<double> cd;
    double gbeta, omega_rot, t_ref, para_a, qd, qnu, t_hot, t_cold, rho0;
    int bc_y, bc_z;
    float scale, inv_scale;
    unsigned seed;  // step index: stochastic rounding of 16-bit stores
    int sr;         // 1: stochastic rounding of 16-bit stores
    const double *rho, *u, *v, *w, *T;
};

// fused step launchers (fin/fout are the population buffers in the context's form)
// in place (AA pattern, k_step_aa.cu): even/odd step kernels on one buffer,
// and the pairwise swap that restores the post-stream layout after an even step
cudaError_t launch_lid_step_aa(int form, bool first, bool odd, void* f, const LidStepArgs& a,
                               cudaStream_t s);
cudaError_t launch_thermal_step_aa(int form, bool first, bool odd, void* f, void* g, void* F,
                                   const ThermalStepArgs& a, cudaStream_t s);
// gt: the heated cavity's temperature populations (NULL for the lid cavity)
cudaError_t launch_aa_swap(int form, const Geom& g, void* f, void* gt, cudaStream_t s);
cudaError_t launch_lid_step(int form, bool first, const void* fin, void* fout,
                            const LidStepArgs& a, cudaStream_t s);
cudaError_t launch_thermal_step(int form, bool first, const void* fin, void* fout,
                                const void* gin, void* gout, void* F, const ThermalStepArgs& a,
                                cudaStream_t s);

// macroscopic fields from the current state (reference macro()/macroT() order)
cudaError_t launch_macro(int form, bool thermal, const Geom& g, const void* f, const void* gt,
                         const void* F, double rho0, float inv_scale, double* rho, double* u,
                         double* v, double* w, double* T, cudaStream_t s);

// equilibrium initialisation from rho,u,v,w (and T): reference initial()
cudaError_t launch_equilibrium(int form, bool thermal, const Geom& g, const double* rho,
                               const double* u, const double* v, const double* w,
                               const double* T, double para_a, double rho0, float scale, void* f,
                               void* gt, cudaStream_t s);

// layout conversion between the reference AoS (double, population fastest)
// and the device SoA form, for cells [cell0, cell0+ncells)
cudaError_t launch_aos_to_soa(int form, int Q, const Geom& g, long long cell0, long long ncells,
                              const double* aos, void* soa, double rho0, float scale,
                              bool shifted, cudaStream_t s);
cudaError_t launch_soa_to_aos(int form, int Q, const Geom& g, long long cell0, long long ncells,
                              const void* soa, double* aos, double rho0, float inv_scale,
                              bool shifted, cudaStream_t s);

// FP64 reductions with fixed-order, deterministic two-pass sums.
// Residual (reference check()):
//   e[0] = sum (u-up)^2 + (v-vp)^2 [+ (w-wp)^2 if with_w]
//   e[1] = sum u^2+v^2+w^2, e[2] = sum |T-Tp|, e[3] = sum |T|
// and up,vp,wp,Tp <- u,v,w,T.  partials holds reduce_blocks()*4 doubles.
int reduce_blocks(long long n);
cudaError_t launch_residual(long long n, const double* u, const double* v, const double* w,
                            const double* T, double* up, double* vp, double* wp, double* Tp,
                            bool with_w, double* partials, double* out4, cudaStream_t s);
// totals: out[0] = sum rho, out[1] = sum rho|u|^2/2, out[2] = sum T
cudaError_t launch_totals(long long n, const double* rho, const double* u, const double* v,
                          const double* w, const double* T, double* partials, double* out3,
                          cudaStream_t s);

// thermal statistics: out[0] = sum w*T, out[1] = sum |u|^2,
// out[2] = sum over the low const-T wall of (9 T_1 - T_2), out[3] = the same at
// the high wall (9 T_n - T_{n-1}); wall_axis 1 = y, 2 = z, 0 = none
cudaError_t launch_thermal_stats(const Geom& g, const double* u, const double* v, const double* w,
                                 const double* T, int wall_axis, double* partials, double* out4,
                                 cudaStream_t s);

}  // namespace mglc
