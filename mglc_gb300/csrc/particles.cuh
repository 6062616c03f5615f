// particles.cuh -- device state of the moving-particle path (D3Q19 spheres)
// shared by k_particle.cu and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mglc {

// CTAs per particle in the boundary-link kernel (z slabs of the node box);
// the link sums are kept per (particle, slab) and added in slab order
constexpr int PART_NSLAB = 4;

// Status codes written by the particle kernels (mirrors orc_pt_step's codes).
enum PartStatus {
    PS_OK = 0,
    PS_NO_OWNER = 1,
    PS_Q_RANGE = 2,
    PS_OVERLAP = 3,
    PS_WALL = 4,
    PS_NO_REFILL_DIR = 5,
    PS_REFILL_FULL = 6,
    PS_DIVERGED = 7,  // a centre, velocity or spin is not finite, or a centre
                      // moved half the periodic length or more in one step
};

struct PartParams {
    int nx, ny, nz, periodic_x, np;
    double rho0, rho_solid, radius, pi;
    double gravity[3], body_force[3];
    double thr_wall, thr_part, scale_wall, scale_part;
    double snu, sq;
};

struct PartDev {
    int* owner_cur;   // -1 fluid, p >= 0 solid node of particle p (interior cells)
    int* owner_new;
    double *xc, *uc, *om;              // np*3, current
    double *xc_old, *uc_old, *om_old;  // np*3
    double *flink, *tlink, *corr;      // np*PART_NSLAB*3 (x2), np*PART_NSLAB: link sums per slab
    double *ftot, *ttot;               // np*3: total force and torque of the last step
    double* prep_sum;                  // np: refill bookkeeping (density)
    int* prep_cnt;                     // np: refill bookkeeping (fluid count change)
    double* partials;                  // bulk-kernel block partials, 2 per block
    int nblocks;                       // number of bulk-kernel partial slots (one per warp)
    long long* n_fluid;                // device scalar
    double* rho_avg;                   // device scalars: [0] at bounce-back, [1] after update
    int* status;                       // device: [0] code, [1] particle, [2] other particle
};

// one fused step of the particle flow (collide + stream + bounce-back on
// walls, interpolated bounce-back and momentum exchange on particles,
// particle update, mask rebuild, refill)
cudaError_t launch_particle_step(int form, bool first, const void* fin, void* fout,
                                 const PartParams& p, const PartDev& d, cudaStream_t s);
// initial state: owner mask from the centres, equilibrium populations,
// fluid count
cudaError_t launch_particle_init(int form, void* f, const PartParams& p, const PartDev& d,
                                 cudaStream_t s);
// macroscopic fields (solid nodes: rho_solid, u = 0); first = the state
// before the first step (fluid rho0, u = 0)
cudaError_t launch_particle_macro(int form, bool first, const void* f, const PartParams& p,
                                  const PartDev& d, double* rho, double* u, double* v, double* w,
                                  cudaStream_t s);
int particle_bulk_blocks(const PartParams& p);  // per-warp partial slots

}  // namespace mglc
