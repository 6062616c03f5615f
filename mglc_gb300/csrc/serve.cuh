// serve.cuh -- device side of the solve server: a table of resident solves
// (lid-driven and heated cavities of different sizes) advanced together by one
// persistent tile-queue kernel per time step.
#pragma once
#include <cuda_runtime.h>

#include "step_cell.cuh"

namespace mglc {

constexpr int SERVE_MAX_ACTIVE = 256;

// One resident solve.  Populations f are FP16 or FP32 deviations (the
// server's form), temperature populations g and the carried F_z are FP32.
struct ServeSolve {
    int kind;  // MGLC_KIND_LID (1) or MGLC_KIND_THERMAL (2)
    int nx, ny, nz;
    unsigned plane;
    int tile0, ntiles;  // first tile index in the queue, tiles of this solve
    void* f[2];
    float* g[2];
    float* F;      // F_z (no rotation in served solves)
    float* uprev;  // 3 planes: velocity at the previous residual check
    float uref;    // velocity scale of the residual
    unsigned step0;  // steps taken before this iteration (stochastic-rounding seed base)
    StepK<float> K;
};

// Active solves, lid-driven ones first: tiles [0, lid_tiles) belong to lid
// solves, tiles [lid_tiles, total_tiles) to heated ones.
struct ServeTable {
    int n_active;
    int total_tiles;
    int lid_tiles;
    int rows_per_tile;
    ServeSolve s[SERVE_MAX_ACTIVE];
};

// Time step k of the iteration for every active solve of one kind (k & 1
// selects the ping-pong buffer, step0 + k seeds the stochastic rounding);
// thermal = 0 runs the lid tiles, 1 the heated ones.
cudaError_t launch_serve_step(int form, int sr, int aa, int thermal, const ServeTable* tab, int k,
                              unsigned* counter, int grid, int block, cudaStream_t st);
// resid[s] = max over cells of |u - uprev| / uref (as float bits); uprev <- u;
// then every solve's step0 advances by steps (the iteration's step count)
cudaError_t launch_serve_resid(int form, ServeTable* tab, unsigned* counter, unsigned* resid,
                               int steps, int grid, int block, cudaStream_t st);
// equilibrium state of one solve (rho = 1, u = 0; wall temperatures)
cudaError_t launch_serve_init(int form, const ServeSolve& s, double t_hot, double t_cold,
                              cudaStream_t st);
// rho, u, v, w (and T) of one solve as FP32 into out (4 or 5 planes)
cudaError_t launch_serve_fields(int form, const ServeSolve& s, float* out, cudaStream_t st);

}  // namespace mglc
