// k_step.cu -- fused lattice-Boltzmann step kernels (lid and thermal cavities).
//
// One thread per lattice cell, push scheme: a thread reads its own cell's
// post-stream populations (coalesced SoA loads), derives rho and u (the
// reference macro), collides, and writes each post-collision population to
// the neighbour it streams to.  Populations that would leave the domain are
// reflected in place (halfway bounce-back), which replaces the reference's
// halo exchange + bounceback sweep; the moving-lid term uses the cell's own
// rho, which is the reference's rho(i,j,nz) from the previous macro().
//
// Reference routines fused here (paths relative to the MGLC repository):
//   lid:     mpi_3d_blocked/{collision.f90:15-202, streaming.f90:8-20,
//            bounce_back.f90:6-83, macro.f90:6-25}
//   thermal: bouyancy3d_mpi.F90 collision :641-864, streaming :867-892,
//            bounceback :895-983, collisionT :1014-1070, streamingT :1073-1098,
//            bouncebackT :1101-1210, macro :986-1010, macroT :1215-1231
#include "step_cell.cuh"

namespace mglc {

template <typename S, bool FIRST, typename IDX, bool SR>
__global__ void __launch_bounds__(128, LidMinBlocks<S>::value)
    k_lid_step(const S* __restrict__ fin, S* __restrict__ fout, StepK<typename St<S>::C> K,
               IDX P, const double* __restrict__ mrho, const double* __restrict__ mu,
               const double* __restrict__ mv, const double* __restrict__ mw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    lid_cell<S, FIRST, IDX, SR>(i, blockIdx.y, blockIdx.z, fin, fout, K, P, mrho, mu, mv, mw,
                                K.seed);
}

template <bool FIRST, typename IDX>
__global__ void __launch_bounds__(128)
    k_lid_step_fx(const double* __restrict__ fin, double* __restrict__ fout, FxK K, IDX P,
                  const double* __restrict__ mrho, const double* __restrict__ mu,
                  const double* __restrict__ mv, const double* __restrict__ mw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    lid_cell_fx<FIRST, IDX>(i, blockIdx.y, blockIdx.z, fin, fout, K, P, mrho, mu, mv, mw);
}

// 4 blocks of 128 per SM (128 registers): measured faster than the 168-register
// allocation at 3 blocks and than 5 blocks with spills
template <bool FIRST, bool ROT, typename IDX>
__global__ void __launch_bounds__(128, 4)
    k_thermal_step_fx(const double* __restrict__ fin, double* __restrict__ fout,
                      const double* __restrict__ gin, double* __restrict__ gout,
                      double* __restrict__ F, FxTK K, IDX P, const double* __restrict__ mrho,
                      const double* __restrict__ mu, const double* __restrict__ mv,
                      const double* __restrict__ mw, const double* __restrict__ mT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    thermal_cell_fx<FIRST, ROT, IDX>(i, blockIdx.y, blockIdx.z, fin, fout, gin, gout, F, K, P,
                                     mrho, mu, mv, mw, mT);
}

template <typename S, bool FIRST, bool ROT, typename IDX, bool SR>
__global__ void __launch_bounds__(128)
    k_thermal_step(const S* __restrict__ fin, S* __restrict__ fout,
                   const typename St<S>::C* __restrict__ gin, typename St<S>::C* __restrict__ gout,
                   typename St<S>::C* __restrict__ F, StepK<typename St<S>::C> K, IDX P,
                   const double* __restrict__ mrho, const double* __restrict__ mu,
                   const double* __restrict__ mv, const double* __restrict__ mw,
                   const double* __restrict__ mT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    thermal_cell<S, FIRST, ROT, IDX, SR>(i, blockIdx.y, blockIdx.z, fin, fout, gin, gout, F, K,
                                         P, mrho, mu, mv, mw, mT, (IDX)2 * P, K.seed);
}

// --------------------------------------------------------------- launch --
static dim3 step_block(int nx) {
    int bx = ((nx + 31) / 32) * 32;
    if (bx > 128) bx = 128;
    return dim3(bx, 1, 1);
}
static dim3 step_grid(const Geom& g, dim3 b) {
    return dim3((g.nx + b.x - 1) / b.x, g.ny, g.nz);
}

template <typename S>
static cudaError_t lid_go(bool first, const void* fin, void* fout, const LidStepArgs& a,
                          cudaStream_t s) {
    using C = typename St<S>::C;
    StepK<C> K = make_k<C>(a.g, a.cd, a.u0, a.rho0, a.scale, a.inv_scale);
    K.seed = a.seed;
    K.sr = a.sr;
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    // stochastic rounding exists for the 16-bit storage types only
    constexpr bool kHalf = sizeof(S) == 2;
#define LID_LAUNCH(FI, IT, SRV)                                                          \
    k_lid_step<S, FI, IT, SRV><<<gr, b, 0, s>>>((const S*)fin, (S*)fout, K, (IT)a.g.plane, \
                                                a.rho, a.u, a.v, a.w)
#define LID_SR(FI, IT)                                  \
    if (kHalf && a.sr) LID_LAUNCH(FI, IT, kHalf);        \
    else LID_LAUNCH(FI, IT, false);
    if (small) {
        if (first) { LID_SR(true, unsigned) } else { LID_SR(false, unsigned) }
    } else {
        if (first) { LID_SR(true, long long) } else { LID_SR(false, long long) }
    }
#undef LID_SR
#undef LID_LAUNCH
    return cudaGetLastError();
}

static cudaError_t lid_go_fx(bool first, const void* fin, void* fout, const LidStepArgs& a,
                             cudaStream_t s) {
    FxK K;
    K.nx = a.g.nx; K.ny = a.g.ny; K.nz = a.g.nz;
    K.c = make_fx_coef(a.cd, a.u0);
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    const double* fi = (const double*)fin;
    double* fo = (double*)fout;
#define FX_LAUNCH(FI, IT) \
    k_lid_step_fx<FI, IT><<<gr, b, 0, s>>>(fi, fo, K, (IT)a.g.plane, a.rho, a.u, a.v, a.w)
    if (small) {
        if (first) FX_LAUNCH(true, unsigned); else FX_LAUNCH(false, unsigned);
    } else {
        if (first) FX_LAUNCH(true, long long); else FX_LAUNCH(false, long long);
    }
#undef FX_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_lid_step(int form, bool first, const void* fin, void* fout,
                            const LidStepArgs& a, cudaStream_t s) {
    switch (form) {
        case FORM_FX64: return lid_go_fx(first, fin, fout, a, s);
        case FORM_FP64: return lid_go<double>(first, fin, fout, a, s);
        case FORM_FP32: return lid_go<float>(first, fin, fout, a, s);
        case FORM_FP16: return lid_go<__half>(first, fin, fout, a, s);
        case FORM_BF16: return lid_go<__nv_bfloat16>(first, fin, fout, a, s);
    }
    return cudaErrorInvalidValue;
}

template <typename S>
static cudaError_t th_go(bool first, const void* fin, void* fout, const void* gin, void* gout,
                         void* F, const ThermalStepArgs& a, cudaStream_t s) {
    using C = typename St<S>::C;
    StepK<C> K = make_k<C>(a.g, a.cd, 0.0, a.rho0, a.scale, a.inv_scale);
    K.seed = a.seed;
    K.sr = a.sr;
    K.gbeta = (C)a.gbeta; K.omega_rot = (C)a.omega_rot; K.t_ref = (C)a.t_ref;
    K.para_a = (C)a.para_a; K.qd = (C)a.qd; K.qnu = (C)a.qnu;
    K.chot = (C)((6.0 + a.para_a) / 21.0 * a.t_hot);
    K.ccold = (C)((6.0 + a.para_a) / 21.0 * a.t_cold);
    K.bc_y = a.bc_y; K.bc_z = a.bc_z;
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    const bool rot = a.omega_rot != 0.0;
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    constexpr bool kHalf = sizeof(S) == 2;
#define TH_LAUNCH2(FI, RO, IT, SRV)                                                            \
    k_thermal_step<S, FI, RO, IT, SRV><<<gr, b, 0, s>>>((const S*)fin, (S*)fout, (const C*)gin, \
                                                        (C*)gout, (C*)F, K, (IT)a.g.plane,     \
                                                        a.rho, a.u, a.v, a.w, a.T)
#define TH_LAUNCH(FI, RO, IT)                                   \
    do {                                                        \
        if (kHalf && a.sr) TH_LAUNCH2(FI, RO, IT, kHalf);       \
        else TH_LAUNCH2(FI, RO, IT, false);                     \
    } while (0)
#define TH_ROT(IT)                                       \
    if (first && rot) TH_LAUNCH(true, true, IT);          \
    else if (first) TH_LAUNCH(true, false, IT);           \
    else if (rot) TH_LAUNCH(false, true, IT);             \
    else TH_LAUNCH(false, false, IT);
    if (small) {
        TH_ROT(unsigned)
    } else {
        TH_ROT(long long)
    }
#undef TH_ROT
#undef TH_LAUNCH
#undef TH_LAUNCH2
    return cudaGetLastError();
}

static cudaError_t th_go_fx(bool first, const void* fin, void* fout, const void* gin, void* gout,
                            void* F, const ThermalStepArgs& a, cudaStream_t s) {
    FxTK K;
    K.nx = a.g.nx; K.ny = a.g.ny; K.nz = a.g.nz; K.bc_y = a.bc_y; K.bc_z = a.bc_z;
    K.t = make_fx_thermal(a.cd, a.gbeta, a.omega_rot, a.t_ref, a.para_a, a.qd, a.qnu, a.t_hot,
                          a.t_cold);
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    const bool rot = a.omega_rot != 0.0;
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    const double* fi = (const double*)fin;
    const double* gi = (const double*)gin;
    double* fo = (double*)fout;
    double* go = (double*)gout;
    double* Fp = (double*)F;
#define THX_LAUNCH(FI, RO, IT) \
    k_thermal_step_fx<FI, RO, IT><<<gr, b, 0, s>>>(fi, fo, gi, go, Fp, K, (IT)a.g.plane, a.rho, a.u, a.v, a.w, a.T)
#define THX_ROT(IT)                                 \
    if (first && rot) THX_LAUNCH(true, true, IT);    \
    else if (first) THX_LAUNCH(true, false, IT);     \
    else if (rot) THX_LAUNCH(false, true, IT);       \
    else THX_LAUNCH(false, false, IT);
    if (small) {
        THX_ROT(unsigned)
    } else {
        THX_ROT(long long)
    }
#undef THX_ROT
#undef THX_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_thermal_step(int form, bool first, const void* fin, void* fout,
                                const void* gin, void* gout, void* F, const ThermalStepArgs& a,
                                cudaStream_t s) {
    switch (form) {
        case FORM_FX64: return th_go_fx(first, fin, fout, gin, gout, F, a, s);
        case FORM_FP64: return th_go<double>(first, fin, fout, gin, gout, F, a, s);
        case FORM_FP32: return th_go<float>(first, fin, fout, gin, gout, F, a, s);
        case FORM_FP16: return th_go<__half>(first, fin, fout, gin, gout, F, a, s);
        case FORM_BF16: return th_go<__nv_bfloat16>(first, fin, fout, gin, gout, F, a, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace mglc

MGLC_OOB_READER(mglc_oob_hits_k_step)
