// k_step_aa.cu -- the lid-driven cavity step in place (AA pattern): one
// population buffer instead of two, the arithmetic of the push kernel.
//
// A step alternates between two kernels (step_cell.cuh, lid_load_aa and the
// SWAP_STORE path of lid_cell_from): the even kernel reads and writes each
// cell's own slots, the odd kernel reads upstream slots and writes
// downstream ones.  k_aa_swap turns the buffer left by an even step into the
// post-stream layout (the reference's f), which getters and checkpoints read.
// Same reference routines as k_step.cu (mpi_3d_blocked/{collision.f90:15-202,
// streaming.f90:8-20, bounce_back.f90:6-83, macro.f90:6-25}).
#include "step_cell.cuh"

namespace mglc {

template <typename S, bool FIRST, typename IDX, bool SR, bool ODD>
__global__ void __launch_bounds__(128, LidMinBlocks<S>::value)
    k_lid_step_aa(S* f, StepK<typename St<S>::C> K, IDX P, const double* __restrict__ mrho,
                  const double* __restrict__ mu, const double* __restrict__ mv,
                  const double* __restrict__ mw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    S raw[Q19];  // every load is issued before the first store
    lid_load_aa<S, IDX, ODD>(i, j, k, f, K.nx, K.ny, K.nz, P, raw);
    lid_cell_from<S, FIRST, IDX, SR, !ODD>(i, j, k, raw, f, K, P, mrho, mu, mv, mw, K.seed);
}

// FX64 lid cavity in place (FP64 storage, Q55 collision)
template <bool FIRST, typename IDX, bool ODD>
__global__ void __launch_bounds__(128, 4)
    k_lid_step_fx_aa(double* f, FxK K, IDX P, const double* __restrict__ mrho,
                     const double* __restrict__ mu, const double* __restrict__ mv,
                     const double* __restrict__ mw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    lid_cell_fx<FIRST, IDX, ODD ? 2 : 1>(i, blockIdx.y, blockIdx.z, f, f, K, P, mrho, mu, mv, mw);
}

// FX64 heated cavity in place (4 blocks of 128 per SM, as the two-buffer kernel)
template <bool FIRST, bool ROT, typename IDX, bool ODD>
__global__ void __launch_bounds__(128, 4)
    k_thermal_step_fx_aa(double* f, double* g, double* __restrict__ F, FxTK K, IDX P,
                         const double* __restrict__ mrho, const double* __restrict__ mu,
                         const double* __restrict__ mv, const double* __restrict__ mw,
                         const double* __restrict__ mT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    thermal_cell_fx<FIRST, ROT, IDX, ODD ? 2 : 1>(i, blockIdx.y, blockIdx.z, f, f, g, g, F, K, P,
                                                  mrho, mu, mv, mw, mT);
}

// Heated cavity in place: flow and temperature populations each on one
// buffer; the carried force is the cell's own (read, then written).
template <typename S, bool FIRST, bool ROT, typename IDX, bool SR, bool ODD>
__global__ void __launch_bounds__(128)
    k_thermal_step_aa(S* f, typename St<S>::C* g, typename St<S>::C* __restrict__ F,
                      StepK<typename St<S>::C> K, IDX P, const double* __restrict__ mrho,
                      const double* __restrict__ mu, const double* __restrict__ mv,
                      const double* __restrict__ mw, const double* __restrict__ mT) {
    using C = typename St<S>::C;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    C fv[Q19], gv[Q7], fp[3];  // every load is issued before the first store
    thermal_load_aa<S, IDX, ODD, ROT>(i, j, k, f, g, F, (IDX)2 * P, K, P, fv, gv, fp);
    thermal_cell_from<S, FIRST, ROT, IDX, SR, !ODD>(i, j, k, fv, gv, fp, f, g, F, K, P, mrho, mu,
                                                    mv, mw, mT, (IDX)2 * P, K.seed);
}

// Pairwise exchange (q, x) <-> (opp(q), x - e_q) for the directions with
// opp(q) > q (nine of D3Q19, three of D3Q7): the streaming half of a step,
// without collision.  The pair is owned by the thread of x, so the exchange
// is race-free; where x - e_q is outside, slot q of x already holds the
// reflected population.
template <typename S, int Q, typename IDX>
__global__ void __launch_bounds__(128) k_aa_swap(S* f, int nx, int ny, int nz, IDX P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
#pragma unroll
    for (int q = 1; q < Q; q++) {
        if (opp19(q) < q) continue;
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(-dx, -dy, -dz)) != 0) continue;
        const IDX ia = (IDX)q * P + cell;
        const IDX ib = (IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) - (IDX)dz * sz;
        if (oob(ia, (IDX)Q * P) || oob(ib, (IDX)Q * P)) continue;
        S* a = f + ia;
        S* b = f + ib;
        const S t = *a;
        *a = *b;
        *b = t;
    }
}

namespace {

dim3 aa_block(int nx) {
    int bx = ((nx + 31) / 32) * 32;
    if (bx > 128) bx = 128;
    return dim3(bx, 1, 1);
}

template <typename S>
cudaError_t lid_go_aa(bool first, bool odd, void* f, const LidStepArgs& a, cudaStream_t s) {
    using C = typename St<S>::C;
    StepK<C> K = make_k<C>(a.g, a.cd, a.u0, a.rho0, a.scale, a.inv_scale);
    K.seed = a.seed;
    K.sr = a.sr;
    const dim3 b = aa_block(a.g.nx), gr((a.g.nx + b.x - 1) / b.x, a.g.ny, a.g.nz);
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    constexpr bool kHalf = sizeof(S) == 2;  // stochastic rounding: 16-bit storage only
    const bool sr = kHalf && a.sr;
    S* fp = (S*)f;
#define AA_LAUNCH(FI, IT, SRV, OD) \
    k_lid_step_aa<S, FI, IT, SRV, OD><<<gr, b, 0, s>>>(fp, K, (IT)a.g.plane, a.rho, a.u, a.v, a.w)
#define AA_PICK(IT)                                                        \
    if (odd) {                                                             \
        if (sr) AA_LAUNCH(false, IT, kHalf, true);                         \
        else AA_LAUNCH(false, IT, false, true);                            \
    } else if (first) {                                                    \
        if (sr) AA_LAUNCH(true, IT, kHalf, false);                         \
        else AA_LAUNCH(true, IT, false, false);                            \
    } else {                                                               \
        if (sr) AA_LAUNCH(false, IT, kHalf, false);                        \
        else AA_LAUNCH(false, IT, false, false);                           \
    }
    if (small) {
        AA_PICK(unsigned)
    } else {
        AA_PICK(long long)
    }
#undef AA_PICK
#undef AA_LAUNCH
    return cudaGetLastError();
}

cudaError_t lid_go_fx_aa(bool first, bool odd, void* f, const LidStepArgs& a, cudaStream_t s) {
    FxK K;
    K.nx = a.g.nx; K.ny = a.g.ny; K.nz = a.g.nz;
    K.c = make_fx_coef(a.cd, a.u0);
    const dim3 b = aa_block(a.g.nx), gr((a.g.nx + b.x - 1) / b.x, a.g.ny, a.g.nz);
    double* fp = (double*)f;
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
#define FA_LAUNCH(FI, IT, OD) \
    k_lid_step_fx_aa<FI, IT, OD><<<gr, b, 0, s>>>(fp, K, (IT)a.g.plane, a.rho, a.u, a.v, a.w)
    if (small) {
        if (odd) FA_LAUNCH(false, unsigned, true);
        else if (first) FA_LAUNCH(true, unsigned, false);
        else FA_LAUNCH(false, unsigned, false);
    } else {
        if (odd) FA_LAUNCH(false, long long, true);
        else if (first) FA_LAUNCH(true, long long, false);
        else FA_LAUNCH(false, long long, false);
    }
#undef FA_LAUNCH
    return cudaGetLastError();
}

template <typename S, int Q>
cudaError_t swap_go(const Geom& g, void* f, cudaStream_t s) {
    const dim3 b = aa_block(g.nx), gr((g.nx + b.x - 1) / b.x, g.ny, g.nz);
    if ((long long)Q19 * g.plane < (1ll << 31))
        k_aa_swap<S, Q, unsigned><<<gr, b, 0, s>>>((S*)f, g.nx, g.ny, g.nz, (unsigned)g.plane);
    else
        k_aa_swap<S, Q, long long><<<gr, b, 0, s>>>((S*)f, g.nx, g.ny, g.nz, (long long)g.plane);
    return cudaGetLastError();
}

template <typename S>
cudaError_t th_go_aa(bool first, bool odd, void* f, void* g, void* F, const ThermalStepArgs& a,
                     cudaStream_t s) {
    using C = typename St<S>::C;
    StepK<C> K = make_k<C>(a.g, a.cd, 0.0, a.rho0, a.scale, a.inv_scale);
    K.seed = a.seed;
    K.sr = a.sr;
    K.gbeta = (C)a.gbeta; K.omega_rot = (C)a.omega_rot; K.t_ref = (C)a.t_ref;
    K.para_a = (C)a.para_a; K.qd = (C)a.qd; K.qnu = (C)a.qnu;
    K.chot = (C)((6.0 + a.para_a) / 21.0 * a.t_hot);
    K.ccold = (C)((6.0 + a.para_a) / 21.0 * a.t_cold);
    K.bc_y = a.bc_y; K.bc_z = a.bc_z;
    const dim3 b = aa_block(a.g.nx), gr((a.g.nx + b.x - 1) / b.x, a.g.ny, a.g.nz);
    const bool rot = a.omega_rot != 0.0;
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    constexpr bool kHalf = sizeof(S) == 2;
    const bool sr = kHalf && a.sr;
    S* fp = (S*)f;
    C* gp = (C*)g;
    C* Fp = (C*)F;
#define TA_LAUNCH(FI, RO, IT, SRV, OD)                                                       \
    k_thermal_step_aa<S, FI, RO, IT, SRV, OD><<<gr, b, 0, s>>>(fp, gp, Fp, K, (IT)a.g.plane, \
                                                               a.rho, a.u, a.v, a.w, a.T)
#define TA_SR(FI, RO, IT, OD)                        \
    do {                                             \
        if (sr) TA_LAUNCH(FI, RO, IT, kHalf, OD);    \
        else TA_LAUNCH(FI, RO, IT, false, OD);       \
    } while (0)
#define TA_PICK(RO, IT)                              \
    if (odd) TA_SR(false, RO, IT, true);             \
    else if (first) TA_SR(true, RO, IT, false);      \
    else TA_SR(false, RO, IT, false);
    if (small) {
        if (rot) { TA_PICK(true, unsigned) } else { TA_PICK(false, unsigned) }
    } else {
        if (rot) { TA_PICK(true, long long) } else { TA_PICK(false, long long) }
    }
#undef TA_PICK
#undef TA_SR
#undef TA_LAUNCH
    return cudaGetLastError();
}

}  // namespace

// first: the step reads the stored macroscopic fields (after initial/load; the
// layout is then the post-stream one, so first implies an even step)
cudaError_t launch_lid_step_aa(int form, bool first, bool odd, void* f, const LidStepArgs& a,
                               cudaStream_t s) {
    if (first && odd) return cudaErrorInvalidValue;
    switch (form) {
        case FORM_FX64: return lid_go_fx_aa(first, odd, f, a, s);
        case FORM_FP64: return lid_go_aa<double>(first, odd, f, a, s);
        case FORM_FP32: return lid_go_aa<float>(first, odd, f, a, s);
        case FORM_FP16: return lid_go_aa<__half>(first, odd, f, a, s);
        case FORM_BF16: return lid_go_aa<__nv_bfloat16>(first, odd, f, a, s);
    }
    return cudaErrorInvalidValue;
}

namespace {
cudaError_t th_go_fx_aa(bool first, bool odd, void* f, void* g, void* F, const ThermalStepArgs& a,
                        cudaStream_t s) {
    FxTK K;
    K.nx = a.g.nx; K.ny = a.g.ny; K.nz = a.g.nz;
    K.bc_y = a.bc_y; K.bc_z = a.bc_z;
    K.t = make_fx_thermal(a.cd, a.gbeta, a.omega_rot, a.t_ref, a.para_a, a.qd, a.qnu, a.t_hot,
                          a.t_cold);
    const dim3 b = aa_block(a.g.nx), gr((a.g.nx + b.x - 1) / b.x, a.g.ny, a.g.nz);
    const bool rot = a.omega_rot != 0.0;
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    double *fp = (double*)f, *gp = (double*)g, *Fp = (double*)F;
#define TFA_LAUNCH(FI, RO, IT, OD)                                                               \
    k_thermal_step_fx_aa<FI, RO, IT, OD><<<gr, b, 0, s>>>(fp, gp, Fp, K, (IT)a.g.plane, a.rho, a.u, \
                                                          a.v, a.w, a.T)
#define TFA_PICK(RO, IT)                               \
    if (odd) TFA_LAUNCH(false, RO, IT, true);          \
    else if (first) TFA_LAUNCH(true, RO, IT, false);   \
    else TFA_LAUNCH(false, RO, IT, false);
    if (small) {
        if (rot) { TFA_PICK(true, unsigned) } else { TFA_PICK(false, unsigned) }
    } else {
        if (rot) { TFA_PICK(true, long long) } else { TFA_PICK(false, long long) }
    }
#undef TFA_PICK
#undef TFA_LAUNCH
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_thermal_step_aa(int form, bool first, bool odd, void* f, void* g, void* F,
                                   const ThermalStepArgs& a, cudaStream_t s) {
    if (first && odd) return cudaErrorInvalidValue;
    switch (form) {
        case FORM_FX64: return th_go_fx_aa(first, odd, f, g, F, a, s);
        case FORM_FP64: return th_go_aa<double>(first, odd, f, g, F, a, s);
        case FORM_FP32: return th_go_aa<float>(first, odd, f, g, F, a, s);
        case FORM_FP16: return th_go_aa<__half>(first, odd, f, g, F, a, s);
        case FORM_BF16: return th_go_aa<__nv_bfloat16>(first, odd, f, g, F, a, s);
    }
    return cudaErrorInvalidValue;
}

// g (heated cavity): D3Q7 populations in the arithmetic type (FP64 or FP32)
cudaError_t launch_aa_swap(int form, const Geom& g, void* f, void* gt, cudaStream_t s) {
    cudaError_t e = cudaErrorInvalidValue;
    switch (form) {
        case FORM_FP64: e = swap_go<double, Q19>(g, f, s); break;
        case FORM_FP32: e = swap_go<float, Q19>(g, f, s); break;
        case FORM_FP16: e = swap_go<__half, Q19>(g, f, s); break;
        case FORM_BF16: e = swap_go<__nv_bfloat16, Q19>(g, f, s); break;
    }
    if (e != cudaSuccess || !gt) return e;
    return form == FORM_FP64 ? swap_go<double, Q7>(g, gt, s) : swap_go<float, Q7>(g, gt, s);
}

}  // namespace mglc

MGLC_OOB_READER(mglc_oob_hits_k_step_aa)
