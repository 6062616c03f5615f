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
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kernels.cuh"

namespace mglc {

// ---------------------------------------------------------------- storage --
template <typename S>
struct St;
template <>
struct St<double> {
    using C = double;
    static constexpr bool SHIFT = false;
    __device__ static C ld(const double* p, float) { return __ldg(p); }
    __device__ static void st(double* p, C v, float) { *p = v; }
};
template <>
struct St<float> {
    using C = float;
    static constexpr bool SHIFT = true;
    __device__ static C ld(const float* p, float) { return __ldg(p); }
    __device__ static void st(float* p, C v, float) { *p = v; }
};
template <>
struct St<__half> {
    using C = float;
    static constexpr bool SHIFT = true;
    __device__ static C ld(const __half* p, float inv) { return __half2float(__ldg(p)) * inv; }
    __device__ static void st(__half* p, C v, float sc) { *p = __float2half_rn(v * sc); }
};
template <>
struct St<__nv_bfloat16> {
    using C = float;
    static constexpr bool SHIFT = true;
    __device__ static C ld(const __nv_bfloat16* p, float inv) {
        return __bfloat162float(__ldg(p)) * inv;
    }
    __device__ static void st(__nv_bfloat16* p, C v, float sc) { *p = __float2bfloat16_rn(v * sc); }
};

template <typename C>
__device__ __forceinline__ C recip(C x) {
    return C(1) / x;
}

// ------------------------------------------------------------ lid kernel --
template <typename S, bool FIRST>
__global__ void __launch_bounds__(128) k_lid_step(const S* __restrict__ fin, S* __restrict__ fout,
                                                  LidStepArgs a, MrtCoef<typename St<S>::C> c) {
    using C = typename St<S>::C;
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= nx) return;
    const long long P = a.g.plane;
    const long long cell = i + (long long)nx * (j + (long long)ny * k);
    C f[Q19];
#pragma unroll
    for (int q = 0; q < Q19; q++) f[q] = St<S>::ld(fin + q * P + cell, a.inv_scale);
    C rho_m, rho, ux, uy, uz;
    if (FIRST) {
        rho = (C)a.rho[cell];
        ux = (C)a.u[cell];
        uy = (C)a.v[cell];
        uz = (C)a.w[cell];
        rho_m = St<S>::SHIFT ? rho - (C)a.rho0 : rho;
    } else {
        C jx, jy, jz;
        moments0(f, rho_m, jx, jy, jz);
        rho = St<S>::SHIFT ? (C)a.rho0 + rho_m : rho_m;
        const C inv = recip(rho);
        ux = jx * inv;
        uy = jy * inv;
        uz = jz * inv;
    }
    mrt_collide<C, false, true>(f, rho_m, rho, ux, uy, uz, C(0), C(0), C(0), c);
    // moving lid: f(14) = f_post(11) - rho/6*U0, f(13) = f_post(12) + rho/6*U0 (bounce_back.f90:77-78)
    C lid = C(0);
    if (k == nz - 1) lid = rho / C(6) * (C)a.u0;
    const long long sy = nx, sz = (long long)nx * ny;
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        bool in = true;
        if (dx > 0) in = in && (i + 1 < nx);
        if (dx < 0) in = in && (i > 0);
        if (dy > 0) in = in && (j + 1 < ny);
        if (dy < 0) in = in && (j > 0);
        if (dz > 0) in = in && (k + 1 < nz);
        if (dz < 0) in = in && (k > 0);
        if (in) {
            St<S>::st(fout + q * P + cell + dx + dy * sy + dz * sz, f[q], a.scale);
        } else {
            C val = f[q];
            if (dz > 0 && dx != 0) val = val - C(dx) * lid;  // lid face written last: wins on edges
            St<S>::st(fout + opp19(q) * P + cell, val, a.scale);
        }
    }
}

// -------------------------------------------------------- thermal kernel --
template <typename S, bool FIRST, bool ROT>
__global__ void __launch_bounds__(128)
    k_thermal_step(const S* __restrict__ fin, S* __restrict__ fout, const S* __restrict__ gin,
                   S* __restrict__ gout, typename St<S>::C* __restrict__ F, ThermalStepArgs a,
                   MrtCoef<typename St<S>::C> c) {
    using C = typename St<S>::C;
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= nx) return;
    const long long P = a.g.plane;
    const long long cell = i + (long long)nx * (j + (long long)ny * k);
    C f[Q19], g[Q7];
#pragma unroll
    for (int q = 0; q < Q19; q++) f[q] = St<S>::ld(fin + q * P + cell, a.inv_scale);
#pragma unroll
    for (int q = 0; q < Q7; q++) g[q] = St<S>::ld(gin + q * P + cell, 1.0f);
    C rho_m, rho, ux, uy, uz, temp;
    if (FIRST) {
        rho = (C)a.rho[cell];
        ux = (C)a.u[cell];
        uy = (C)a.v[cell];
        uz = (C)a.w[cell];
        temp = (C)a.T[cell];
        rho_m = St<S>::SHIFT ? rho - (C)a.rho0 : rho;
    } else {
        C jx, jy, jz;
        moments0(f, rho_m, jx, jy, jz);
        rho = St<S>::SHIFT ? (C)a.rho0 + rho_m : rho_m;
        const C inv = recip(rho);
        // u^n = (sum f e + F^n/2)/rho^n with the force carried from the previous step
        C fxp = C(0), fyp = C(0);
        if (ROT) {
            fxp = F[cell];
            fyp = F[P + cell];
        }
        const C fzp = F[2 * P + cell];
        ux = (jx + C(0.5) * fxp) * inv;
        uy = (jy + C(0.5) * fyp) * inv;
        uz = (jz + C(0.5) * fzp) * inv;
        temp = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + g[6]);
    }
    // body force from (rho,u,T) of the previous macro (bouyancy3d_mpi.F90:743-745)
    C fx = C(0), fy = C(0);
    if (ROT) {
        fx = C(-2) * rho * uy * (C)a.omega_rot;
        fy = C(2) * rho * ux * (C)a.omega_rot;
        F[cell] = fx;
        F[P + cell] = fy;
    }
    const C fz = rho * (C)a.gbeta * (temp - (C)a.t_ref);
    F[2 * P + cell] = fz;
    mrt_collide<C, true, false>(f, rho_m, rho, ux, uy, uz, fx, fy, fz, c);
    mrt_collide_t<C>(g, temp, ux, uy, uz, (C)a.para_a, (C)a.qd, (C)a.qnu);

    const long long sy = nx, sz = (long long)nx * ny;
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        bool in = true;
        if (dx > 0) in = in && (i + 1 < nx);
        if (dx < 0) in = in && (i > 0);
        if (dy > 0) in = in && (j + 1 < ny);
        if (dy < 0) in = in && (j > 0);
        if (dz > 0) in = in && (k + 1 < nz);
        if (dz < 0) in = in && (k > 0);
        if (in)
            St<S>::st(fout + q * P + cell + dx + dy * sy + dz * sz, f[q], a.scale);
        else
            St<S>::st(fout + opp19(q) * P + cell, f[q], a.scale);
    }
    // D3Q7: adiabatic walls reflect, constant-T walls anti-bounce-back
    // g_in = -g_out + (6+paraA)/21 * T_wall (bouyancy3d_mpi.F90:1101-1210)
    const C chot = (C)((6.0 + a.para_a) / 21.0 * a.t_hot);
    const C ccold = (C)((6.0 + a.para_a) / 21.0 * a.t_cold);
#pragma unroll
    for (int q = 0; q < Q7; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        bool in = true;
        if (dx > 0) in = in && (i + 1 < nx);
        if (dx < 0) in = in && (i > 0);
        if (dy > 0) in = in && (j + 1 < ny);
        if (dy < 0) in = in && (j > 0);
        if (dz > 0) in = in && (k + 1 < nz);
        if (dz < 0) in = in && (k > 0);
        if (in) {
            St<S>::st(gout + q * P + cell + dx + dy * sy + dz * sz, g[q], 1.0f);
        } else {
            C val = g[q];
            if (dy != 0 && a.bc_y) val = -val + (dy < 0 ? chot : ccold);
            if (dz != 0 && a.bc_z) val = -val + (dz < 0 ? chot : ccold);
            St<S>::st(gout + opp19(q) * P + cell, val, 1.0f);
        }
    }
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
    MrtCoef<C> c = cast_coef<C>(a.cd);
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    if (first)
        k_lid_step<S, true><<<gr, b, 0, s>>>((const S*)fin, (S*)fout, a, c);
    else
        k_lid_step<S, false><<<gr, b, 0, s>>>((const S*)fin, (S*)fout, a, c);
    return cudaGetLastError();
}

cudaError_t launch_lid_step(int form, bool first, const void* fin, void* fout,
                            const LidStepArgs& a, cudaStream_t s) {
    switch (form) {
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
    MrtCoef<C> c = cast_coef<C>(a.cd);
    dim3 b = step_block(a.g.nx), gr = step_grid(a.g, b);
    const bool rot = a.omega_rot != 0.0;
#define TH_LAUNCH(FI, RO)                                                                   \
    k_thermal_step<S, FI, RO><<<gr, b, 0, s>>>((const S*)fin, (S*)fout, (const S*)gin, (S*)gout, \
                                               (C*)F, a, c)
    if (first && rot) TH_LAUNCH(true, true);
    else if (first) TH_LAUNCH(true, false);
    else if (rot) TH_LAUNCH(false, true);
    else TH_LAUNCH(false, false);
#undef TH_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_thermal_step(int form, bool first, const void* fin, void* fout,
                                const void* gin, void* gout, void* F, const ThermalStepArgs& a,
                                cudaStream_t s) {
    switch (form) {
        case FORM_FP64: return th_go<double>(first, fin, fout, gin, gout, F, a, s);
        case FORM_FP32: return th_go<float>(first, fin, fout, gin, gout, F, a, s);
        case FORM_FP16: return th_go<__half>(first, fin, fout, gin, gout, F, a, s);
        case FORM_BF16: return th_go<__nv_bfloat16>(first, fin, fout, gin, gout, F, a, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace mglc
