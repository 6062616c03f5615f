// k_aux.cu -- macroscopic fields, equilibrium initialisation, layout
// conversion between the reference's AoS arrays and the device SoA planes,
// and deterministic FP64 reductions (residual, totals).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "kernels.cuh"

namespace mglc {

template <typename S>
__device__ __forceinline__ double to_d(S v);
template <>
__device__ __forceinline__ double to_d<double>(double v) { return v; }
template <>
__device__ __forceinline__ double to_d<float>(float v) { return (double)v; }
template <>
__device__ __forceinline__ double to_d<__half>(__half v) { return (double)__half2float(v); }
template <>
__device__ __forceinline__ double to_d<__nv_bfloat16>(__nv_bfloat16 v) {
    return (double)__bfloat162float(v);
}
template <typename S>
__device__ __forceinline__ S from_d(double v);
template <>
__device__ __forceinline__ double from_d<double>(double v) { return v; }
template <>
__device__ __forceinline__ float from_d<float>(double v) { return (float)v; }
template <>
__device__ __forceinline__ __half from_d<__half>(double v) { return __float2half_rn((float)v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_d<__nv_bfloat16>(double v) {
    return __float2bfloat16_rn((float)v);
}

// stored value -> absolute population (FP64)
template <typename S>
__device__ __forceinline__ double pop_abs(const S* p, long long idx, int q, double rho0,
                                          double inv_scale, bool shifted) {
    double v = to_d<S>(p[idx]);
    if (shifted) v = v * inv_scale + w19(q) * rho0;
    return v;
}

// ------------------------------------------------------------- macro() --
// Reference order: rho = sum over alpha from 0..18 sequentially, momentum in
// the order of the alpha loop (macro.f90:6-25 / bouyancy3d_mpi.F90:986-1010),
// with the thermal half-force shift.  Uses IEEE-rounded adds, multiplies and
// divisions so that for FP64 storage the fields equal the reference's.
// storage type of the temperature populations for a given f storage type
template <typename S> struct GType { using T = float; };
template <> struct GType<double> { using T = double; };

template <typename S, bool THERMAL>
__global__ void k_macro(const S* __restrict__ f, const typename GType<S>::T* __restrict__ gt,
                        const void* Fv,
                        Geom g, double rho0, double inv_scale, double* rho, double* u, double* v,
                        double* w, double* T) {
    const long long n = g.plane;
    const bool shifted = !std::is_same<S, double>::value;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        double fq[Q19];
#pragma unroll
        for (int q = 0; q < Q19; q++) fq[q] = pop_abs<S>(f, q * n + c, q, rho0, inv_scale, shifted);
        double r = fq[0];
#pragma unroll
        for (int q = 1; q < Q19; q++) r = __dadd_rn(r, fq[q]);
        double jx = 0.0, jy = 0.0, jz = 0.0;
        bool fx_ = false, fy_ = false, fz_ = false;
#pragma unroll
        for (int q = 1; q < Q19; q++) {
            if (ex19(q)) { jx = fx_ ? __dadd_rn(jx, ex19(q) * fq[q]) : ex19(q) * fq[q]; fx_ = true; }
            if (ey19(q)) { jy = fy_ ? __dadd_rn(jy, ey19(q) * fq[q]) : ey19(q) * fq[q]; fy_ = true; }
            if (ez19(q)) { jz = fz_ ? __dadd_rn(jz, ez19(q) * fq[q]) : ez19(q) * fq[q]; fz_ = true; }
        }
        if (THERMAL) {
            double Fx, Fy, Fz;
            if (std::is_same<S, double>::value) {
                const double* F = (const double*)Fv;
                Fx = F[c]; Fy = F[n + c]; Fz = F[2 * n + c];
            } else {
                const float* F = (const float*)Fv;
                Fx = F[c]; Fy = F[n + c]; Fz = F[2 * n + c];
            }
            jx = __dadd_rn(jx, __dmul_rn(0.5, Fx));
            jy = __dadd_rn(jy, __dmul_rn(0.5, Fy));
            jz = __dadd_rn(jz, __dmul_rn(0.5, Fz));
            double t = (double)gt[c];
#pragma unroll
            for (int q = 1; q < Q7; q++) t = __dadd_rn(t, (double)gt[q * n + c]);
            T[c] = t;
        }
        rho[c] = r;
        u[c] = __ddiv_rn(jx, r);
        v[c] = __ddiv_rn(jy, r);
        w[c] = __ddiv_rn(jz, r);
    }
}

static int grid_for(long long n, int block) {
    long long b = (n + block - 1) / block;
    if (b > 152 * 32) b = 152 * 32;
    if (b < 1) b = 1;
    return (int)b;
}

template <typename S>
static cudaError_t macro_go(bool thermal, const Geom& g, const void* f, const void* gt,
                            const void* F, double rho0, double inv, double* rho, double* u,
                            double* v, double* w, double* T, cudaStream_t s) {
    int gr = grid_for(g.plane, 256);
    if (thermal)
        k_macro<S, true><<<gr, 256, 0, s>>>((const S*)f, (const typename GType<S>::T*)gt, F, g, rho0, inv, rho, u, v, w, T);
    else
        k_macro<S, false><<<gr, 256, 0, s>>>((const S*)f, nullptr, nullptr, g, rho0, inv, rho, u, v, w, T);
    return cudaGetLastError();
}

cudaError_t launch_macro(int form, bool thermal, const Geom& g, const void* f, const void* gt,
                         const void* F, double rho0, float inv_scale, double* rho, double* u,
                         double* v, double* w, double* T, cudaStream_t s) {
    switch (form) {
        case FORM_FP64: return macro_go<double>(thermal, g, f, gt, F, rho0, 1.0, rho, u, v, w, T, s);
        case FORM_FP32: return macro_go<float>(thermal, g, f, gt, F, rho0, 1.0, rho, u, v, w, T, s);
        case FORM_FP16: return macro_go<__half>(thermal, g, f, gt, F, rho0, inv_scale, rho, u, v, w, T, s);
        case FORM_BF16: return macro_go<__nv_bfloat16>(thermal, g, f, gt, F, rho0, 1.0, rho, u, v, w, T, s);
    }
    return cudaErrorInvalidValue;
}

// ------------------------------------------------------ equilibrium init --
// f = rho*omega*(1 + 3 un + 4.5 un^2 - 1.5 us2)   (initial.f90:67-72)
// g = omegaT*T*(1 + 21/(6+paraA) un)               (bouyancy3d_mpi.F90:586-589)
// IEEE-rounded operations in the reference's order (bit-equal for FP64).
template <typename S, bool THERMAL>
__global__ void k_equilibrium(Geom g, const double* rho, const double* u, const double* v,
                              const double* w, const double* T, double para_a, double rho0,
                              double scale, S* f, typename GType<S>::T* gt) {
    const long long n = g.plane;
    const bool shifted = !std::is_same<S, double>::value;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const double uu = u[c], vv = v[c], ww = w[c], r = rho[c];
        const double us2 = __dadd_rn(__dadd_rn(__dmul_rn(uu, uu), __dmul_rn(vv, vv)), __dmul_rn(ww, ww));
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            double un = __dadd_rn(__dadd_rn(__dmul_rn(uu, (double)ex19(q)), __dmul_rn(vv, (double)ey19(q))),
                                  __dmul_rn(ww, (double)ez19(q)));
            double poly = __dsub_rn(__dadd_rn(__dadd_rn(1.0, __dmul_rn(3.0, un)),
                                              __dmul_rn(__dmul_rn(4.5, un), un)),
                                    __dmul_rn(1.5, us2));
            double fe = __dmul_rn(__dmul_rn(r, w19(q)), poly);
            if (shifted) fe = (fe - w19(q) * rho0) * scale;
            f[q * n + c] = from_d<S>(fe);
        }
        if (THERMAL) {
            const double t = T[c];
            const double wt0 = (1.0 - para_a) / 7.0, wt = (para_a + 6.0) / 42.0;
            const double coef = 21.0 / (6.0 + para_a);
#pragma unroll
            for (int q = 0; q < Q7; q++) {
                double un = __dadd_rn(__dadd_rn(__dmul_rn(uu, (double)ex19(q)), __dmul_rn(vv, (double)ey19(q))),
                                      __dmul_rn(ww, (double)ez19(q)));
                double ge = __dmul_rn(__dmul_rn(q == 0 ? wt0 : wt, t), __dadd_rn(1.0, __dmul_rn(coef, un)));
                gt[q * n + c] = (typename GType<S>::T)ge;
            }
        }
    }
}

template <typename S>
static cudaError_t eq_go(bool thermal, const Geom& g, const double* rho, const double* u,
                         const double* v, const double* w, const double* T, double para_a,
                         double rho0, double scale, void* f, void* gt, cudaStream_t s) {
    int gr = grid_for(g.plane, 256);
    if (thermal)
        k_equilibrium<S, true><<<gr, 256, 0, s>>>(g, rho, u, v, w, T, para_a, rho0, scale, (S*)f,
                                                  (typename GType<S>::T*)gt);
    else
        k_equilibrium<S, false><<<gr, 256, 0, s>>>(g, rho, u, v, w, T, para_a, rho0, scale, (S*)f, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_equilibrium(int form, bool thermal, const Geom& g, const double* rho,
                               const double* u, const double* v, const double* w,
                               const double* T, double para_a, double rho0, float scale, void* f,
                               void* gt, cudaStream_t s) {
    switch (form) {
        case FORM_FP64: return eq_go<double>(thermal, g, rho, u, v, w, T, para_a, rho0, 1.0, f, gt, s);
        case FORM_FP32: return eq_go<float>(thermal, g, rho, u, v, w, T, para_a, rho0, 1.0, f, gt, s);
        case FORM_FP16: return eq_go<__half>(thermal, g, rho, u, v, w, T, para_a, rho0, scale, f, gt, s);
        case FORM_BF16: return eq_go<__nv_bfloat16>(thermal, g, rho, u, v, w, T, para_a, rho0, 1.0, f, gt, s);
    }
    return cudaErrorInvalidValue;
}

// ------------------------------------------------------ layout conversion --
template <typename S>
__global__ void k_aos_to_soa(int Q, long long plane, long long cell0, long long ncells,
                             const double* __restrict__ aos, S* __restrict__ soa, double rho0,
                             double scale, bool shifted) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells;
         c += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < Q; q++) {
            double v = aos[(long long)Q * c + q];
            if (shifted) v = (v - w19(q) * rho0) * scale;
            soa[q * plane + cell0 + c] = from_d<S>(v);
        }
    }
}
template <typename S>
__global__ void k_soa_to_aos(int Q, long long plane, long long cell0, long long ncells,
                             const S* __restrict__ soa, double* __restrict__ aos, double rho0,
                             double inv_scale, bool shifted) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells;
         c += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < Q; q++) {
            double v = to_d<S>(soa[q * plane + cell0 + c]);
            if (shifted) v = v * inv_scale + w19(q) * rho0;
            aos[(long long)Q * c + q] = v;
        }
    }
}

cudaError_t launch_aos_to_soa(int form, int Q, const Geom& g, long long cell0, long long ncells,
                              const double* aos, void* soa, double rho0, float scale,
                              bool shifted, cudaStream_t s) {
    int gr = grid_for(ncells, 256);
    switch (form) {
        case FORM_FP64: k_aos_to_soa<double><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, aos, (double*)soa, rho0, 1.0, false); break;
        case FORM_FP32: k_aos_to_soa<float><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, aos, (float*)soa, rho0, 1.0, shifted); break;
        case FORM_FP16: k_aos_to_soa<__half><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, aos, (__half*)soa, rho0, scale, shifted); break;
        case FORM_BF16: k_aos_to_soa<__nv_bfloat16><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, aos, (__nv_bfloat16*)soa, rho0, 1.0, shifted); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(int form, int Q, const Geom& g, long long cell0, long long ncells,
                              const void* soa, double* aos, double rho0, float inv_scale,
                              bool shifted, cudaStream_t s) {
    int gr = grid_for(ncells, 256);
    switch (form) {
        case FORM_FP64: k_soa_to_aos<double><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, (const double*)soa, aos, rho0, 1.0, false); break;
        case FORM_FP32: k_soa_to_aos<float><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, (const float*)soa, aos, rho0, 1.0, shifted); break;
        case FORM_FP16: k_soa_to_aos<__half><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, (const __half*)soa, aos, rho0, inv_scale, shifted); break;
        case FORM_BF16: k_soa_to_aos<__nv_bfloat16><<<gr, 256, 0, s>>>(Q, g.plane, cell0, ncells, (const __nv_bfloat16*)soa, aos, rho0, 1.0, shifted); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------ reductions --
constexpr int RED_BLOCK = 256;
constexpr int RED_MAX_BLOCKS = 152 * 8;

int reduce_blocks(long long n) {
    long long b = (n + RED_BLOCK - 1) / RED_BLOCK;
    if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
    if (b < 1) b = 1;
    return (int)b;
}

// block-wide sum of NV values, warp shuffles then shared memory; fixed order
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* out) {
    __shared__ double sh[RED_BLOCK / 32][NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sh[wid][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; k++) {
            double t = 0.0;
            for (int wv = 0; wv < RED_BLOCK / 32; wv++) t += sh[wv][k];
            out[k] = t;
        }
    }
}

__global__ void __launch_bounds__(RED_BLOCK)
    k_residual(long long n, const double* u, const double* v, const double* w, const double* T,
               double* up, double* vp, double* wp, double* Tp, bool with_w, double* partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long c = blockIdx.x * (long long)RED_BLOCK + threadIdx.x; c < n;
         c += (long long)gridDim.x * RED_BLOCK) {
        const double uu = u[c], vv = v[c], ww = w[c];
        const double a = uu - up[c], b = vv - vp[c], cw = ww - wp[c];
        acc[0] += a * a + b * b + (with_w ? cw * cw : 0.0);
        acc[1] += uu * uu + vv * vv + ww * ww;
        up[c] = uu;
        vp[c] = vv;
        wp[c] = ww;
        if (T) {
            const double t = T[c];
            acc[2] += fabs(t - Tp[c]);
            acc[3] += fabs(t);
            Tp[c] = t;
        }
    }
    block_sum<4>(acc, partials + 4 * blockIdx.x);
}

template <int NV>
__global__ void k_finish(int nblocks, const double* partials, double* out) {
    // one warp: each lane sums a strided subset in order, then a fixed tree
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += 32)
#pragma unroll
        for (int k = 0; k < NV; k++) acc[k] += partials[NV * b + k];
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = acc[k];
}

cudaError_t launch_residual(long long n, const double* u, const double* v, const double* w,
                            const double* T, double* up, double* vp, double* wp, double* Tp,
                            bool with_w, double* partials, double* out4, cudaStream_t s) {
    int nb = reduce_blocks(n);
    k_residual<<<nb, RED_BLOCK, 0, s>>>(n, u, v, w, T, up, vp, wp, Tp, with_w, partials);
    k_finish<4><<<1, 32, 0, s>>>(nb, partials, out4);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(RED_BLOCK)
    k_totals(long long n, const double* rho, const double* u, const double* v, const double* w,
             const double* T, double* partials) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (long long c = blockIdx.x * (long long)RED_BLOCK + threadIdx.x; c < n;
         c += (long long)gridDim.x * RED_BLOCK) {
        const double r = rho[c], uu = u[c], vv = v[c], ww = w[c];
        acc[0] += r;
        acc[1] += 0.5 * r * (uu * uu + vv * vv + ww * ww);
        if (T) acc[2] += T[c];
    }
    block_sum<3>(acc, partials + 3 * blockIdx.x);
}

cudaError_t launch_totals(long long n, const double* rho, const double* u, const double* v,
                          const double* w, const double* T, double* partials, double* out3,
                          cudaStream_t s) {
    int nb = reduce_blocks(n);
    k_totals<<<nb, RED_BLOCK, 0, s>>>(n, rho, u, v, w, T, partials);
    k_finish<3><<<1, 32, 0, s>>>(nb, partials, out3);
    return cudaGetLastError();
}

// calNuRe (mpi_blocked/RaNu.F90:13-47) sums plus the wall-gradient sums of the
// hot/cold wall Nusselt numbers.  The wall sits half a cell outside the first
// node, so dT/dn|wall = (9 T_1 - T_2 - 8 T_wall)/3 (second order).
__global__ void __launch_bounds__(RED_BLOCK)
    k_thermal_stats(Geom g, const double* u, const double* v, const double* w, const double* T,
                    int wall_axis, double* partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const long long n = g.plane;
    const long long sxy = (long long)g.nx * g.ny;
    for (long long c = blockIdx.x * (long long)RED_BLOCK + threadIdx.x; c < n;
         c += (long long)gridDim.x * RED_BLOCK) {
        const double uu = u[c], vv = v[c], ww = w[c], t = T[c];
        acc[0] += ww * t;
        acc[1] += uu * uu + vv * vv + ww * ww;
        if (wall_axis == 1) {
            const int j = (int)((c / g.nx) % g.ny);
            if (j == 0) acc[2] += 9.0 * t - T[c + g.nx];
            if (j == g.ny - 1) acc[3] += 9.0 * t - T[c - g.nx];
        } else if (wall_axis == 2) {
            const long long k = c / sxy;
            if (k == 0) acc[2] += 9.0 * t - T[c + sxy];
            if (k == g.nz - 1) acc[3] += 9.0 * t - T[c - sxy];
        }
    }
    block_sum<4>(acc, partials + 4 * blockIdx.x);
}

cudaError_t launch_thermal_stats(const Geom& g, const double* u, const double* v, const double* w,
                                 const double* T, int wall_axis, double* partials, double* out4,
                                 cudaStream_t s) {
    int nb = reduce_blocks(g.plane);
    k_thermal_stats<<<nb, RED_BLOCK, 0, s>>>(g, u, v, w, T, wall_axis, partials);
    k_finish<4><<<1, 32, 0, s>>>(nb, partials, out4);
    return cudaGetLastError();
}

}  // namespace mglc
