// k_serve.cu -- kernels of the solve server.
//
// k_serve_step is a persistent kernel: every warp of a grid sized to the SM
// count pulls tiles (rows_per_tile x-rows of one solve) from a queue shared by
// the resident solves of one kind, through one atomic counter per step, and
// runs the fused step of that solve on the tile's cells.  Lid and heated
// solves have separate kernels (each with its own register budget) that run
// concurrently.  Small and large grids, lid and
// heated cavities are mixed in one launch, so small solves no longer leave
// the GPU idle.  The per-cell arithmetic is exactly that of the one-solve
// kernels (step_cell.cuh), so a solve's result does not depend on which
// other solves share the launch.
#include "serve.cuh"

namespace mglc {

// solve that owns queue tile t (binary search over tile0)
__device__ __forceinline__ int find_solve(const ServeTable* tab, int t) {
    int lo = 0, hi = tab->n_active - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab->s[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Each warp pulls its own tiles (no block-wide barriers): lane 0 takes the
// next index from the step's counter and broadcasts it.
__device__ __forceinline__ int next_tile_warp(unsigned* counter) {
    int t = 0;
    if ((threadIdx.x & 31) == 0) t = (int)atomicAdd(counter, 1u);
    return __shfl_sync(0xffffffffu, t, 0);
}

// lid tiles: [0, lid_tiles); heated tiles: [lid_tiles, total_tiles)
// AA: solves stream in place on one buffer (step_cell.cuh: even steps read and
// write each cell's own slots, odd steps read upstream and write downstream;
// iterations have an even step count, so a solve is in the post-stream layout
// whenever the residual or the field readers see it).
// resident CTAs of 256 threads per SM the register allocation is held to
#ifndef MGLC_SERVE_LID_MINB
#define MGLC_SERVE_LID_MINB 3
#endif
#ifndef MGLC_SERVE_HEAT_MINB
#define MGLC_SERVE_HEAT_MINB 2
#endif

template <typename S, bool THERMAL, bool SR, bool AA>
__global__ void __launch_bounds__(256, THERMAL ? MGLC_SERVE_HEAT_MINB : MGLC_SERVE_LID_MINB)
    k_serve_step(const ServeTable* __restrict__ tab, int kstep, unsigned* counter) {
    const int parity = kstep & 1;
    const int base = THERMAL ? tab->lid_tiles : 0;
    const int ntiles = (THERMAL ? tab->total_tiles : tab->lid_tiles) - base;
    const int R = tab->rows_per_tile;
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int tl = next_tile_warp(counter);
        if (tl >= ntiles) break;
        const int t = base + tl;
        const ServeSolve& sv = tab->s[find_solve(tab, t)];
        const int nx = sv.nx, ny = sv.ny, nz = sv.nz;
        const int r0 = (t - sv.tile0) * R;
        const int r1 = min(r0 + R, ny * nz);
        const int ncell = (r1 - r0) * nx;
        const S* fin = (const S*)sv.f[parity];
        S* fout = (S*)sv.f[parity ^ 1];
        const unsigned seed = sv.step0 + (unsigned)kstep;
        // cell coordinates of idx = lane, lane + 32, ... kept incrementally
        // (one division per tile instead of three per cell)
        int i = lane % nx, j, k;
        {
            const int r = r0 + lane / nx;
            j = r % ny;
            k = r / ny;
        }
        for (int idx = lane; idx < ncell; idx += 32) {
            if (idx != lane) {
                i += 32;
                while (i >= nx) {  // at most 32 / nx + 1 passes
                    i -= nx;
                    if (++j == ny) {
                        j = 0;
                        ++k;
                    }
                }
            }
            if (AA) {
                S* f = (S*)sv.f[0];
                if (!THERMAL) {
                    S raw[Q19];
                    if (parity) {
                        lid_load_aa<S, unsigned, true>(i, j, k, f, nx, ny, nz, sv.plane, raw);
                        lid_cell_from<S, false, unsigned, SR, false>(
                            i, j, k, raw, f, sv.K, sv.plane, nullptr, nullptr, nullptr, nullptr, seed);
                    } else {
                        lid_load_aa<S, unsigned, false>(i, j, k, f, nx, ny, nz, sv.plane, raw);
                        lid_cell_from<S, false, unsigned, SR, true>(
                            i, j, k, raw, f, sv.K, sv.plane, nullptr, nullptr, nullptr, nullptr, seed);
                    }
                } else {
                    float fv[Q19], gv[Q7], fp[3];
                    if (parity) {
                        thermal_load_aa<S, unsigned, true>(i, j, k, f, sv.g[0], sv.F, 0u, sv.K,
                                                           sv.plane, fv, gv, fp);
                        thermal_cell_from<S, false, false, unsigned, SR, false>(
                            i, j, k, fv, gv, fp, f, sv.g[0], sv.F, sv.K, sv.plane, nullptr, nullptr,
                            nullptr, nullptr, nullptr, 0u, seed);
                    } else {
                        thermal_load_aa<S, unsigned, false>(i, j, k, f, sv.g[0], sv.F, 0u, sv.K,
                                                            sv.plane, fv, gv, fp);
                        thermal_cell_from<S, false, false, unsigned, SR, true>(
                            i, j, k, fv, gv, fp, f, sv.g[0], sv.F, sv.K, sv.plane, nullptr, nullptr,
                            nullptr, nullptr, nullptr, 0u, seed);
                    }
                }
            } else if (!THERMAL) {
                lid_cell<S, false, unsigned, SR>(i, j, k, fin, fout, sv.K, sv.plane, nullptr,
                                                 nullptr, nullptr, nullptr, seed);
            } else {
                thermal_cell<S, false, false, unsigned, SR>(
                    i, j, k, fin, fout, sv.g[parity], sv.g[parity ^ 1], sv.F, sv.K, sv.plane,
                    nullptr, nullptr, nullptr, nullptr, nullptr, 0u, seed);
            }
        }
    }
}

// max |u - uprev| / uref per solve; uprev <- u (all solves, warp tiles)
template <typename S>
__global__ void k_serve_resid(const ServeTable* __restrict__ tab, unsigned* counter,
                              unsigned* resid) {
    const int total = tab->total_tiles;
    const int R = tab->rows_per_tile;
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int t = next_tile_warp(counter);
        if (t >= total) break;
        const int si = find_solve(tab, t);
        const ServeSolve& sv = tab->s[si];
        const int nx = sv.nx, ny = sv.ny, nz = sv.nz;
        const unsigned P = sv.plane;
        const int r0 = (t - sv.tile0) * R;
        const int r1 = min(r0 + R, ny * nz);
        const int ncell = (r1 - r0) * nx;
        const S* f = (const S*)sv.f[0];  // residual runs after an even number of steps
        float m = 0.0f;
        for (int idx = lane; idx < ncell; idx += 32) {
            const unsigned cell = (unsigned)(r0 * nx + idx);
            float fq[Q19];
#pragma unroll
            for (int q = 0; q < Q19; q++) fq[q] = St<S>::ld(f + (q * P + cell), sv.K.inv_scale);
            float rho_m, jx, jy, jz;
            moments0(fq, rho_m, jx, jy, jz);
            const float rho = 1.0f + rho_m;
            if (sv.kind == 2) jz += 0.5f * sv.F[cell];
            const float ux = jx / rho, uy = jy / rho, uz = jz / rho;
            float d = fmaxf(fabsf(ux - sv.uprev[cell]),
                            fmaxf(fabsf(uy - sv.uprev[P + cell]), fabsf(uz - sv.uprev[2 * P + cell])));
            d = d / sv.uref;
            if (!(d == d)) d = __int_as_float(0x7f800000);  // NaN -> inf: never converges
            m = fmaxf(m, d);
            sv.uprev[cell] = ux;
            sv.uprev[P + cell] = uy;
            sv.uprev[2 * P + cell] = uz;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
        if (lane == 0) atomicMax(resid + si, __float_as_uint(m));
    }
}

template <typename S>
__global__ void k_serve_init(ServeSolve sv, float t_hot, float t_cold) {
    const unsigned P = sv.plane;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < P; c += gridDim.x * blockDim.x) {
        S* f = (S*)sv.f[0];
#pragma unroll
        for (int q = 0; q < Q19; q++) St<S>::st(f + (q * P + c), 0.0f, 1.0f);  // f = w (rho = 1, u = 0)
        sv.uprev[c] = 0.0f;
        sv.uprev[P + c] = 0.0f;
        sv.uprev[2 * P + c] = 0.0f;
        if (sv.kind == 2) {
            const int j = (int)((c / sv.nx) % sv.ny);
            const float T = j == 0 ? t_hot : (j == sv.ny - 1 ? t_cold : 0.0f);
            const float a = sv.K.para_a;
            const float w0 = (1.0f - a) / 7.0f, wi = (a + 6.0f) / 42.0f;
            float* g = sv.g[0];
            g[c] = w0 * T;
#pragma unroll
            for (int q = 1; q < Q7; q++) g[q * P + c] = wi * T;
            sv.F[c] = 0.0f;
        }
    }
}

template <typename S>
__global__ void k_serve_fields(ServeSolve sv, float* out) {
    const unsigned P = sv.plane;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < P; c += gridDim.x * blockDim.x) {
        const S* f = (const S*)sv.f[0];
        float fq[Q19];
#pragma unroll
        for (int q = 0; q < Q19; q++) fq[q] = St<S>::ld(f + (q * P + c), sv.K.inv_scale);
        float rho_m, jx, jy, jz;
        moments0(fq, rho_m, jx, jy, jz);
        const float rho = 1.0f + rho_m;
        if (sv.kind == 2) jz += 0.5f * sv.F[c];
        out[c] = rho;
        out[P + c] = jx / rho;
        out[2 * P + c] = jy / rho;
        out[3 * P + c] = jz / rho;
        if (sv.kind == 2) {
            const float* g = sv.g[0];
            out[4 * P + c] = ((g[c] + g[P + c]) + (g[2 * P + c] + g[3 * P + c])) +
                             ((g[4 * P + c] + g[5 * P + c]) + g[6 * P + c]);
        }
    }
}

template <typename S, bool SR>
static void serve_go(int thermal, int aa, const ServeTable* tab, int k, unsigned* counter,
                     int grid, int block, cudaStream_t st) {
    if (thermal && aa) k_serve_step<S, true, SR, true><<<grid, block, 0, st>>>(tab, k, counter);
    else if (thermal) k_serve_step<S, true, SR, false><<<grid, block, 0, st>>>(tab, k, counter);
    else if (aa) k_serve_step<S, false, SR, true><<<grid, block, 0, st>>>(tab, k, counter);
    else k_serve_step<S, false, SR, false><<<grid, block, 0, st>>>(tab, k, counter);
}

cudaError_t launch_serve_step(int form, int sr, int aa, int thermal, const ServeTable* tab, int k,
                              unsigned* counter, int grid, int block, cudaStream_t st) {
    if (form == FORM_FP16 && sr) serve_go<__half, true>(thermal, aa, tab, k, counter, grid, block, st);
    else if (form == FORM_FP16) serve_go<__half, false>(thermal, aa, tab, k, counter, grid, block, st);
    else if (form == FORM_FP32) serve_go<float, false>(thermal, aa, tab, k, counter, grid, block, st);
    else if (form == FORM_BF16 && sr)
        serve_go<__nv_bfloat16, true>(thermal, aa, tab, k, counter, grid, block, st);
    else if (form == FORM_BF16)
        serve_go<__nv_bfloat16, false>(thermal, aa, tab, k, counter, grid, block, st);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// step0 += steps for every active solve (after the iteration's steps)
__global__ void k_serve_advance(ServeTable* tab, int steps) {
    for (int s = threadIdx.x; s < tab->n_active; s += blockDim.x) tab->s[s].step0 += (unsigned)steps;
}

cudaError_t launch_serve_resid(int form, ServeTable* tab, unsigned* counter, unsigned* resid,
                               int steps, int grid, int block, cudaStream_t st) {
    if (form == FORM_FP16) k_serve_resid<__half><<<grid, block, 0, st>>>(tab, counter, resid);
    else if (form == FORM_FP32) k_serve_resid<float><<<grid, block, 0, st>>>(tab, counter, resid);
    else if (form == FORM_BF16) k_serve_resid<__nv_bfloat16><<<grid, block, 0, st>>>(tab, counter, resid);
    else return cudaErrorInvalidValue;
    k_serve_advance<<<1, 256, 0, st>>>(tab, steps);
    return cudaGetLastError();
}

cudaError_t launch_serve_init(int form, const ServeSolve& s, double t_hot, double t_cold,
                              cudaStream_t st) {
    const int grid = (int)std::min<unsigned>((s.plane + 255) / 256, 152 * 8);
    if (form == FORM_FP16) k_serve_init<__half><<<grid, 256, 0, st>>>(s, (float)t_hot, (float)t_cold);
    else if (form == FORM_FP32) k_serve_init<float><<<grid, 256, 0, st>>>(s, (float)t_hot, (float)t_cold);
    else if (form == FORM_BF16) k_serve_init<__nv_bfloat16><<<grid, 256, 0, st>>>(s, (float)t_hot, (float)t_cold);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_serve_fields(int form, const ServeSolve& s, float* out, cudaStream_t st) {
    const int grid = (int)std::min<unsigned>((s.plane + 255) / 256, 152 * 8);
    if (form == FORM_FP16) k_serve_fields<__half><<<grid, 256, 0, st>>>(s, out);
    else if (form == FORM_FP32) k_serve_fields<float><<<grid, 256, 0, st>>>(s, out);
    else if (form == FORM_BF16) k_serve_fields<__nv_bfloat16><<<grid, 256, 0, st>>>(s, out);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace mglc

MGLC_OOB_READER(mglc_oob_hits_k_serve)
