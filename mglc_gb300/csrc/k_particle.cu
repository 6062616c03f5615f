// k_particle.cu -- moving spheres in a D3Q19 channel (periodic x, no-slip y/z
// walls): the 3-D generalisation of the reference's Micro_particles step
// (MPI/Micro_particles/fortran/case4/mpi_particle, main.F90:35-73).
//
// Per time step:
//   k_pbulk     fluid cells: macro, forced MRT collision, push to the
//               neighbours (x wraps, y/z walls bounce back in place);
//               solid cells do nothing.  Block partials of sum rho and of
//               the post-collision mass feed the average density.
//   k_pfinish   fixed-order sums -> rho_avg (particle_bounceback.F90:15-35)
//   k_plinks    PART_NSLAB CTAs per particle: every fluid node x with a neighbour
//               x+e inside the particle is a boundary link.  The
//               post-collision values the quadratic interpolated bounce-back
//               needs (particle_bounceback.F90:65-75) are read from the
//               streamed array: fp(a,y) sits in f(a, y+e_a) after the push
//               (including solid destination cells, which only fluid pushes
//               write).  Writes f(abar,x) and accumulates the Wen 2014
//               momentum exchange (particle_force.F90:59-66) in FP64.
//   k_pforce    one warp per particle: springs, gravity, body force
//               (particle_force.F90:96-190)
//   k_pmove     explicit update (particle_update.F90:26-50)
//   k_pmark     new owner mask from the new centres (particle_update.F90:80-93)
//   k_pprep     density bookkeeping of nodes that change phase
//   k_prefill   refill of nodes that left a particle (:134-193), two phases
//               per particle (all reads, then all writes).
// Any kernel that detects a failure (no owner, q out of range, overlap, wall
// penetration) writes a status code; every kernel returns at once while the
// status is set, so the state freezes at the failing step and the host
// reports MGLC_ERR_PARTICLE.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "particles.cuh"

namespace mglc {

constexpr int PB = 256;             // threads of the per-particle kernels
constexpr int NSLAB = PART_NSLAB;   // CTAs per particle in k_plinks
constexpr int REFILL_MAX = 256;     // refilled nodes one particle may produce per step

template <typename S>
struct PSt;
template <>
struct PSt<double> {
    static constexpr bool SHIFT = false;
    __device__ static double ld(const double* p) { return *p; }
    __device__ static void st(double* p, double v) { *p = v; }
};
template <>
struct PSt<float> {
    static constexpr bool SHIFT = true;
    __device__ static double ld(const float* p) { return (double)*p; }
    __device__ static void st(float* p, double v) { *p = (float)v; }
};

// absolute population value (FP64) of a stored slot
template <typename S>
__device__ __forceinline__ double pabs(const S* f, long long idx, int q, double rho0) {
    double v = PSt<S>::ld(f + idx);
    return PSt<S>::SHIFT ? v + w19(q) * rho0 : v;
}
template <typename S>
__device__ __forceinline__ void pset(S* f, long long idx, int q, double v, double rho0) {
    PSt<S>::st(f + idx, PSt<S>::SHIFT ? v - w19(q) * rho0 : v);
}

// Signed x separation with the nearest periodic image.  Centres stay in
// [0.5, nx + 0.5) and nodes in [1, nx], so one shift by L brings d into
// [-L/2, L/2]; a larger |d| (a centre that jumped, which k_pmove reports)
// takes the closed form d - L rint(d/L).  A non-finite d is returned as is:
// no loop depends on it.
__device__ __forceinline__ double dxp(double a, double b, const PartParams& p) {
    double d = a - b;
    if (p.periodic_x && isfinite(d)) {
        const double L = (double)p.nx, h = 0.5 * L;
        if (d > h) d -= L;
        else if (d < -h) d += L;
        if (d > h || d < -h) d -= L * rint(d / L);
    }
    return d;
}
// ((x-xc)^2 + (y-yc)^2 + (z-zc)^2) <= R^2 with IEEE-rounded operations
__device__ __forceinline__ bool inside(double x, double y, double z, const double* X, double R,
                                       const PartParams& p) {
    const double a = dxp(x, X[0], p), b = y - X[1], c = z - X[2];
    double d = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
    return d <= __dmul_rn(R, R);
}
__device__ __forceinline__ int wrapx(int i, int nx) { return i < 0 ? i + nx : (i >= nx ? i - nx : i); }

template <int NV>
__device__ __forceinline__ void block_sum_to(double (&v)[NV], double* out, int stride) {
    __shared__ double sh[32][NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sh[wid][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) {
            double t = 0.0;
            for (int q = 0; q < nw; q++) t += sh[q][k];
            out[k * stride] = t;
        }
    __syncthreads();
}

// ------------------------------------------------------------- bulk step --
// compute type: FP64 for FP64 storage; FP32 (on deviations f - w rho0) for
// FP32 storage
template <typename S> struct PC { using C = double; };
template <> struct PC<float> { using C = float; };

// per-step constants of the bulk kernel in its arithmetic type (converted
// once on the host: double -> float conversions are slow on the device)
template <typename C> struct PBulkK {
    C rho0, ax, ay, az;
};

// One thread per node of an x-row segment.  Fluid nodes collide and push
// their populations (walls at y, z and, unless periodic, x bounce them back in
// place); solid nodes do nothing.  Each warp writes its partial sums of the
// fluid density before collision and of the post-collision mass to its own
// slot, so no block barrier is needed and the totals are added in a fixed
// order by k_pfinish.
// resident 128-thread blocks per SM the FP32 bulk kernel holds its registers to
#ifndef MGLC_PBULK_MINB
#define MGLC_PBULK_MINB 8
#endif
template <typename S, bool FIRST, typename IDX>
__global__ void __launch_bounds__(128, (sizeof(S) == 4 ? MGLC_PBULK_MINB : 4))
    k_pbulk(const S* __restrict__ fin, S* __restrict__ fout, const int* __restrict__ owner,
            PartParams p, MrtCoef<typename PC<S>::C> cd, PBulkK<typename PC<S>::C> bk,
            double* partials, const int* status) {
    using C = typename PC<S>::C;
    constexpr bool DEV = PSt<S>::SHIFT;
    if (status[0]) return;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const IDX P = (IDX)nx * ny * nz;
    C cacc[2] = {C(0), C(0)};  // per-cell sums in the arithmetic type, widened per warp
    const bool active = i < nx;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * k);
    // the populations are loaded before the mask answers (solid cells read
    // in-bounds values they do not use), so both loads are in flight together
    C f[Q19];
    if (active) {
#pragma unroll
        for (int q = 0; q < Q19; q++) f[q] = (C)__ldg(fin + (q * P + cell));
    }
    const bool fluid = active && __ldg(owner + cell) < 0;
    if (fluid) {
        const C rho0 = bk.rho0, ax = bk.ax, ay = bk.ay, az = bk.az;
        C rho_m, rho, ux, uy, uz;
        if (FIRST) {  // the reference's initial fields: rho0, u = 0
            rho = rho0;
            rho_m = DEV ? C(0) : rho0;
            ux = uy = uz = C(0);
        } else {
            C jx, jy, jz;
            moments0(f, rho_m, jx, jy, jz);
            rho = DEV ? rho0 + rho_m : rho_m;
            // u = (sum f e + F/2)/rho with F = rho*a (thermal macro form); FP32
            // multiplies by the correctly rounded reciprocal, FP64 divides
            if constexpr (sizeof(C) == 4) {
                const C inv = __frcp_rn(rho);
                ux = (jx + C(0.5) * (rho * ax)) * inv;
                uy = (jy + C(0.5) * (rho * ay)) * inv;
                uz = (jz + C(0.5) * (rho * az)) * inv;
            } else {
                ux = (jx + C(0.5) * (rho * ax)) / rho;
                uy = (jy + C(0.5) * (rho * ay)) / rho;
                uz = (jz + C(0.5) * (rho * az)) / rho;
            }
        }
        // deviation storage sums deviations (rho0 added back per warp)
        cacc[0] = DEV ? rho_m : rho;
        mrt_collide<C, true, false>(f, rho_m, rho, ux, uy, uz, rho * ax, rho * ay, rho * az, cd);
        C m = C(0);
#pragma unroll
        for (int q = 0; q < Q19; q++) m += f[q];
        cacc[1] = m;
        const IDX sy = nx, sz = (IDX)nx * ny;
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1) {
            // interior node: every population streams, no wrap
#pragma unroll
            for (int q = 0; q < Q19; q++)
                fout[q * P + cell + (IDX)ex19(q) + (IDX)ey19(q) * sy + (IDX)ez19(q) * sz] = (S)f[q];
        } else {
#pragma unroll
            for (int q = 0; q < Q19; q++) {
                const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
                const int jj = j + dy, kk = k + dz, ir = i + dx;
                const bool xwall = !p.periodic_x && (ir < 0 || ir >= nx);
                if (xwall || jj < 0 || jj >= ny || kk < 0 || kk >= nz) {
                    fout[opp19(q) * P + cell] = (S)f[q];  // no-slip wall
                } else {
                    const int ii = wrapx(ir, nx);
                    fout[q * P + ((IDX)ii + sy * jj + sz * kk)] = (S)f[q];
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cacc[q] += __shfl_down_sync(0xffffffffu, cacc[q], o);
    // fluid cells of this warp (deviation storage adds rho0 for each of them)
    const unsigned fl = __ballot_sync(0xffffffffu, fluid);
    if ((threadIdx.x & 31) == 0) {  // FP64 only for the warp leaders
        const int nw = blockDim.x >> 5;
        const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        const int slot = b * nw + (threadIdx.x >> 5);
        const int nslot = gridDim.x * gridDim.y * gridDim.z * nw;
        const double nf = DEV ? (double)__popc(fl) * p.rho0 : 0.0;
        partials[slot] = (double)cacc[0] + nf;
        partials[nslot + slot] = (double)cacc[1] + nf;
    }
}

constexpr int FINISH_BLOCKS = 32;

// stage 1: FINISH_BLOCKS contiguous ranges of the bulk partials
__global__ void k_pfinish(PartDev d, int nblocks) {
    if (d.status[0]) return;
    const int per = (nblocks + FINISH_BLOCKS - 1) / FINISH_BLOCKS;
    const int b0 = blockIdx.x * per, b1 = min(nblocks, b0 + per);
    double acc[2] = {0.0, 0.0};
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        acc[0] += d.partials[b];
        acc[1] += d.partials[nblocks + b];
    }
    __shared__ double out[2];
    block_sum_to<2>(acc, out, 1);
    if (threadIdx.x == 0) {
        d.partials[2 * nblocks + blockIdx.x] = out[0];
        d.partials[2 * nblocks + FINISH_BLOCKS + blockIdx.x] = out[1];
    }
}
// stage 2 (one warp): rho_avg at bounce-back and the post-collision mass
__global__ void k_pfinish2(PartDev d, int nblocks) {
    if (d.status[0]) return;
    const int lane = threadIdx.x;
    double a0 = d.partials[2 * nblocks + lane], a1 = d.partials[2 * nblocks + FINISH_BLOCKS + lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    if (lane == 0) {
        d.rho_avg[0] = a0 / (double)d.n_fluid[0];
        d.rho_avg[2] = a1;
    }
}
// average density over the new fluid set, used by the refill (one warp,
// fixed order): (mass after bounce-back + link corrections + phase changes)
// / (fluid count + its change)
__global__ void k_prefill_avg(PartParams p, PartDev d) {
    if (d.status[0]) return;
    const int lane = threadIdx.x;
    double sum = 0.0;
    long long cnt = 0;
    for (int q = lane; q < p.np; q += 32) {
        for (int sl = 0; sl < NSLAB; sl++) sum += d.corr[q * NSLAB + sl];
        sum += d.prep_sum[q];
        cnt += d.prep_cnt[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
        const long long n1 = d.n_fluid[0] + cnt;
        d.rho_avg[1] = (d.rho_avg[2] + sum) / (double)n1;
        d.n_fluid[1] = n1;  // moved into slot 0 by k_pcommit
    }
}

// --------------------------------------------------- boundary links (IBB) --
// Deviation f - w rho0 of the post-collision value fp(q, c) of node c
// (coordinates as 0-based indices), read from the streamed array; nodes
// outside the walls hold the reference's ghost value omega*rho0 (deviation 0).
// L: arithmetic type of the population work (FP64 for FP64 storage, FP32 for
// FP32 storage).
template <typename S, typename L>
__device__ __forceinline__ L fp_dev(const S* f, int q, int i, int j, int k, const PartParams& p) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    if (j < 0 || j >= ny || k < 0 || k >= nz) return L(0);
    if (!p.periodic_x && (i < 0 || i >= nx)) return L(0);
    const long long P = (long long)nx * ny * nz;
    i = wrapx(i, nx);
    const int jj = j + ey19(q), kk = k + ez19(q), ir = i + ex19(q);
    long long idx;
    int qq = q;
    if (jj < 0 || jj >= ny || kk < 0 || kk >= nz || (!p.periodic_x && (ir < 0 || ir >= nx))) {
        qq = opp19(q);  // bounced back into slot opp(q) of c (w_q = w_opp(q))
        idx = qq * P + (i + (long long)nx * (j + (long long)ny * k));
    } else {
        idx = q * P + (wrapx(ir, nx) + (long long)nx * (jj + (long long)ny * kk));
    }
    if (PSt<S>::SHIFT) return (L)f[idx];
    return (L)((double)f[idx] - w19(qq) * p.rho0);
}

// Direction components for a direction index held in a register: 2-bit
// fields (component + 1) of one 64-bit constant per axis, so no compare chain.
__host__ __device__ constexpr unsigned long long pack_e(int axis) {
    unsigned long long v = 0;
    for (int a = 0; a < Q19; a++) {
        const int e = axis == 0 ? ex19(a) : (axis == 1 ? ey19(a) : ez19(a));
        v |= (unsigned long long)(e + 1) << (2 * a);
    }
    return v;
}
__device__ __forceinline__ int e_rt(unsigned long long pack, int a) {
    return (int)((pack >> (2 * a)) & 3ull) - 1;
}
constexpr unsigned long long EX_PACK = pack_e(0), EY_PACK = pack_e(1), EZ_PACK = pack_e(2);
__host__ __device__ constexpr int opp_rt(int a) {
    // 1<->2, 3<->4, 5<->6; 7<->10, 8<->9, 11<->14, 12<->13, 15<->18, 16<->17
    return a <= 6 ? (a & 1 ? a + 1 : a - 1) : ((a - 7) & 3) == 0 ? a + 3 : ((a - 7) & 3) == 3 ? a - 3
                                            : ((a - 7) & 3) == 1 ? a + 1 : a - 1;
}

constexpr bool opp_rt_ok() {
    for (int a = 1; a < Q19; a++)
        if (opp_rt(a) != opp19(a)) return false;
    return true;
}
static_assert(opp_rt_ok(), "opp_rt must match opp19");

// largest owner tile k_plinks stages in dynamic shared memory (beside its
// ~38 KB of static shared memory); bigger spheres read the mask from global
constexpr size_t TILE_MAX_BYTES = 160 * 1024;

// Link-list capacity of k_plinks: one scan round adds at most PB * 18 links,
// so the list is processed as soon as fewer than that many slots are free.
constexpr int LINK_CAP = PB * 27;

// Is node (i, j, k) (0-based, x unwrapped) a fluid node, or a ghost beyond a
// wall?  Only those have a post-collision value of this step.
__device__ __forceinline__ bool node_avail(int i, int j, int k, const PartParams& p,
                                           const int* __restrict__ owner) {
    if (j < 0 || j >= p.ny || k < 0 || k >= p.nz) return true;
    if (i < 0 || i >= p.nx) {
        if (!p.periodic_x) return true;
        i = wrapx(i, p.nx);
    }
    return owner[i + (long long)p.nx * (j + (long long)p.ny * k)] < 0;
}

// The interpolation weights of the quadratic bounce-back sum to one, so it is
// applied to deviations directly.  The momentum exchange of a link,
//   (e - u_w) fp - (-e - u_w) f_new = 2 e w rho0 + (e - u_w) dfp + (e + u_w) df_new,
// splits into a constant part and a small variable part.  The constant parts
// are summed exactly as integers: with m = 2 (axis links, w = 1/18) or 1
// (diagonal links, w = 1/36),
//   sum 2 e w rho0        = rho0/18 * sum m e
//   sum r x (2 e w rho0)  = rho0/18 * (sum m n x e - X x sum m e)
// because r = o + q e gives r x e = o x e, and o = n - X with n the node's
// (unwrapped) coordinates.  The variable parts use the population arithmetic
// type; q (calQ2) is computed in FP64 for the FP64 form and, from the FP64
// |x - X|^2 - R^2, in FP32 for the FP32 form.
// TILE: the owner ids of the slab's box plus a one-node halo are staged in
// dynamic shared memory (walls and, without periodicity, the x faces as -2),
// so the scan's 19 lookups per node stay on chip.
template <typename S, bool TILE>
__global__ void __launch_bounds__(PB) k_plinks(S* __restrict__ f, PartParams p, PartDev d) {
    using L = typename PC<S>::C;
    if (d.status[0]) return;
    const int c = blockIdx.x, slab = blockIdx.y;
    const double X0 = d.xc[3 * c], X1 = d.xc[3 * c + 1], X2 = d.xc[3 * c + 2];
    const L Ux = (L)d.uc[3 * c], Uy = (L)d.uc[3 * c + 1], Uz = (L)d.uc[3 * c + 2];
    const L Ox = (L)d.om[3 * c], Oy = (L)d.om[3 * c + 1], Oz = (L)d.om[3 * c + 2];
    const double R = p.radius;
    const L ravg = (L)d.rho_avg[0];
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const long long P = (long long)nx * ny * nz;
    // box of nodes within R+2 of the centre (1-based coordinate = index + 1)
    const int h = (int)ceil(R) + 2;
    const int ci = (int)floor(X0) - 1, cj = (int)floor(X1) - 1, ck = (int)floor(X2) - 1;
    const int bw = 2 * h + 2;
    const int kz0 = slab * bw / NSLAB, kz1 = (slab + 1) * bw / NSLAB;
    const int nbox = bw * bw * (kz1 - kz0);
    const float reach2f = (float)((R + 1.8) * (R + 1.8));  // |x - X| <= R + sqrt(2) for a link
    const float Xf0 = (float)X0, Xf1 = (float)X1, Xf2 = (float)X2, Lf = (float)p.nx;
    int nf[3] = {0, 0, 0};  // sum m e
    int nt[3] = {0, 0, 0};  // sum m (n x e)
    L av[7] = {L(0), L(0), L(0), L(0), L(0), L(0), L(0)};  // variable force, torque, mass change
    // Links are listed (box index, direction) over the scan rounds of PB box
    // nodes, in a deterministic order, and processed one per thread once the
    // list is nearly full or the box is done.
    __shared__ int s_t[LINK_CAP];
    __shared__ unsigned char s_dir[LINK_CAP];
    __shared__ int s_n;
    __shared__ int s_wsum[PB / 32];
    extern __shared__ int s_own[];
    const int TX = bw + 2, TY = bw + 2, TZ = kz1 - kz0 + 2;
    if (TILE) {
        for (int e = threadIdx.x; e < TX * TY * TZ; e += PB) {
            const int ti = e % TX, tj = (e / TX) % TY, tk = e / (TX * TY);
            int i = ci - h + ti - 1;
            const int j = cj - h + tj - 1, k = ck - h + kz0 + tk - 1;
            int o = -2;
            if (j >= 0 && j < ny && k >= 0 && k < nz) {
                if (p.periodic_x) i = i < 0 ? i + nx : (i >= nx ? i - nx : i);
                if (i >= 0 && i < nx) o = d.owner_cur[i + (long long)nx * (j + (long long)ny * k)];
            }
            s_own[e] = o;
        }
    }
    auto own_at = [&](int bi, int bj, int bk) {  // box coordinates, bk absolute in the box
        return s_own[(bi + 1) + TX * ((bj + 1) + TY * (bk - kz0 + 1))];
    };
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t0 = 0; t0 < nbox; t0 += PB) {
        unsigned my_dirs = 0;  // bit a: direction a is a boundary link of my node
        const int t = t0 + threadIdx.x;
        if (t < nbox) {
            const int bi = t % bw, bj = (t / bw) % bw, bk = kz0 + t / (bw * bw);
            int i = ci - h + bi;
            const int j = cj - h + bj, k = ck - h + bk;
            bool ok = !(j < 0 || j >= ny || k < 0 || k >= nz);
            if (ok) {
                // a filter only: every link node lies within R + sqrt(2) of the
                // centre, well inside the R + 1.8 kept here, so FP32 suffices
                float ox = (float)(i + 1) - Xf0;
                if (p.periodic_x) {
                    if (ox > 0.5f * Lf) ox -= Lf;
                    else if (ox < -0.5f * Lf) ox += Lf;
                }
                const float oy = (float)(j + 1) - Xf1, oz = (float)(k + 1) - Xf2;
                ok = ox * ox + oy * oy + oz * oz <= reach2f;
            }
            if (ok) {
                if (p.periodic_x) i = wrapx(i, nx);
                else ok = i >= 0 && i < nx;
            }
            if (TILE) {
                if (ok && own_at(bi, bj, bk) < 0) {
#pragma unroll
                    for (int a = 1; a < Q19; a++)
                        if (own_at(bi + ex19(a), bj + ey19(a), bk + ez19(a)) == c) my_dirs |= 1u << a;
                }
            } else if (ok && d.owner_cur[i + (long long)nx * (j + (long long)ny * k)] < 0) {
                for (int a = 1; a < Q19; a++) {
                    const int jn = j + ey19(a), kn = k + ez19(a);
                    if (jn < 0 || jn >= ny || kn < 0 || kn >= nz) continue;
                    int in = i + ex19(a);
                    if (p.periodic_x) in = wrapx(in, nx);
                    else if (in < 0 || in >= nx) continue;
                    if (d.owner_cur[in + (long long)nx * (jn + (long long)ny * kn)] != c) continue;
                    my_dirs |= 1u << a;
                }
            }
        }
        // deterministic slots: exclusive prefix sum of the per-thread link counts
        const int cnt = __popc(my_dirs);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) s_wsum[wid] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = s_n;
            for (int q = 0; q < PB / 32; q++) {
                const int v = s_wsum[q];
                s_wsum[q] = run;
                run += v;
            }
            s_n = run;
        }
        __syncthreads();
        int slot = s_wsum[wid] + incl - cnt;
        for (unsigned m = my_dirs; m; m &= m - 1) {
            s_t[slot] = t;
            s_dir[slot] = (unsigned char)(__ffs(m) - 1);
            slot++;
        }
        const int nl = s_n;
        if (nl <= LINK_CAP - PB * 18 && t0 + PB < nbox) continue;  // uniform over the block
        __syncthreads();
        for (int e = threadIdx.x; e < nl; e += PB) {
            const int tt = s_t[e], a = s_dir[e];
            const int bi = tt % bw, bj = (tt / bw) % bw, bk = kz0 + tt / (bw * bw);
            const int iu = ci - h + bi, j = cj - h + bj, k = ck - h + bk;  // iu: unwrapped
            const int i = p.periodic_x ? wrapx(iu, nx) : iu;
            const int ea = e_rt(EX_PACK, a), eb = e_rt(EY_PACK, a), ec = e_rt(EZ_PACK, a);
            const int m = a <= 6 ? 2 : 1;
            // the node lies within R + 1.8 < nx / 2 of the centre: the unwrapped
            // difference is the periodic minimum image
            const double ox = (double)(iu + 1) - X0, oy = (double)(j + 1) - X1,
                         oz = (double)(k + 1) - X2;
            // q: ray-sphere root from the node (calQ2, particle_bounceback.F90:144-185)
            const double sx = ea > 0 ? ox : (ea < 0 ? -ox : 0.0);
            const double sy = eb > 0 ? oy : (eb < 0 ? -oy : 0.0);
            const double sz = ec > 0 ? oz : (ec < 0 ? -oz : 0.0);
            const double cc = ox * ox + oy * oy + oz * oz - R * R;
            double qd = -1.0;
            bool exact = true;
            if constexpr (sizeof(L) == 4) {
                // FP32 form: |x - X|^2 - R^2 (the cancelling part) in FP64, the
                // root in FP32.  Its error grows where the ray is nearly tangent
                // (small delta) and matters where q is near 0 or 1, the ends
                // the range check tests: those links take the FP64 root, so the
                // FP32 and FP64 forms accept and reject the same links.
                const float cbf = 2.0f * (float)(sx + sy + sz);
                const float delta = cbf * cbf - (a <= 6 ? 4.0f : 8.0f) * (float)cc;
                const float qf = (-cbf - sqrtf(fmaxf(delta, 0.0f))) * (a <= 6 ? 0.5f : 0.25f);
                exact = !(delta > 1e-2f * cbf * cbf + 1e-3f && qf > 1e-3f && qf < 1.0f - 1e-3f);
                if (!exact) qd = (double)qf;
            }
            if (exact) {
                const double cb = 2.0 * (sx + sy + sz);
                const double delta = cb * cb - (a <= 6 ? 4.0 : 8.0) * cc;
                if (delta < 0) { atomicCAS(d.status, 0, PS_Q_RANGE); d.status[1] = c; continue; }
                qd = (-cb - sqrt(delta)) * (a <= 6 ? 0.5 : 0.25);  // /(2 |e|^2), exact
                if (qd > 1.0 || qd < 0.0) { atomicCAS(d.status, 0, PS_Q_RANGE); d.status[1] = c; continue; }
            }
            // constant parts (integers)
            const int n0 = iu + 1, n1 = j + 1, n2 = k + 1;
            nf[0] += m * ea;
            nf[1] += m * eb;
            nf[2] += m * ec;
            nt[0] += m * (n1 * ec - n2 * eb);
            nt[1] += m * (n2 * ea - n0 * ec);
            nt[2] += m * (n0 * eb - n1 * ea);
            // wall point relative to the centre and its velocity U + Omega x r
            const L q = (L)qd;
            const L rx = (L)ox + q * (L)ea, ry = (L)oy + q * (L)eb, rz = (L)oz + q * (L)ec;
            const L uw0 = Ux + (Oy * rz - Oz * ry);
            const L uw1 = Uy + (Oz * rx - Ox * rz);
            const L uw2 = Uz + (Ox * ry - Oy * rx);
            const int ra = opp_rt(a);
            const L w = a <= 6 ? L(1.0 / 18.0) : L(1.0 / 36.0);
            const L mv = L(6) * w * ravg * (-(L)ea * uw0 - (L)eb * uw1 - (L)ec * uw2);  // moving wall
            const L dpa = fp_dev<S, L>(f, a, i, j, k, p);
            // interpolation nodes inside a solid have no post-collision value
            // of this step: fall back to the linear IBB, then to simple
            // bounce-back (nodes beyond the walls are ghosts and available)
            const bool av1 = node_avail(i - ea, j - eb, k - ec, p, d.owner_cur);
            L dn;
            if (q < L(0.5)) {
                const bool av2 = node_avail(i - 2 * ea, j - 2 * eb, k - 2 * ec, p, d.owner_cur);
                if (av1 && av2) {
                    const L c0 = q * (L(1) + L(2) * q), c1 = L(1) - L(4) * q * q,
                            c2 = q * (L(1) - L(2) * q);
                    const L d1 = fp_dev<S, L>(f, a, i - ea, j - eb, k - ec, p);
                    const L d2 = fp_dev<S, L>(f, a, i - 2 * ea, j - 2 * eb, k - 2 * ec, p);
                    dn = c0 * dpa + c1 * d1 - c2 * d2 + mv;
                } else if (av1) {  // case1/mpi_complete/particle_bounceback.F90:66-69
                    const L d1 = fp_dev<S, L>(f, a, i - ea, j - eb, k - ec, p);
                    dn = L(2) * q * dpa + (L(1) - L(2) * q) * d1 + mv;
                } else {
                    dn = dpa + mv;
                }
            } else if (av1) {
                const L iq = L(1) / q, i2 = L(1) / (L(1) + L(2) * q), a2 = L(2) * q - L(1);
                const L g0 = fp_dev<S, L>(f, ra, i, j, k, p);
                const L g1 = fp_dev<S, L>(f, ra, i - ea, j - eb, k - ec, p);
                dn = (iq * i2) * dpa + (a2 * iq) * g0 - (a2 * i2) * g1 + (iq * i2) * mv;
            } else {  // case1/mpi_complete/particle_bounceback.F90:70-73
                const L h = L(0.5) / q;
                const L g0 = fp_dev<S, L>(f, ra, i, j, k, p);
                dn = h * dpa + (L(1) - h) * g0 + h * mv;
            }
            const long long fslot = ra * P + (i + (long long)nx * (j + (long long)ny * k));
            if (PSt<S>::SHIFT) {
                f[fslot] = (S)dn;
                dn = (L)f[fslot];  // as stored
            } else {
                const double wd = a <= 6 ? 1.0 / 18.0 : 1.0 / 36.0;
                f[fslot] = (S)((double)dn + wd * p.rho0);
                dn = (L)((double)f[fslot] - wd * p.rho0);
            }
            // Wen et al. 2014 Galilean-invariant momentum exchange, variable part
            const L F0 = ((L)ea - uw0) * dpa + ((L)ea + uw0) * dn;
            const L F1 = ((L)eb - uw1) * dpa + ((L)eb + uw1) * dn;
            const L F2 = ((L)ec - uw2) * dpa + ((L)ec + uw2) * dn;
            av[0] += F0;
            av[1] += F1;
            av[2] += F2;
            av[3] += ry * F2 - rz * F1;
            av[4] += rz * F0 - rx * F2;
            av[5] += rx * F1 - ry * F0;
            av[6] += dn - dpa;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_n = 0;
    }
    double acc[13];
#pragma unroll
    for (int q = 0; q < 7; q++) acc[q] = (double)av[q];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        acc[7 + q] = (double)nf[q];  // integers: the block sums are exact
        acc[10 + q] = (double)nt[q];
    }
    __shared__ double out[13];
    block_sum_to<13>(acc, out, 1);
    if (threadIdx.x == 0) {
        const double k0 = p.rho0 / 18.0;
        const double NF0 = out[7], NF1 = out[8], NF2 = out[9];
        const double fc[3] = {k0 * NF0, k0 * NF1, k0 * NF2};
        const double tc[3] = {k0 * (out[10] - (X1 * NF2 - X2 * NF1)),
                              k0 * (out[11] - (X2 * NF0 - X0 * NF2)),
                              k0 * (out[12] - (X0 * NF1 - X1 * NF0))};
        const int sl = c * NSLAB + slab;  // per-slab partials, summed in slab order by readers
        for (int q = 0; q < 3; q++) {
            d.flink[3 * sl + q] = fc[q] + out[q];
            d.tlink[3 * sl + q] = tc[q] + out[3 + q];
        }
        d.corr[sl] = out[6];
    }
}

// The node t = bi + bw (bj + bw bk) of a particle's box, walked by one thread
// in strides of PB without divisions: PB's digits in base bw are added with
// carries (the same nodes, in the same order, as t % bw, (t / bw) % bw, ...).
struct BoxWalk {
    int bi, bj, bk, ai, aj, ak, bw;
    __device__ BoxWalk(long long t0, int bw_) : bw(bw_) {
        const long long b2 = (long long)bw_ * bw_;
        bi = (int)(t0 % bw_);
        bj = (int)((t0 / bw_) % bw_);
        bk = (int)(t0 / b2);
        ai = PB % bw_;
        aj = (int)(((long long)PB / bw_) % bw_);
        ak = (int)((long long)PB / b2);
    }
    __device__ void next() {
        bi += ai;
        int carry = 0;
        if (bi >= bw) { bi -= bw; carry = 1; }
        bj += aj + carry;
        carry = 0;
        if (bj >= bw) { bj -= bw; carry = 1; }
        bk += ak + carry;
    }
};

// ----------------------------------------------------------- update --------
// particle_force.F90:96-190 in 3-D: one warp per particle; the lanes split the
// pair loop and a fixed shuffle tree adds their spring forces.
__global__ void k_pforce(PartParams p, PartDev d) {
    if (d.status[0]) return;
    const int np = p.np;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= np) return;
    const double R0 = p.radius, ravg = d.rho_avg[0];
    const double vol = 4.0 / 3.0 * p.pi * R0 * R0 * R0;
    const double* X = d.xc + 3 * c;
    double fij[3] = {0.0, 0.0, 0.0};
    const double Rc = R0;
    for (int c2 = lane; c2 < np; c2 += 32) {
        if (c2 == c) continue;
        const double* X2 = d.xc + 3 * c2;
        const double d0 = dxp(X[0], X2[0], p), d1 = X[1] - X2[1], d2 = X[2] - X2[2];
        const double thr = p.thr_part;
        const double reach = Rc + R0 + thr;
        if (fabs(d0) >= reach || fabs(d1) >= reach || fabs(d2) >= reach) continue;  // out of range
        const double dij = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        if (dij >= Rc + R0 + thr) {
        } else if (dij >= Rc + R0) {
            const double t = (dij - Rc - R0 - thr) / thr;
            fij[0] = fij[0] + p.scale_part * (t * t) * d0 / dij;
            fij[1] = fij[1] + p.scale_part * (t * t) * d1 / dij;
            fij[2] = fij[2] + p.scale_part * (t * t) * d2 / dij;
        } else {
            if (atomicCAS(d.status, 0, PS_OVERLAP) == 0) {
                d.status[1] = c;
                d.status[2] = c2;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fij[q] += __shfl_down_sync(0xffffffffu, fij[q], o);
    if (lane != 0) return;
    double fw[3] = {0.0, 0.0, 0.0};
    const double thw = p.thr_wall;
    for (int ax = 0; ax < 3; ax++) {
        if (ax == 0 && p.periodic_x) continue;
        const int nax = ax == 0 ? p.nx : (ax == 1 ? p.ny : p.nz);
        double dw = X[ax] - Rc - 1.0;
        if (dw < 0) {
            if (atomicCAS(d.status, 0, PS_WALL) == 0) d.status[1] = c;
        } else if (dw < thw) {
            fw[ax] = fw[ax] + p.scale_wall * ((dw - thw) / thw) * ((dw - thw) / thw);
        }
        dw = (double)nax - X[ax] - Rc;
        if (dw < 0) {
            if (atomicCAS(d.status, 0, PS_WALL) == 0) d.status[1] = c;
        } else if (dw < thw) {
            fw[ax] = fw[ax] - p.scale_wall * ((dw - thw) / thw) * ((dw - thw) / thw);
        }
    }
    for (int q = 0; q < 3; q++) {
        double fl = 0.0, tl = 0.0;
        for (int sl = 0; sl < NSLAB; sl++) {
            fl += d.flink[3 * (c * NSLAB + sl) + q];
            tl += d.tlink[3 * (c * NSLAB + sl) + q];
        }
        double tot = fl + (p.rho_solid - ravg) * vol * p.gravity[q] + fij[q] + fw[q];
        tot = tot + ravg * vol * p.body_force[q];
        d.ftot[3 * c + q] = tot;
        d.ttot[3 * c + q] = tl;
    }
}

// particle_update.F90:26-50 in 3-D, one thread per particle
__global__ void k_pmove(PartParams p, PartDev d) {
    if (d.status[0]) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.np) return;
    const double R0 = p.radius;
    const double M = p.rho_solid * 4.0 / 3.0 * p.pi * R0 * R0 * R0;
    const double I = 0.4 * M * R0 * R0;
    bool ok = true;
    for (int q = 0; q < 3; q++) {
        d.xc_old[3 * c + q] = d.xc[3 * c + q];
        d.uc_old[3 * c + q] = d.uc[3 * c + q];
        d.om_old[3 * c + q] = d.om[3 * c + q];
        const double a = d.ftot[3 * c + q] / M;
        d.uc[3 * c + q] = d.uc_old[3 * c + q] + a;
        d.om[3 * c + q] = d.om_old[3 * c + q] + d.ttot[3 * c + q] / I;
        d.xc[3 * c + q] = d.xc_old[3 * c + q] + d.uc_old[3 * c + q] + 0.5 * a;
        ok = ok && isfinite(d.xc[3 * c + q]) && isfinite(d.uc[3 * c + q]) &&
             isfinite(d.om[3 * c + q]);
    }
    if (p.periodic_x) {
        // one wrap per step is enough only while the step moves the centre by
        // less than half the periodic length
        const double L = (double)p.nx;
        ok = ok && fabs(d.xc[3 * c] - d.xc_old[3 * c]) < 0.5 * L;
        if (d.xc[3 * c] >= L + 0.5) d.xc[3 * c] -= L;
        if (d.xc[3 * c] < 0.5) d.xc[3 * c] += L;
    }
    if (!ok && atomicCAS(d.status, 0, PS_DIVERGED) == 0) d.status[1] = c;
}

// -------------------------------------------------------------- new mask --
__global__ void __launch_bounds__(PB) k_pmark(int* owner, const double* xc, PartParams p,
                                                const int* status, bool check_status) {
    if (check_status && status[0]) return;
    const int c = blockIdx.x;
    const double* X = xc + 3 * c;
    const double R = p.radius;
    const int h = (int)ceil(R) + 1;
    const int ci = (int)floor(X[0]) - 1, cj = (int)floor(X[1]) - 1, ck = (int)floor(X[2]) - 1;
    const int bw = 2 * h + 2;
    const long long nbox = (long long)bw * bw * bw;
    const float Xf0 = (float)X[0], Xf1 = (float)X[1], Xf2 = (float)X[2], Lf = (float)p.nx;
    const float Xmax = fmaxf(fabsf(Xf0), fmaxf(fabsf(Xf1), fabsf(Xf2))) + Lf;  // wrapped nodes too
    BoxWalk bw_it(threadIdx.x, bw);
    for (long long t = threadIdx.x; t < nbox; t += PB, bw_it.next()) {
        const int bi = bw_it.bi, bj = bw_it.bj, bk = bw_it.bk;
        int i = ci - h + bi;
        const int j = cj - h + bj, k = ck - h + bk;
        if (j < 0 || j >= p.ny || k < 0 || k >= p.nz) continue;
        if (p.periodic_x) i = wrapx(i, p.nx);
        else if (i < 0 || i >= p.nx) continue;
        // FP32 decides far from the surface; nodes within tol of it use the
        // IEEE-rounded FP64 test.  tol bounds the FP32 error of d2 (the centre
        // rounded to FP32, then the differences, squares and sums) at least
        // twice over, so wherever FP32 decides, its decision is the FP64 test's.
        float fx = (float)(i + 1) - Xf0;
        if (p.periodic_x) {
            if (fx > 0.5f * Lf) fx -= Lf;
            else if (fx < -0.5f * Lf) fx += Lf;
        }
        const float fy = (float)(j + 1) - Xf1, fz = (float)(k + 1) - Xf2;
        const float d2 = fx * fx + fy * fy + fz * fz, r2 = (float)(R * R);
        const float tol = 1e-3f * r2 + 4e-6f * (float)(h + 1) * (Xmax + (float)(h + 1)) + 1e-6f * d2;
        bool in;
        if (fabsf(d2 - r2) > tol) in = d2 < r2;
        else in = inside((double)(i + 1), (double)(j + 1), (double)(k + 1), X, R, p);
        if (in) owner[i + (long long)p.nx * (j + (long long)p.ny * k)] = c;
    }
}

// nodes that change phase: density bookkeeping of the average used by the refill
template <typename S>
__global__ void __launch_bounds__(PB) k_pprep(const S* __restrict__ f, PartParams p, PartDev d) {
    if (d.status[0]) return;
    const int c = blockIdx.x;
    const long long P = (long long)p.nx * p.ny * p.nz;
    double sum = 0.0;
    int cnt = 0;
    for (int pass = 0; pass < 2; pass++) {
        const double* X = (pass == 0 ? d.xc_old : d.xc) + 3 * c;
        const int h = (int)ceil(p.radius) + 1;
        const int ci = (int)floor(X[0]) - 1, cj = (int)floor(X[1]) - 1, ck = (int)floor(X[2]) - 1;
        const int bw = 2 * h + 2;
        const long long nbox = (long long)bw * bw * bw;
        BoxWalk bw_it(threadIdx.x, bw);
        for (long long t = threadIdx.x; t < nbox; t += PB, bw_it.next()) {
            const int bi = bw_it.bi, bj = bw_it.bj, bk = bw_it.bk;
            int i = ci - h + bi;
            const int j = cj - h + bj, k = ck - h + bk;
            if (j < 0 || j >= p.ny || k < 0 || k >= p.nz) continue;
            if (p.periodic_x) i = wrapx(i, p.nx);
            else if (i < 0 || i >= p.nx) continue;
            const long long cell = i + (long long)p.nx * (j + (long long)p.ny * k);
            const int oc = d.owner_cur[cell], on = d.owner_new[cell];
            if (pass == 0 && oc == c && on < 0) {  // leaves particle c: counted with rho_solid
                sum += p.rho_solid;
                cnt += 1;
            }
            if (pass == 1 && oc < 0 && on == c) {  // enters particle c: drop its density
                double r = 0.0;
                for (int q = 0; q < Q19; q++) r += pabs<S>(f, q * P + cell, q, p.rho0);
                sum -= r;
                cnt -= 1;
            }
        }
    }
    double acc[2] = {sum, (double)cnt};
    __shared__ double out[2];
    block_sum_to<2>(acc, out, 1);
    if (threadIdx.x == 0) {
        d.prep_sum[c] = out[0];
        d.prep_cnt[c] = (int)llround(out[1]);
    }
}

// D3Q19 forward moments and inverse in the reference's basis, FP64
__device__ void moments19d(const double* f, double* m) {
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] +
           f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    m[1] = -30.0 * f[0] - 11.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6]) +
           8.0 * (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18]);
    m[2] = 12.0 * f[0] - 4.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6]) + f[7] + f[8] + f[9] +
           f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    m[3] = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[4] = -4.0 * (f[1] - f[2]) + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[5] = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[6] = -4.0 * (f[3] - f[4]) + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[7] = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[8] = -4.0 * (f[5] - f[6]) + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[9] = 2.0 * (f[1] + f[2]) - f[3] - f[4] - f[5] - f[6] + f[7] + f[8] + f[9] + f[10] + f[11] +
           f[12] + f[13] + f[14] - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[10] = -4.0 * (f[1] + f[2]) + 2.0 * (f[3] + f[4] + f[5] + f[6]) + f[7] + f[8] + f[9] + f[10] +
            f[11] + f[12] + f[13] + f[14] - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[11] = f[3] + f[4] - f[5] - f[6] + f[7] + f[8] + f[9] + f[10] - (f[11] + f[12] + f[13] + f[14]);
    m[12] = -2.0 * (f[3] + f[4] - f[5] - f[6]) + (f[7] + f[8] + f[9] + f[10]) - (f[11] + f[12] + f[13] + f[14]);
    m[13] = f[7] - f[8] - f[9] + f[10];
    m[14] = f[15] - f[16] - f[17] + f[18];
    m[15] = f[11] - f[12] - f[13] + f[14];
    m[16] = f[7] - f[8] + f[9] - f[10] - f[11] + f[12] - f[13] + f[14];
    m[17] = -f[7] - f[8] + f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    m[18] = f[11] + f[12] - f[13] - f[14] - f[15] - f[16] + f[17] + f[18];
}
// f = M^-1 m with M^-1 = M^T diag(1/|M_k|^2)
__device__ void inverse19d(const double* m, double* f) {
    const double a0 = m[0] / 19.0, a1 = m[1] / 2394.0, a2 = m[2] / 252.0;
    const double b3 = m[3] / 10.0, b4 = m[4] / 40.0, b5 = m[5] / 10.0, b6 = m[6] / 40.0,
                 b7 = m[7] / 10.0, b8 = m[8] / 40.0;
    const double c9 = m[9] / 36.0, c10 = m[10] / 72.0, c11 = m[11] / 12.0, c12 = m[12] / 24.0;
    const double d13 = m[13] / 4.0, d14 = m[14] / 4.0, d15 = m[15] / 4.0;
    const double e16 = m[16] / 8.0, e17 = m[17] / 8.0, e18 = m[18] / 8.0;
    f[0] = a0 - 30.0 * a1 + 12.0 * a2;
    const double ax = a0 - 11.0 * a1 - 4.0 * a2, ed = a0 + 8.0 * a1 + a2;
    f[1] = ax + (b3 - 4.0 * b4) + (2.0 * c9 - 4.0 * c10);
    f[2] = ax - (b3 - 4.0 * b4) + (2.0 * c9 - 4.0 * c10);
    f[3] = ax + (b5 - 4.0 * b6) - c9 + 2.0 * c10 + c11 - 2.0 * c12;
    f[4] = ax - (b5 - 4.0 * b6) - c9 + 2.0 * c10 + c11 - 2.0 * c12;
    f[5] = ax + (b7 - 4.0 * b8) - c9 + 2.0 * c10 - c11 + 2.0 * c12;
    f[6] = ax - (b7 - 4.0 * b8) - c9 + 2.0 * c10 - c11 + 2.0 * c12;
    const double E = ed + c9 + c10;
    f[7] = E + c11 + c12 + d13 + (b3 + b4 + b5 + b6) + e16 - e17;
    f[10] = E + c11 + c12 + d13 - (b3 + b4 + b5 + b6) - e16 + e17;
    f[9] = E + c11 + c12 - d13 + (b3 + b4 - b5 - b6) + e16 + e17;
    f[8] = E + c11 + c12 - d13 - (b3 + b4 - b5 - b6) - e16 - e17;
    f[11] = E - c11 - c12 + d15 + (b3 + b4 + b7 + b8) - e16 + e18;
    f[14] = E - c11 - c12 + d15 - (b3 + b4 + b7 + b8) + e16 - e18;
    f[13] = E - c11 - c12 - d15 + (b3 + b4 - b7 - b8) - e16 - e18;
    f[12] = E - c11 - c12 - d15 - (b3 + b4 - b7 - b8) + e16 + e18;
    const double Ez = ed - 2.0 * c9 - 2.0 * c10;
    f[15] = Ez + d14 + (b5 + b6 + b7 + b8) + e17 - e18;
    f[18] = Ez + d14 - (b5 + b6 + b7 + b8) - e17 + e18;
    f[17] = Ez - d14 + (b5 + b6 - b7 - b8) + e17 + e18;
    f[16] = Ez - d14 - (b5 + b6 - b7 - b8) - e17 - e18;
}

// refill (particle_update.F90:134-193 in 3-D): extrapolate along the lattice
// direction closest to the outward normal, then reset the momentum moments to
// rho_avg times the wall velocity.  All of a particle's refills read before
// any of them is written.
template <typename S>
__global__ void __launch_bounds__(PB) k_prefill(S* __restrict__ f, PartParams p, PartDev d,
                                                int nblocks_bulk) {
    if (d.status[0]) return;
    const int c = blockIdx.x;
    const long long P = (long long)p.nx * p.ny * p.nz;
    __shared__ double s_val[REFILL_MAX][Q19];
    __shared__ long long s_cell[REFILL_MAX];
    __shared__ int s_n;
    __shared__ double s_ravg;
    if (threadIdx.x == 0) {
        s_n = 0;
        s_ravg = d.rho_avg[1];
    }
    __syncthreads();
    const double* X = d.xc + 3 * c;       // new centre
    const double* Xo = d.xc_old + 3 * c;  // old centre: the nodes it covered
    const double* U = d.uc + 3 * c;
    const double* O = d.om + 3 * c;
    const int h = (int)ceil(p.radius) + 1;
    const int ci = (int)floor(Xo[0]) - 1, cj = (int)floor(Xo[1]) - 1, ck = (int)floor(Xo[2]) - 1;
    const int bw = 2 * h + 2;
    const long long nbox = (long long)bw * bw * bw;
    BoxWalk bw_it(threadIdx.x, bw);
    for (long long t = threadIdx.x; t < nbox; t += PB, bw_it.next()) {
        const int bi = bw_it.bi, bj = bw_it.bj, bk = bw_it.bk;
        int i = ci - h + bi;
        const int j = cj - h + bj, k = ck - h + bk;
        if (j < 0 || j >= p.ny || k < 0 || k >= p.nz) continue;
        if (p.periodic_x) i = wrapx(i, p.nx);
        else if (i < 0 || i >= p.nx) continue;
        const long long cell = i + (long long)p.nx * (j + (long long)p.ny * k);
        if (!(d.owner_cur[cell] == c && d.owner_new[cell] < 0)) continue;
        const double rx = dxp((double)(i + 1), X[0], p), ry = (double)(j + 1) - X[1],
                     rz = (double)(k + 1) - X[2];
        double out = 0.0;
        int ec = 0;
        const double rn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
        for (int a = 1; a < Q19; a++) {
            const double tn = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, (double)ex19(a)), __dmul_rn(ry, (double)ey19(a))),
                                                  __dmul_rn(rz, (double)ez19(a))), rn);
            if (tn > out) {
                out = tn;
                ec = a;
            }
        }
        if (ec == 0) {
            atomicCAS(d.status, 0, PS_NO_REFILL_DIR);
            continue;
        }
        const int e0 = ex19(ec), e1 = ey19(ec), e2 = ez19(ec);
        double fl[Q19], m[Q19];
        for (int a = 0; a < Q19; a++) {
            double fv[3];
            for (int s = 1; s <= 3; s++) {
                const int ii = p.periodic_x ? wrapx(i + s * e0, p.nx) : i + s * e0;
                const int jj = j + s * e1, kk = k + s * e2;
                if (ii < 0 || ii >= p.nx || jj < 0 || jj >= p.ny || kk < 0 || kk >= p.nz)
                    fv[s - 1] = w19(a) * p.rho0;  // ghost value
                else
                    fv[s - 1] = pabs<S>(f, a * P + (ii + (long long)p.nx * (jj + (long long)p.ny * kk)), a, p.rho0);
            }
            // 3 f(x+e) - 3 f(x+2e) + f(x+3e) (particle_update.F90:157-159)
            fl[a] = __dadd_rn(__dsub_rn(__dmul_rn(3.0, fv[0]), __dmul_rn(3.0, fv[1])), fv[2]);
        }
        moments19d(fl, m);
        const double x0 = X[0] + rx, y0 = (double)(j + 1), z0 = (double)(k + 1);
        const double qx = x0 - X[0], qy = y0 - X[1], qz = z0 - X[2];
        m[3] = s_ravg * (U[0] + (O[1] * qz - O[2] * qy));
        m[5] = s_ravg * (U[1] + (O[2] * qx - O[0] * qz));
        m[7] = s_ravg * (U[2] + (O[0] * qy - O[1] * qx));
        inverse19d(m, fl);
        const int slot = atomicAdd(&s_n, 1);
        if (slot >= REFILL_MAX) {
            atomicCAS(d.status, 0, PS_REFILL_FULL);
            continue;
        }
        s_cell[slot] = cell;
        for (int a = 0; a < Q19; a++) s_val[slot][a] = fl[a];
    }
    __syncthreads();
    const int n = min(s_n, REFILL_MAX);
    for (int t = threadIdx.x; t < n * Q19; t += PB) {
        const int slot = t / Q19, a = t % Q19;
        pset<S>(f, a * P + s_cell[slot], a, s_val[slot][a], p.rho0);
    }
}

__global__ void k_pcommit(PartDev d) {
    if (d.status[0]) return;
    d.n_fluid[0] = d.n_fluid[1];
}

// ------------------------------------------------------------ initialise --
template <typename S>
__global__ void k_pinit_f(S* f, const int* owner, PartParams p) {
    const long long P = (long long)p.nx * p.ny * p.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P;
         c += (long long)gridDim.x * blockDim.x) {
        const bool fluid = owner[c] < 0;
        for (int q = 0; q < Q19; q++) pset<S>(f, q * P + c, q, fluid ? w19(q) * (1.0 + 0.0) : 0.0, p.rho0);
    }
}
__global__ void k_pcount(const int* owner, long long n, long long* out) {
    long long cnt = 0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        cnt += owner[c] < 0;
    double acc[1] = {(double)cnt};
    __shared__ double o[1];
    block_sum_to<1>(acc, o, 1);
    if (threadIdx.x == 0) out[0] = llround(o[0]);
}

template <typename S>
__global__ void k_pmacro(const S* f, const int* owner, PartParams p, bool first, double* rho,
                         double* u, double* v, double* w) {
    const long long P = (long long)p.nx * p.ny * p.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P;
         c += (long long)gridDim.x * blockDim.x) {
        if (owner[c] >= 0) {
            rho[c] = p.rho_solid;
            u[c] = v[c] = w[c] = 0.0;
            continue;
        }
        if (first) {
            rho[c] = p.rho0;
            u[c] = v[c] = w[c] = 0.0;
            continue;
        }
        double fq[Q19];
        for (int q = 0; q < Q19; q++) fq[q] = pabs<S>(f, q * P + c, q, p.rho0);
        double r = fq[0];
        for (int q = 1; q < Q19; q++) r += fq[q];
        double jx = 0.0, jy = 0.0, jz = 0.0;
        for (int q = 1; q < Q19; q++) {
            jx += ex19(q) * fq[q];
            jy += ey19(q) * fq[q];
            jz += ez19(q) * fq[q];
        }
        rho[c] = r;
        u[c] = (jx + 0.5 * (r * p.body_force[0])) / r;
        v[c] = (jy + 0.5 * (r * p.body_force[1])) / r;
        w[c] = (jz + 0.5 * (r * p.body_force[2])) / r;
    }
}

// ---------------------------------------------------------------- launch --
static dim3 pblock(int nx) {
    int bx = ((nx + 31) / 32) * 32;
    return dim3(bx > 128 ? 128 : bx, 1, 1);
}
// number of per-warp partial slots of the bulk kernel
int particle_bulk_blocks(const PartParams& p) {
    dim3 b = pblock(p.nx);
    return ((p.nx + b.x - 1) / b.x) * p.ny * p.nz * (int)(b.x / 32);
}

template <typename S>
static cudaError_t pstep_go(bool first, const void* fin, void* fout, const PartParams& p,
                            const PartDev& d, cudaStream_t s) {
    using C = typename PC<S>::C;
    dim3 b = pblock(p.nx), g((p.nx + b.x - 1) / b.x, p.ny, p.nz);
    MrtCoef<C> cd = cast_coef<C>(make_mrt_coef(p.snu, p.sq));
    const PBulkK<C> bk = {(C)p.rho0, (C)p.body_force[0], (C)p.body_force[1], (C)p.body_force[2]};
    // 32-bit indices while every population index (and the +-1 neighbour
    // offsets) fits in int
    const bool i32 = (long long)p.nx * p.ny * p.nz * (Q19 + 1) < (1LL << 31);
    const S* fi = (const S*)fin;
    S* fo = (S*)fout;
    if (first && i32) k_pbulk<S, true, int><<<g, b, 0, s>>>(fi, fo, d.owner_cur, p, cd, bk, d.partials, d.status);
    else if (first) k_pbulk<S, true, long long><<<g, b, 0, s>>>(fi, fo, d.owner_cur, p, cd, bk, d.partials, d.status);
    else if (i32) k_pbulk<S, false, int><<<g, b, 0, s>>>(fi, fo, d.owner_cur, p, cd, bk, d.partials, d.status);
    else k_pbulk<S, false, long long><<<g, b, 0, s>>>(fi, fo, d.owner_cur, p, cd, bk, d.partials, d.status);
    k_pfinish<<<FINISH_BLOCKS, 256, 0, s>>>(d, d.nblocks);
    k_pfinish2<<<1, 32, 0, s>>>(d, d.nblocks);
    if (p.np > 0) {
        const int bw = 2 * ((int)ceil(p.radius) + 2) + 2;
        const size_t tile = sizeof(int) * (size_t)(bw + 2) * (bw + 2) * ((bw + NSLAB - 1) / NSLAB + 2);
        if (tile <= TILE_MAX_BYTES) {
            // the shared-memory opt-in is a per-device attribute of the kernel
            static std::atomic<unsigned long long> opted{0};  // bit = device ordinal
            int dev = 0;
            cudaGetDevice(&dev);
            const unsigned long long bit = 1ull << (dev & 63);
            if (!(opted.load() & bit)) {
                cudaError_t e = cudaFuncSetAttribute(k_plinks<S, true>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)TILE_MAX_BYTES);
                if (e != cudaSuccess) return e;
                opted.fetch_or(bit);
            }
            k_plinks<S, true><<<dim3(p.np, NSLAB), PB, tile, s>>>((S*)fout, p, d);
        } else {
            k_plinks<S, false><<<dim3(p.np, NSLAB), PB, 0, s>>>((S*)fout, p, d);
        }
        // one warp per particle, one warp per block: the particles spread over the SMs
        k_pforce<<<p.np, 32, 0, s>>>(p, d);
        k_pmove<<<(p.np + 31) / 32, 32, 0, s>>>(p, d);
    }
    cudaError_t e = cudaMemsetAsync(d.owner_new, 0xFF, sizeof(int) * (size_t)p.nx * p.ny * p.nz, s);
    if (e != cudaSuccess) return e;
    if (p.np > 0) {
        k_pmark<<<p.np, PB, 0, s>>>(d.owner_new, d.xc, p, d.status, true);
        k_pprep<S><<<p.np, PB, 0, s>>>((const S*)fout, p, d);
        k_prefill_avg<<<1, 32, 0, s>>>(p, d);
        k_prefill<S><<<p.np, PB, 0, s>>>((S*)fout, p, d, d.nblocks);
        k_pcommit<<<1, 1, 0, s>>>(d);
    }
    return cudaGetLastError();
}

cudaError_t launch_particle_step(int form, bool first, const void* fin, void* fout,
                                 const PartParams& p, const PartDev& d, cudaStream_t s) {
    if (form == FORM_FP64) return pstep_go<double>(first, fin, fout, p, d, s);
    if (form == FORM_FP32) return pstep_go<float>(first, fin, fout, p, d, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_particle_init(int form, void* f, const PartParams& p, const PartDev& d,
                                 cudaStream_t s) {
    const long long n = (long long)p.nx * p.ny * p.nz;
    cudaError_t e = cudaMemsetAsync(d.owner_cur, 0xFF, sizeof(int) * (size_t)n, s);
    if (e != cudaSuccess) return e;
    if (p.np > 0) k_pmark<<<p.np, PB, 0, s>>>(d.owner_cur, d.xc, p, d.status, false);
    int gb = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    if (form == FORM_FP64) k_pinit_f<double><<<gb, 256, 0, s>>>((double*)f, d.owner_cur, p);
    else k_pinit_f<float><<<gb, 256, 0, s>>>((float*)f, d.owner_cur, p);
    k_pcount<<<1, 1024, 0, s>>>(d.owner_cur, n, d.n_fluid);
    return cudaGetLastError();
}

cudaError_t launch_particle_macro(int form, bool first, const void* f, const PartParams& p,
                                  const PartDev& d, double* rho, double* u, double* v, double* w,
                                  cudaStream_t s) {
    const long long n = (long long)p.nx * p.ny * p.nz;
    int gb = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    if (form == FORM_FP64)
        k_pmacro<double><<<gb, 256, 0, s>>>((const double*)f, d.owner_cur, p, first, rho, u, v, w);
    else
        k_pmacro<float><<<gb, 256, 0, s>>>((const float*)f, d.owner_cur, p, first, rho, u, v, w);
    return cudaGetLastError();
}

}  // namespace mglc
