// step_cell.cuh -- per-cell bodies of the fused lattice-Boltzmann steps,
// shared by the one-solve kernels (k_step.cu) and the multi-solve tile-queue
// kernel of the solve server (k_serve.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "fixed64.cuh"
#include "kernels.cuh"

namespace mglc {

// ---------------------------------------------------------------- storage --
template <typename S>
struct St;
// SCALED (16-bit types): the cell bodies compute in units of the storage
// scale (a power of two, so every product with it is exact and the results
// are bitwise those of unscaled arithmetic); cvt_s / st_s / st_sr_s convert
// without the scale multiply.
template <>
struct St<double> {
    using C = double;
    static constexpr bool SHIFT = false;
    static constexpr bool SCALED = false;
    __device__ static C cvt_s(double v) { return v; }
    __device__ static void st_s(double* p, C v) { *p = v; }
    __device__ static void st_sr_s(double* p, C v, unsigned) { *p = v; }
    __device__ static C ld(const double* p, float) { return __ldg(p); }
    __device__ static double raw(const double* p) { return __ldg(p); }
    // raw_rw: plain load, for a buffer that the same kernel also writes
    __device__ static double raw_rw(const double* p) { return *p; }
    __device__ static void st_sr(double* p, C v, float, unsigned) { *p = v; }
    __device__ static C cvt(double v, float) { return v; }
    __device__ static void st(double* p, C v, float) { *p = v; }
};
template <>
struct St<float> {
    using C = float;
    static constexpr bool SHIFT = true;
    static constexpr bool SCALED = false;
    __device__ static C cvt_s(float v) { return v; }
    __device__ static void st_s(float* p, C v) { *p = v; }
    __device__ static void st_sr_s(float* p, C v, unsigned) { *p = v; }
    __device__ static C ld(const float* p, float) { return __ldg(p); }
    __device__ static float raw(const float* p) { return __ldg(p); }
    __device__ static float raw_rw(const float* p) { return *p; }
    __device__ static void st_sr(float* p, C v, float, unsigned) { *p = v; }
    __device__ static C cvt(float v, float) { return v; }
    __device__ static void st(float* p, C v, float) { *p = v; }
};
template <>
struct St<__half> {
    using C = float;
    static constexpr bool SHIFT = true;
    static constexpr bool SCALED = true;
    __device__ static C cvt_s(__half v) { return __half2float(v); }
    __device__ static void st_s(__half* p, C v) { *p = __float2half_rn(v); }
    __device__ static void st_sr_s(__half* p, C v, unsigned r) {
        *p = __float2half_rz(__uint_as_float(__float_as_uint(v) + (r >> 19)));
    }
    // two values rounded stochastically by the conversion itself (cvt.rs):
    // a into the high half, b into the low half, each with its own 16 bits
    // of r; NaN and infinities convert as themselves
    __device__ static unsigned pack_sr(float a, float b, unsigned r) {
        unsigned d;
        asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a), "f"(b), "r"(r));
        return d;
    }
    __device__ static void st_bits(__half* p, unsigned short v) { *p = __ushort_as_half(v); }
    __device__ static C ld(const __half* p, float inv) { return __half2float(__ldg(p)) * inv; }
    __device__ static __half raw(const __half* p) { return __ldg(p); }
    __device__ static __half raw_rw(const __half* p) { return *p; }
    // stochastic rounding: 13 uniform bits added below the 10 kept mantissa
    // bits, then truncation (unbiased; rounding errors do not correlate from
    // step to step, so they do not accumulate into a drift)
    // (finite values only: adding to a NaN pattern could wrap into the sign
    // bit; the cell bodies round to nearest in cells whose rho or u is not finite)
    __device__ static void st_sr(__half* p, C v, float sc, unsigned r) {
        *p = __float2half_rz(__uint_as_float(__float_as_uint(v * sc) + (r >> 19)));
    }
    __device__ static C cvt(__half v, float inv) { return __half2float(v) * inv; }
    __device__ static void st(__half* p, C v, float sc) { *p = __float2half_rn(v * sc); }
};
template <>
struct St<__nv_bfloat16> {
    using C = float;
    static constexpr bool SHIFT = true;
    static constexpr bool SCALED = true;
    __device__ static C cvt_s(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static void st_s(__nv_bfloat16* p, C v) { *p = __float2bfloat16_rn(v); }
    __device__ static void st_sr_s(__nv_bfloat16* p, C v, unsigned r) {
        *p = __float2bfloat16_rz(__uint_as_float(__float_as_uint(v) + (r >> 16)));
    }
    __device__ static unsigned pack_sr(float a, float b, unsigned r) {
        unsigned d;
        asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a), "f"(b), "r"(r));
        return d;
    }
    __device__ static void st_bits(__nv_bfloat16* p, unsigned short v) {
        *p = __ushort_as_bfloat16(v);
    }
    __device__ static C ld(const __nv_bfloat16* p, float inv) {
        return __bfloat162float(__ldg(p)) * inv;
    }
    __device__ static __nv_bfloat16 raw(const __nv_bfloat16* p) { return __ldg(p); }
    __device__ static __nv_bfloat16 raw_rw(const __nv_bfloat16* p) { return *p; }
    __device__ static void st_sr(__nv_bfloat16* p, C v, float sc, unsigned r) {
        *p = __float2bfloat16_rz(__uint_as_float(__float_as_uint(v * sc) + (r >> 16)));
    }
    __device__ static C cvt(__nv_bfloat16 v, float inv) { return __bfloat162float(v) * inv; }
    __device__ static void st(__nv_bfloat16* p, C v, float sc) { *p = __float2bfloat16_rn(v * sc); }
};

// ----------------------------------------------------- bounds checking --
// Built with MGLC_BOUNDS_CHECK (mglc_gb300/build.py, environment variable of
// the same name), every global access of the cell bodies below checks its
// element index against its array's extent; an index outside is counted
// (per translation unit, read by the host through mglc_debug_bounds_hits)
// and the access is skipped: a diagnostic build that cannot fault on a bad
// index.  Without the macro the checks compile to nothing.
#ifdef MGLC_BOUNDS_CHECK
static __device__ unsigned long long g_oob_hits;
template <typename IDX>
__device__ __forceinline__ bool oob(IDX idx, IDX limit) {
    if ((long long)idx < 0 || idx >= limit) {
        atomicAdd(&g_oob_hits, 1ull);
        return true;
    }
    return false;
}
#define MGLC_OOB_READER(NAME)                                                  \
    extern "C" unsigned long long NAME() {                                     \
        unsigned long long h = 0;                                              \
        if (cudaMemcpyFromSymbol(&h, mglc::g_oob_hits, sizeof h) != cudaSuccess) {\
            cudaGetLastError();                                                \
            return ~0ull;                                                      \
        }                                                                      \
        return h;                                                              \
    }
#else
template <typename IDX>
__device__ __forceinline__ bool oob(IDX, IDX) {
    return false;
}
#define MGLC_OOB_READER(NAME)
#endif
// checked store p[idx] = v (skipped when idx is outside [0, limit))
template <typename T, typename V, typename IDX>
__device__ __forceinline__ void st_chk(T* p, IDX idx, IDX limit, V v) {
    if (!oob(idx, limit)) p[idx] = v;
}

// Reciprocal of the density (rho is within a few percent of 1 in every
// cavity flow).  FP32: the hardware reciprocal.  FP64: Newton-Raphson
// refinement r <- r + r(1 - x r) of a single-precision seed; two steps take
// the 2^-23 seed error below 2^-52 with four FP64 FMAs, about half the FP64
// work of an IEEE division.
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip(double x) {
    double r = (double)__frcp_rn((float)x);
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Minimum resident blocks of 128 threads per SM for the lid step kernels: the
// FP64 kernels are bound by the FP64 pipe, and 8 blocks (64 registers, a few
// spilled values) measured 5% faster at 384^3 than the compiler's own 80
// registers and 6 blocks (7 blocks: 4%); the other forms keep the compiler's
// choice (0: no bound; a bound of 12 or 16 blocks slowed the 16-bit kernels by
// 7-30%).
template <typename S>
struct LidMinBlocks {
    static constexpr int value = std::is_same<S, double>::value ? 8 : 0;
};

// Scalar constants converted once on the host to the arithmetic type.
template <typename C>
struct StepK {
    int nx, ny, nz;
    C u0, rho0;
    float scale, inv_scale;
    unsigned seed;  // one-solve kernels: the step index (stochastic rounding)
    int sr;         // 1: 16-bit stores round stochastically, 0: to nearest
    MrtCoef<C> c;
    // thermal
    C gbeta, omega_rot, t_ref, para_a, qd, qnu, chot, ccold;
    int bc_y, bc_z;
};

template <typename C>
inline StepK<C> make_k(const Geom& g, const MrtCoef<double>& cd, double u0, double rho0,
                       float scale, float inv_scale) {
    StepK<C> k{};
    k.nx = g.nx; k.ny = g.ny; k.nz = g.nz;
    k.u0 = (C)u0; k.rho0 = (C)rho0;
    k.scale = scale; k.inv_scale = inv_scale;
    k.c = cast_coef<C>(cd);
    return k;
}

// Face mask of a cell: bit 0/1 = low/high x face, 2/3 = y, 4/5 = z.
__device__ __forceinline__ unsigned face_mask(int i, int j, int k, int nx, int ny, int nz) {
    return (unsigned)(i == 0) | ((unsigned)(i == nx - 1) << 1) | ((unsigned)(j == 0) << 2) |
           ((unsigned)(j == ny - 1) << 3) | ((unsigned)(k == 0) << 4) |
           ((unsigned)(k == nz - 1) << 5);
}
// does direction (dx,dy,dz) leave the domain from a cell with face mask m
__host__ __device__ constexpr unsigned leave_bits(int dx, int dy, int dz) {
    return (dx < 0 ? 1u : 0u) | (dx > 0 ? 2u : 0u) | (dy < 0 ? 4u : 0u) | (dy > 0 ? 8u : 0u) |
           (dz < 0 ? 16u : 0u) | (dz > 0 ? 32u : 0u);
}

// Uniform bits for the stochastic rounding of 16-bit stores: one integer
// hash (lowbias32 finaliser) of (cell, step) per cell, then the high bits of
// its product with a distinct odd constant per population.
__device__ __forceinline__ unsigned sr_hash(unsigned x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ unsigned sr_cell(unsigned cell, unsigned step) {
    return sr_hash(cell * 0x9E3779B1u ^ sr_hash(step + 0x632BE5ABu));
}
__device__ __forceinline__ unsigned sr_pop(unsigned h, int q) {
    return h * (0x2545F491u + 2u * 0x9E3779B9u * (unsigned)q);
}
// Random bits of population pair p (populations 2p and 2p+1, rounded by one
// cvt.rs): the cell hash times a distinct odd constant per pair, plus its
// high half so that the low 16 bits depend on every bit of the hash.
__device__ __forceinline__ unsigned sr_pair(unsigned h, unsigned hh, int p) {
    return h * (0x2545F491u + 2u * 0x9E3779B9u * (unsigned)p) + hh;
}
constexpr int NPAIR19 = (Q19 + 1) / 2;

// Stochastically rounded 16-bit words of f[19], two populations per
// conversion (population 2p in the high half of w[p], 2p+1 in the low half).
template <typename S, typename C>
__device__ __forceinline__ void sr_pack19(const C (&f)[Q19], unsigned cell, unsigned seed,
                                          unsigned (&w)[NPAIR19]) {
    const unsigned h0 = sr_cell(cell, seed), hh = h0 >> 16;
#pragma unroll
    for (int p = 0; p < NPAIR19; p++)
        w[p] = St<S>::pack_sr(f[2 * p], 2 * p + 1 < Q19 ? f[2 * p + 1] : C(0), sr_pair(h0, hh, p));
}
__device__ __forceinline__ unsigned short sr_half(const unsigned (&w)[NPAIR19], int q) {
    return (unsigned short)((q & 1) ? (w[q >> 1] & 0xFFFFu) : (w[q >> 1] >> 16));
}

// ------------------------------------------------------------ lid kernel --
// IDX: 32-bit element indices when Q*cells < 2^31, 64-bit otherwise.
// lid_cell_from: collide and push one cell whose 19 stored populations are
// already in registers (raw); lid_cell: load them, then the same.  SR: the
// 16-bit stores round stochastically (a compile-time choice, so the
// round-to-nearest kernels carry none of its code).
//
// In-place (AA) pattern, one population buffer: an even step reads the
// cell's own slots and writes each post-collision population q into the
// cell's own slot opp(q) (SWAP_STORE); an odd step reads population q from
// slot opp(q) of the upstream cell x - e_q (or, when that cell is outside,
// from the cell's own slot q, which the even step filled with the reflected
// value) and writes like the push kernel, into slot q of x + e_q or, at a
// wall, into the cell's own slot opp(q).  Every slot is read and then written
// by one thread only, so a step needs no second buffer.  Wall reflections
// and the lid term are applied when a population is written, with that
// step's rho, exactly as in the push kernel: the arithmetic, and so every
// bit of the result, is the push kernel's.  After an odd step the buffer
// holds the post-stream populations (the push layout); after an even step a
// pairwise swap (k_aa_swap) restores that layout.
template <typename S, bool FIRST, typename IDX, bool SR = false, bool SWAP_STORE = false>
__device__ __forceinline__ void lid_cell_from(int i, int j, int k, const S (&raw)[Q19],
                                              S* __restrict__ fout,
                                              const StepK<typename St<S>::C>& K, IDX P,
                                              const double* __restrict__ mrho,
                                              const double* __restrict__ mu,
                                              const double* __restrict__ mv,
                                              const double* __restrict__ mw, unsigned seed) {
    using C = typename St<S>::C;
    const int nx = K.nx, ny = K.ny, nz = K.nz;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    // f, rho_m and the momenta in units of the storage scale sc (1 unless
    // SCALED); rho and u are unscaled, rhos = sc * rho
    const C sc = St<S>::SCALED ? (C)K.scale : C(1);
    C f[Q19];
#pragma unroll
    for (int q = 0; q < Q19; q++) f[q] = St<S>::cvt_s(raw[q]);
    C rho_m, rho, ux, uy, uz;
    if (FIRST) {
        rho = (C)mrho[cell];
        ux = (C)mu[cell];
        uy = (C)mv[cell];
        uz = (C)mw[cell];
        rho_m = St<S>::SHIFT ? (rho - K.rho0) * sc : rho;
    } else {
        C jx, jy, jz;
        moments0(f, rho_m, jx, jy, jz);
        rho = St<S>::SHIFT ? K.rho0 + (St<S>::SCALED ? rho_m * (C)K.inv_scale : rho_m) : rho_m;
        const C inv = St<S>::SCALED ? recip(rho) * (C)K.inv_scale : recip(rho);
        ux = jx * inv;
        uy = jy * inv;
        uz = jz * inv;
    }
    const C rhos = St<S>::SCALED ? rho * sc : rho;
    // The pair form rounds the equilibrium itself (error ~ eps |feq|, where
    // the moment form rounds only m - meq), and that rounding leaks into the
    // conserved density and momentum step after step.  In FP64 the leak is
    // ~1e-15 relative and in the 16-bit forms far below the storage error,
    // but FP32 storage keeps 1e-7 of the FP64 result only with the moment
    // form (64^3, Re = 400, 2000 steps: velocity 4e-6 with the pair form).
    // The first step after initial or load takes rho and u from the macro
    // arrays, so the pair form adds back what its relaxation would take from
    // the conserved sums of f (zero when the arrays agree with f).
    if (std::is_same<S, float>::value) {
        mrt_collide<C, false, true>(f, rho_m, rhos, ux, uy, uz, C(0), C(0), C(0), K.c, sc);
    } else if (FIRST) {
        C rf, jx, jy, jz;
        moments0(f, rf, jx, jy, jz);
        trt_collide_lid<C, true>(f, rho_m, rhos, ux, uy, uz, K.c, sc, rf - rho_m,
                                 jx - rhos * ux, jy - rhos * uy, jz - rhos * uz);
    } else {
        trt_collide_lid<C>(f, rho_m, rhos, ux, uy, uz, K.c, sc);
    }
    // moving lid: f(14) = f_post(11) - rho/6*U0, f(13) = f_post(12) + rho/6*U0
    // (bounce_back.f90:77-78).  On the top layer populations 11 and 12 always
    // leave through the lid (the lid face is written last, so it wins on
    // edges); the term is applied to them before the stores.
    if (k == nz - 1) {
        const C lid = rhos / C(6) * K.u0;
        f[11] = f[11] - lid;
        f[12] = f[12] + lid;
    }
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
    unsigned w[NPAIR19];
    if constexpr (SR) sr_pack19<S>(f, (unsigned)cell, seed, w);
    auto put = [&](IDX idx, int q) {
        if (oob(idx, (IDX)Q19 * P)) return;
        if constexpr (SR) St<S>::st_bits(fout + idx, sr_half(w, q));
        else St<S>::st_s(fout + idx, f[q]);
    };
    if (SWAP_STORE) {  // in-place even step: own cell, slot opp(q)
#pragma unroll
        for (int q = 0; q < Q19; q++) put((IDX)opp19(q) * P + cell, q);
        return;
    }
    if (bm == 0) {  // interior cell: every population streams
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
            put((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz, q);
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(dx, dy, dz)) == 0)
            put((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz, q);
        else
            put((IDX)opp19(q) * P + cell, q);
    }
}

template <typename S, typename IDX>
__device__ __forceinline__ void lid_load(int i, int j, int k, const S* __restrict__ fin, int nx,
                                         int ny, IDX P, S (&raw)[Q19]) {
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const IDX idx = (IDX)q * P + cell;
        raw[q] = oob(idx, (IDX)Q19 * P) ? S() : St<S>::raw(fin + idx);
    }
}

// in-place pattern loads (plain loads: the buffer is written by the same kernel).
// ODD: population q from slot opp(q) of the upstream cell, or from the cell's
// own slot q where the upstream cell is outside the domain.
template <typename S, typename IDX, bool ODD>
__device__ __forceinline__ void lid_load_aa(int i, int j, int k, const S* f, int nx, int ny,
                                            int nz, IDX P, S (&raw)[Q19]) {
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    auto ldaa = [&](IDX idx) -> S { return oob(idx, (IDX)Q19 * P) ? S() : St<S>::raw_rw(f + idx); };
    if (!ODD) {
#pragma unroll
        for (int q = 0; q < Q19; q++) raw[q] = ldaa((IDX)q * P + cell);
        return;
    }
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
    if (bm == 0) {  // interior cell: every upstream cell is inside
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
            raw[q] = ldaa((IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) -
                                        (IDX)dz * sz);
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(-dx, -dy, -dz)) != 0)
            raw[q] = ldaa((IDX)q * P + cell);
        else
            raw[q] = ldaa((IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) -
                                        (IDX)dz * sz);
    }
}

template <typename S, bool FIRST, typename IDX, bool SR = false>
__device__ __forceinline__ void lid_cell(int i, int j, int k, const S* __restrict__ fin,
                                         S* __restrict__ fout, const StepK<typename St<S>::C>& K,
                                         IDX P, const double* __restrict__ mrho,
                                         const double* __restrict__ mu,
                                         const double* __restrict__ mv,
                                         const double* __restrict__ mw, unsigned seed) {
    S raw[Q19];  // every load is issued before the first conversion
    lid_load<S, IDX>(i, j, k, fin, K.nx, K.ny, P, raw);
    lid_cell_from<S, FIRST, IDX, SR>(i, j, k, raw, fout, K, P, mrho, mu, mv, mw, seed);
}

// ------------------------------------------------------ lid kernel, FX64 --
// FP64 storage, Q55 fixed-point collision (fixed64.cuh); the same streaming,
// halfway bounce-back and lid term as lid_cell.
struct FxK {
    int nx, ny, nz;
    FxCoef c;
};
// populations converted on the FP64 unit (the rest with integer bit
// operations), balancing that unit against the integer pipe
#ifndef FX_CVT_IN
#define FX_CVT_IN 17
#endif
#ifndef FX_CVT_OUT
#define FX_CVT_OUT 17
#endif

// AAM: 0 push (fin -> fout), 1 in-place even step, 2 in-place odd step (fin ==
// fout; plain loads; see lid_cell_from for the pattern)
template <bool FIRST, typename IDX, int AAM = 0>
__device__ __forceinline__ void lid_cell_fx(int i, int j, int k, const double* fin,
                                            double* fout, const FxK& K, IDX P,
                                            const double* __restrict__ mrho,
                                            const double* __restrict__ mu,
                                            const double* __restrict__ mv,
                                            const double* __restrict__ mw) {
    const int nx = K.nx, ny = K.ny, nz = K.nz;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    long long f[Q19];
    {
        // all loads issued before any conversion
        double raw[Q19];
        if (AAM == 0) {
#pragma unroll
            for (int q = 0; q < Q19; q++) raw[q] = oob((IDX)q * P + cell, (IDX)Q19 * P) ? 0.0 : __ldg(fin + ((IDX)q * P + cell));
        } else {
            lid_load_aa<double, IDX, AAM == 2>(i, j, k, fin, nx, ny, nz, P, raw);
        }
#pragma unroll
        for (int q = 0; q < Q19; q++) f[q] = __double_as_longlong(raw[q]);
    }
    bool bad = false;
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        bad |= fx_bad(__longlong_as_double(f[q]));
        f[q] = q < FX_CVT_IN ? d2q_cvt(__longlong_as_double(f[q])) : d2q(__longlong_as_double(f[q]));
    }
    long long rin = 0, uin = 0, vin = 0, win = 0;
    if (FIRST) {
        const double r = mrho[cell], a = mu[cell], b = mv[cell], c = mw[cell];
        bad |= ((unsigned)(__double_as_longlong(r) >> 52) & 0x7FFu) >= 1024u;  // rho >= 2
        bad |= fx_bad(a) || fx_bad(b) || fx_bad(c);
        rin = d2q(r);
        uin = d2q(a);
        vin = d2q(b);
        win = d2q(c);
    }
    long long rho;
    bad |= !mrt_collide_fx<FIRST>(f, rin, uin, vin, win, K.c, rho);
    // moving lid: f(14) = f_post(11) - rho/6*U0, f(13) = f_post(12) + rho/6*U0
    // (bounce_back.f90:77-78); on the top layer populations 11 and 12 always
    // leave through the lid, so the term is applied to them before rounding
    if (k == nz - 1) {
        const long long lid = qmulc(rho, K.c.u0_6);
        f[11] -= lid;
        f[12] += lid;
    }
    // one rounding per population; the store pattern below moves doubles only
    double o[Q19];
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
    for (int q = 0; q < Q19; q++) o[q] = bad ? nan : (q < FX_CVT_OUT ? q2d_cvt(f[q]) : q2d(f[q]));
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
    if (AAM == 1) {  // in-place even step: own cell, slot opp(q) (lid term already in o)
#pragma unroll
        for (int q = 0; q < Q19; q++) st_chk(fout, (IDX)opp19(q) * P + cell, (IDX)Q19 * P, o[q]);
        return;
    }
    if (bm == 0) {
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
            st_chk(fout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q19 * P, o[q]);
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(dx, dy, dz)) == 0)
            st_chk(fout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q19 * P, o[q]);
        else
            st_chk(fout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q19 * P, o[q]);
    }
}

// -------------------------------------------------------- thermal kernel --
// Temperature populations are kept in the arithmetic type (FP64, or FP32 for
// the reduced forms): g_0 ~ 0.7 T has a 16-bit ulp (~2e-4) far above the
// per-step diffusive increments, so 16-bit g would stagnate.
// thermal_cell_from: collide and push one cell whose populations and carried
// force are already loaded (f converted to the arithmetic type, g, fp =
// F_x, F_y, F_z of the previous step; load_carried); SWAP_STORE: the in-place
// even step (own cell, slot opp(q), reflected and anti-bounce-back values
// formed as the push kernel forms them).  thermal_cell: load, then the same.
// The carried force is loaded with the populations, not where it is used: a
// load left inside the cell body has been issued only after the population
// loads were consumed in some builds (a second memory round trip per cell,
// halving the 16-bit forms' speed).
template <typename C, bool ROT, typename IDX>
__device__ __forceinline__ void load_carried(const C* F, IDX P, IDX cell, IDX fz_off,
                                             C (&fp)[3]) {
    fp[0] = fp[1] = C(0);
    if (ROT) {
        fp[0] = oob(P + cell, (IDX)3 * P) ? C(0) : F[cell];
        fp[1] = oob(P + cell, (IDX)3 * P) ? C(0) : F[P + cell];
    }
    fp[2] = oob(fz_off + cell, fz_off + P) ? C(0) : F[fz_off + cell];
}

template <typename S, bool FIRST, bool ROT, typename IDX, bool SR = false, bool SWAP_STORE = false>
__device__ __forceinline__ void thermal_cell_from(
    int i, int j, int k, typename St<S>::C (&f)[Q19], typename St<S>::C (&g)[Q7],
    const typename St<S>::C (&fp)[3], S* __restrict__ fout, typename St<S>::C* __restrict__ gout,
    typename St<S>::C* __restrict__ F, const StepK<typename St<S>::C>& K, IDX P,
    const double* __restrict__ mrho, const double* __restrict__ mu, const double* __restrict__ mv,
    const double* __restrict__ mw, const double* __restrict__ mT, IDX fz_off, unsigned seed) {
    // F holds F_x, F_y at planes 0 and 1 (rotation only) and F_z at element offset fz_off
    using C = typename St<S>::C;
    const int nx = K.nx, ny = K.ny, nz = K.nz;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    // f (as loaded by the caller), rho_m and the momenta in units of the
    // storage scale sc (1 unless SCALED); rho, u, T and the carried force are
    // unscaled
    const C sc = St<S>::SCALED ? (C)K.scale : C(1);
    C rho_m, rho, ux, uy, uz, temp;
    const C fxp = fp[0], fyp = fp[1], fzp = fp[2];  // carried from the previous step
    if (FIRST) {
        rho = (C)mrho[cell];
        ux = (C)mu[cell];
        uy = (C)mv[cell];
        uz = (C)mw[cell];
        temp = (C)mT[cell];
        rho_m = St<S>::SHIFT ? (rho - K.rho0) * sc : rho;
    } else {
        C jx, jy, jz;
        moments0(f, rho_m, jx, jy, jz);
        if (St<S>::SCALED) {
            jx = jx * (C)K.inv_scale;
            jy = jy * (C)K.inv_scale;
            jz = jz * (C)K.inv_scale;
        }
        rho = St<S>::SHIFT ? K.rho0 + (St<S>::SCALED ? rho_m * (C)K.inv_scale : rho_m) : rho_m;
        const C inv = recip(rho);
        // u^n = (sum f e + F^n/2)/rho^n with the force carried from the previous step
        ux = (jx + C(0.5) * fxp) * inv;
        uy = (jy + C(0.5) * fyp) * inv;
        uz = (jz + C(0.5) * fzp) * inv;
        temp = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + g[6]);
    }
    // body force from (rho,u,T) of the previous macro (bouyancy3d_mpi.F90:743-745)
    C fx = C(0), fy = C(0);
    if (ROT) {
        fx = C(-2) * rho * uy * K.omega_rot;
        fy = C(2) * rho * ux * K.omega_rot;
        if (!oob(P + cell, (IDX)3 * P)) {
            F[cell] = fx;
            F[P + cell] = fy;
        }
    }
    const C fz = rho * K.gbeta * (temp - K.t_ref);
    if (!oob(fz_off + cell, fz_off + P)) F[fz_off + cell] = fz;
    // the pair form where its equilibrium rounding stays below the storage
    // error (FP64 and the 16-bit forms; see lid_cell_from)
    if (std::is_same<S, float>::value) {
        mrt_collide<C, true, false>(f, rho_m, rho, ux, uy, uz, fx, fy, fz, K.c);
    } else if (FIRST) {
        // rho, u from the macro arrays: the odd term is e.(2 (j - rho u) + F)/10
        // and the density projection goes back in (trt_collide_forced)
        C rf, jx, jy, jz;
        moments0(f, rf, jx, jy, jz);
        const C rhos = rho * sc;
        trt_collide_forced<C, ROT, true>(
            f, rho_m, rhos, ux, uy, uz, fx * sc, fy * sc, fz * sc,
            fx * sc + C(2) * (jx - rhos * ux), fy * sc + C(2) * (jy - rhos * uy),
            fz * sc + C(2) * (jz - rhos * uz), K.c, rf - rho_m);
    } else if (St<S>::SCALED) {
        trt_collide_forced<C, ROT>(f, rho_m, rho * sc, ux, uy, uz, fx * sc, fy * sc, fz * sc,
                                   (fx - fxp) * sc, (fy - fyp) * sc, (fz - fzp) * sc, K.c);
    } else {
        trt_collide_forced<C, ROT>(f, rho_m, rho, ux, uy, uz, fx, fy, fz, fx - fxp, fy - fyp,
                                   fz - fzp, K.c);
    }
    // D3Q7: the pair form in FP64; the FP32 temperature populations of the
    // reduced forms keep the moment form (its rounding does not leak into
    // the conserved sum of g; see lid_cell_from for the FP32 measurement)
    if (!std::is_same<C, double>::value) {
        mrt_collide_t<C>(g, temp, ux, uy, uz, K.para_a, K.qd, K.qnu);
    } else if (FIRST) {
        const C sg = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + g[6]);
        trt_collide_t<C, true>(g, temp, ux, uy, uz, K.para_a, K.qd, K.qnu, sg - temp);
    } else {
        trt_collide_t<C>(g, temp, ux, uy, uz, K.para_a, K.qd, K.qnu);
    }

    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
    unsigned w[NPAIR19];
    if constexpr (SR) sr_pack19<S>(f, (unsigned)cell, seed, w);
    auto put = [&](IDX idx, int q) {
        if (oob(idx, (IDX)Q19 * P)) return;
        if constexpr (SR) St<S>::st_bits(fout + idx, sr_half(w, q));
        else St<S>::st_s(fout + idx, f[q]);
    };
    if (SWAP_STORE) {  // in-place even step: own cell, slot opp(q)
#pragma unroll
        for (int q = 0; q < Q19; q++) put((IDX)opp19(q) * P + cell, q);
#pragma unroll
        for (int q = 0; q < Q7; q++) {
            const int dy = ey19(q), dz = ez19(q);
            C val = g[q];
            if ((bm & leave_bits(ex19(q), dy, dz)) != 0) {
                if (dy != 0 && K.bc_y) val = -val + (dy < 0 ? K.chot : K.ccold);
                if (dz != 0 && K.bc_z) val = -val + (dz < 0 ? K.chot : K.ccold);
            }
            st_chk(gout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q7 * P, val);
        }
        return;
    }
    if (bm == 0) {
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
            put((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz, q);
        }
#pragma unroll
        for (int q = 0; q < Q7; q++) {
            const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
            st_chk(gout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q7 * P, g[q]);
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(dx, dy, dz)) == 0)
            put((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz, q);
        else
            put((IDX)opp19(q) * P + cell, q);
    }
    // D3Q7: adiabatic walls reflect, constant-T walls anti-bounce-back
    // g_in = -g_out + (6+paraA)/21 * T_wall (bouyancy3d_mpi.F90:1101-1210)
#pragma unroll
    for (int q = 0; q < Q7; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(dx, dy, dz)) == 0) {
            st_chk(gout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q7 * P, g[q]);
        } else {
            C val = g[q];
            if (dy != 0 && K.bc_y) val = -val + (dy < 0 ? K.chot : K.ccold);
            if (dz != 0 && K.bc_z) val = -val + (dz < 0 ? K.chot : K.ccold);
            st_chk(gout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q7 * P, val);
        }
    }
}


template <typename S, bool FIRST, bool ROT, typename IDX, bool SR = false>
__device__ __forceinline__ void thermal_cell(
    int i, int j, int k, const S* __restrict__ fin, S* __restrict__ fout,
    const typename St<S>::C* __restrict__ gin, typename St<S>::C* __restrict__ gout,
    typename St<S>::C* __restrict__ F, const StepK<typename St<S>::C>& K, IDX P,
    const double* __restrict__ mrho, const double* __restrict__ mu, const double* __restrict__ mv,
    const double* __restrict__ mw, const double* __restrict__ mT, IDX fz_off, unsigned seed) {
    using C = typename St<S>::C;
    const IDX cell = (IDX)i + (IDX)K.nx * ((IDX)j + (IDX)K.ny * (IDX)k);
    // every load is issued before the first conversion (as in lid_cell):
    // left to itself the scheduler has interleaved them with the arithmetic
    // in some builds of the 16-bit forms, halving their speed
    S raw[Q19];
    C f[Q19], g[Q7], fp[3];
#pragma unroll
    for (int q = 0; q < Q19; q++)
        raw[q] = oob((IDX)q * P + cell, (IDX)Q19 * P) ? S() : St<S>::raw(fin + ((IDX)q * P + cell));
#pragma unroll
    for (int q = 0; q < Q7; q++)
        g[q] = oob((IDX)q * P + cell, (IDX)Q7 * P) ? C(0) : St<C>::raw(gin + ((IDX)q * P + cell));
    load_carried<C, ROT, IDX>(F, P, cell, fz_off, fp);
#pragma unroll
    for (int q = 0; q < Q19; q++) f[q] = St<S>::cvt_s(raw[q]);
    thermal_cell_from<S, FIRST, ROT, IDX, SR>(i, j, k, f, g, fp, fout, gout, F, K, P, mrho, mu,
                                              mv, mw, mT, fz_off, seed);
}

// in-place pattern loads of a heated-cavity cell (plain loads; ODD: from the
// upstream cells' opposite slots, or the own slot where upstream is outside)
template <typename S, typename IDX, bool ODD, bool ROT = false>
__device__ __forceinline__ void thermal_load_aa(int i, int j, int k, const S* f,
                                                const typename St<S>::C* g,
                                                const typename St<S>::C* F, IDX fz_off,
                                                const StepK<typename St<S>::C>& K, IDX P,
                                                typename St<S>::C (&fv)[Q19],
                                                typename St<S>::C (&gv)[Q7],
                                                typename St<S>::C (&fp)[3]) {
    const int nx = K.nx, ny = K.ny, nz = K.nz;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
    // an interior cell (bm == 0) reads every population from upstream
    auto src = [&](int q) -> IDX {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if (!ODD || (bm != 0 && (bm & leave_bits(-dx, -dy, -dz)) != 0)) return (IDX)q * P + cell;
        return (IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) - (IDX)dz * sz;
    };
    S raw[Q19];
#pragma unroll
    for (int q = 0; q < Q19; q++) raw[q] = oob(src(q), (IDX)Q19 * P) ? S() : St<S>::raw_rw(f + src(q));
    // g through L2 only (ld.global.cg, coherent): measured 1.3x faster for the
    // stochastically rounded 16-bit form, neutral for the others
#pragma unroll
    for (int q = 0; q < Q7; q++)
        gv[q] = oob(src(q), (IDX)Q7 * P) ? typename St<S>::C(0) : __ldcg(g + src(q));
    load_carried<typename St<S>::C, ROT, IDX>(F, P, cell, fz_off, fp);
#pragma unroll
    for (int q = 0; q < Q19; q++) fv[q] = St<S>::cvt_s(raw[q]);  // in units of the storage scale
}

// -------------------------------------------------- heated cavity, FX64 --
// FP64 storage (f, g and the carried force as in the FP64 form); forced
// D3Q19 and D3Q7 collisions in Q55 (fixed64.cuh); the streaming, bounce-back
// and anti-bounce-back of thermal_cell.
// temperature populations converted on the FP64 unit (the rest with integer
// bit operations)
#ifndef FXT_CVT_G
#define FXT_CVT_G 4
#endif
struct FxTK {
    int nx, ny, nz, bc_y, bc_z;
    FxThermalCoef t;
};

// AAM: 0 push, 1 in-place even step, 2 in-place odd step (as lid_cell_fx)
template <bool FIRST, bool ROT, typename IDX, int AAM = 0>
__device__ __forceinline__ void thermal_cell_fx(
    int i, int j, int k, const double* fin, double* fout, const double* gin, double* gout,
    double* __restrict__ F,
    const FxTK& K, IDX P, const double* __restrict__ mrho, const double* __restrict__ mu,
    const double* __restrict__ mv, const double* __restrict__ mw, const double* __restrict__ mT) {
    using ll = long long;
    const int nx = K.nx, ny = K.ny, nz = K.nz;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    ll f[Q19], g[Q7];
    bool bad = false;
    {
        double rf[Q19], rg[Q7];
        if (AAM == 0) {
#pragma unroll
            for (int q = 0; q < Q19; q++) rf[q] = oob((IDX)q * P + cell, (IDX)Q19 * P) ? 0.0 : __ldg(fin + ((IDX)q * P + cell));
#pragma unroll
            for (int q = 0; q < Q7; q++) rg[q] = oob((IDX)q * P + cell, (IDX)Q7 * P) ? 0.0 : __ldg(gin + ((IDX)q * P + cell));
        } else {
            const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
            const unsigned bm = face_mask(i, j, k, nx, ny, nz);
            auto src = [&](int q) -> IDX {
                const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
                if (AAM != 2 || (bm & leave_bits(-dx, -dy, -dz)) != 0) return (IDX)q * P + cell;
                return (IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) - (IDX)dz * sz;
            };
#pragma unroll
            for (int q = 0; q < Q19; q++) rf[q] = fin[src(q)];
#pragma unroll
            for (int q = 0; q < Q7; q++) rg[q] = oob(src(q), (IDX)Q7 * P) ? 0.0 : __ldcg(gin + src(q));
        }
#pragma unroll
        for (int q = 0; q < Q19; q++) {
            bad |= fx_bad(rf[q]);
            f[q] = q < FX_CVT_IN ? d2q_cvt(rf[q]) : d2q(rf[q]);
        }
#pragma unroll
        for (int q = 0; q < Q7; q++) {
            bad |= fx_bad2(rg[q]);
            g[q] = q < FXT_CVT_G ? d2q_cvt(rg[q]) : d2q(rg[q]);
        }
    }
    ll rho, ux, uy, uz, temp, rux, ruy, ruz;
    if (FIRST) {
        const double r = mrho[cell], a = mu[cell], b = mv[cell], c = mw[cell], t = mT[cell];
        bad |= ((unsigned)(__double_as_longlong(r) >> 52) & 0x7FFu) >= 1024u;
        bad |= fx_bad(a) || fx_bad(b) || fx_bad(c) || fx_bad2(t);
        rho = d2q(r); ux = d2q(a); uy = d2q(b); uz = d2q(c); temp = d2q(t);
        rux = qmul(rho, ux); ruy = qmul(rho, uy); ruz = qmul(rho, uz);
    } else {
        // u = (sum f e + F/2) / rho with the force carried from the previous step
        ll fxp = 0, fyp = 0;
        if (ROT) {
            fxp = d2q(oob(P + cell, (IDX)3 * P) ? 0.0 : F[cell]);
            fyp = d2q(oob(P + cell, (IDX)3 * P) ? 0.0 : F[P + cell]);
        }
        const ll fzp = d2q(oob((IDX)2 * P + cell, (IDX)3 * P) ? 0.0 : F[2 * P + cell]);
        const ll s1 = f[1] + f[2], s2 = f[3] + f[4], s3 = f[5] + f[6];
        const ll s4 = f[7] + f[10], s5 = f[9] + f[8], s6 = f[11] + f[14], s7 = f[13] + f[12];
        const ll s8 = f[15] + f[18], s9 = f[17] + f[16];
        rho = f[0] + (s1 + s2 + s3) + ((s4 + s5) + (s6 + s7) + (s8 + s9));
        const ll d4 = f[7] - f[10], d5 = f[9] - f[8], d6 = f[11] - f[14], d7 = f[13] - f[12];
        const ll d8 = f[15] - f[18], d9 = f[17] - f[16];
        rux = (f[1] - f[2]) + (d4 + d5) + (d6 + d7) + (fxp >> 1);
        ruy = (f[3] - f[4]) + (d4 - d5) + (d8 + d9) + (fyp >> 1);
        ruz = (f[5] - f[6]) + (d6 - d7) + (d8 - d9) + (fzp >> 1);
        const ll inv = fx_recip(rho);
        ux = qmul(rux, inv);
        uy = qmul(ruy, inv);
        uz = qmul(ruz, inv);
        temp = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + g[6]);
    }
    // body force from (rho, u, T) of the previous macro (bouyancy3d_mpi.F90:743-745)
    ll fx = 0, fy = 0;
    if (ROT) {
        fx = -qmul(qmul(rho, uy), K.t.omega2);
        fy = qmul(qmul(rho, ux), K.t.omega2);
        if (!oob(P + cell, (IDX)3 * P)) {
            F[cell] = q2d(fx);
            F[P + cell] = q2d(fy);
        }
    }
    const ll fz = qmul(rho, qmulc(temp - K.t.t_ref, K.t.gbeta));
    if (!oob((IDX)2 * P + cell, (IDX)3 * P)) F[2 * P + cell] = q2d(fz);
    bad |= !mrt_collide_fx_forced(f, rho, ux, uy, uz, rux, ruy, ruz, fx, fy, fz, K.t);
    mrt_collide_t_fx(g, temp, ux, uy, uz, K.t);

    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
#pragma unroll
    for (int q = 0; q < Q19; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        const double o = bad ? nan : (q < FX_CVT_OUT ? q2d_cvt(f[q]) : q2d(f[q]));
        if (AAM == 1)  // in-place even step: own cell, slot opp(q)
            st_chk(fout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q19 * P, o);
        else if ((bm & leave_bits(dx, dy, dz)) == 0)
            st_chk(fout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q19 * P, o);
        else
            st_chk(fout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q19 * P, o);
    }
    // D3Q7: adiabatic walls reflect, constant-T walls anti-bounce-back
#pragma unroll
    for (int q = 0; q < Q7; q++) {
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(dx, dy, dz)) == 0) {
            const double o = bad ? nan : (q < FXT_CVT_G ? q2d_cvt(g[q]) : q2d(g[q]));
            if (AAM == 1)
                st_chk(gout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q7 * P, o);
            else
                st_chk(gout, (IDX)((IDX)q * P + cell + (IDX)(dx + dy * (int)sy) + (IDX)dz * sz), (IDX)Q7 * P, o);
        } else {
            ll val = g[q];
            if (dy != 0 && K.bc_y) val = -val + (dy < 0 ? K.t.chot : K.t.ccold);
            if (dz != 0 && K.bc_z) val = -val + (dz < 0 ? K.t.chot : K.t.ccold);
            st_chk(gout, (IDX)((IDX)opp19(q) * P + cell), (IDX)Q7 * P, bad ? nan : (q < FXT_CVT_G ? q2d_cvt(val) : q2d(val)));
        }
    }
}

}  // namespace mglc
