// k_particle2d.cu -- D2Q9 moving circles, the reference's case4 step
// (MPI/Micro_particles/fortran/case4/mpi_particle, main.F90:35-73) and, as the
// P2_SHEAR variant, its case1 step (MPI/Micro_particles/fortran/case1/
// mpi_complete, main.F90:34-67: a circle carried through the shear between
// two moving walls, periodic in x, both compile-time frames and both
// interpolation orders).  The case4 routines are:
//
//   collision (fluid.F90:14-64, solid nodes skipped), streaming from fluid
//   sources (:97-108), four halfway-bounce-back walls (:115-161),
//   bounceback_particle (particle_bounceback.F90:15-97, calQ :101-141 or
//   calQ2 :144-185), macro (fluid.F90:164-184), calForce (particle_force.F90:
//   35-190), updateCenter and refill (particle_update.F90:26-193).
//
// Layout: populations as f(0:8, i, j) with two ghost layers each side, the
// reference's arrays (-1..nx+2 filled with omega*rho0; one more zero layer).
// Everything is FP64 and this file is compiled without FMA contraction, so
// each expression rounds as the reference's statement does.  Steps whose
// order matters in the reference keep its loop order: the density averages
// are exact parallel replays of the sequential sum (the k_gs_* kernels), each
// circle's link sums are evaluated by a warp and added in loop order, and the
// refill sweep refills its sorted node list on one thread; the rest is one
// thread per node.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "mglc.h"
#include "particles2d.cuh"

namespace mglc {

namespace {

__device__ __constant__ int c_ex[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
__device__ __constant__ int c_ey[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
__device__ __constant__ int c_r[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
__device__ __constant__ double c_w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                         1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

enum { S_NO_OWNER = 1, S_Q = 2, S_OVERLAP = 3, S_WALL = 4, S_NO_DIR = 5 };

struct D2 {
    P2Params p;
    int X;  // padded row length nx + 6
    double *f, *fp, *rho, *u, *v;
    int *ob, *on;
    double *xc, *uc, *om, *xco, *uco, *omo, *force, *torque;  // np x 3
    double* ravg;                                             // [0] current average
    int* status;                                              // [0] code, [1] particle
    // boundary links of the current mask, per (node, direction 1..8): the
    // circle that owns the solid end (-1: none) and calQ's q, x0, y0
    int* lc;
    double* lq;  // 3 doubles per link
    // per-chunk records of the ordered density sums (GsBuf)
    double *gs_part, *gs_pre;
    void* gs_map;  // GridSeg[nch]
    long long* gs_ub;
    int *gs_e, *gs_flag, *gs_cnt;
    int *rf_count, *rf_list;  // nodes to refill: count, list of RF_CAP
};

__device__ __forceinline__ int IX(const D2& d, int i, int j) { return (i + 2) + d.X * (j + 2); }
__device__ __forceinline__ double& F(const D2& d, int a, int i, int j) { return d.f[9 * IX(d, i, j) + a]; }
__device__ __forceinline__ double& FP(const D2& d, int a, int i, int j) { return d.fp[9 * IX(d, i, j) + a]; }
__device__ __forceinline__ double sq(double x) { return x * x; }

// ((x - xc)^2 + (y - yc)^2) <= R^2 (particle_bounceback.F90:50-52)
__device__ __forceinline__ bool inside(const D2& d, const double* cen, int c, double x, double y) {
    const double r = d.p.radius;
    return sq(x - cen[3 * c]) + sq(y - cen[3 * c + 1]) <= sq(r);
}

__device__ void fail(const D2& d, int code, int c) {
    if (atomicCAS(d.status, 0, code) == 0) d.status[1] = c;
}

// x index of a population read: case1 is periodic in x (its MPI exchange
// fills the ghost columns with the periodic partner's values); case4 reads
// its own ghost columns
__device__ __forceinline__ int wxi(const D2& d, int i) {
    if (d.p.variant != P2_SHEAR) return i;
    return i < 1 ? i + d.p.nx : (i > d.p.nx ? i - d.p.nx : i);
}

// ------------------------------------------------------------------ fluid --
__global__ void k2_collide(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0] || d.ob[IX(d, i, j)] != 0) return;
    double f[9], m[9], meq[9], s[9], mp[9];
    for (int a = 0; a < 9; a++) f[a] = F(d, a, i, j);
    const double rho = d.rho[IX(d, i, j)], u = d.u[IX(d, i, j)], v = d.v[IX(d, i, j)];
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
    if (d.p.variant == P2_SHEAR) {  // case1 fluid.F90:15-16 groups the sums
        m[1] = -4.0 * f[0] - f[1] - f[2] - f[3] - f[4] + 2.0 * (f[5] + f[6] + f[7] + f[8]);
        m[2] = 4.0 * f[0] - 2.0 * (f[1] + f[2] + f[3] + f[4]) + f[5] + f[6] + f[7] + f[8];
    } else {
        m[1] = -4.0 * f[0] - f[1] - f[2] - f[3] - f[4] + 2.0 * f[5] + 2.0 * f[6] + 2.0 * f[7] + 2.0 * f[8];
        m[2] = 4.0 * f[0] - 2.0 * f[1] - 2.0 * f[2] - 2.0 * f[3] - 2.0 * f[4] + f[5] + f[6] + f[7] + f[8];
    }
    m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
    m[4] = -2.0 * f[1] + 2.0 * f[3] + f[5] - f[6] - f[7] + f[8];
    m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    m[6] = -2.0 * f[2] + 2.0 * f[4] + f[5] + f[6] - f[7] - f[8];
    m[7] = f[1] - f[2] + f[3] - f[4];
    m[8] = f[5] - f[6] + f[7] - f[8];
    meq[0] = rho;
    meq[1] = rho * (-2.0 + 3.0 * (u * u + v * v));
    meq[2] = rho * (1.0 - 3.0 * (u * u + v * v));
    meq[3] = rho * u;
    meq[4] = -meq[3];
    meq[5] = rho * v;
    meq[6] = -meq[5];
    meq[7] = rho * (u * u - v * v);
    meq[8] = rho * (u * v);
    const double Snu = d.p.snu, Sq = d.p.sq;
    s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq; s[5] = 0.0; s[6] = Sq;
    s[7] = Snu; s[8] = Snu;
    for (int a = 0; a < 9; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]);
    FP(d, 0, i, j) = (mp[0] - mp[1] + mp[2]) / 9.0;
    FP(d, 1, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[3] / 6.0 - mp[4] / 6.0 + mp[7] * 0.25;
    FP(d, 2, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 + mp[5] / 6.0 - mp[6] / 6.0 - mp[7] * 0.25;
    FP(d, 3, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[3] / 6.0 + mp[4] / 6.0 + mp[7] * 0.25;
    FP(d, 4, i, j) = mp[0] / 9.0 - mp[1] / 36.0 - mp[2] / 18.0 - mp[5] / 6.0 + mp[6] / 6.0 - mp[7] * 0.25;
    FP(d, 5, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 + mp[5] / 6.0 +
                     mp[6] / 12.0 + mp[8] * 0.25;
    FP(d, 6, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 + mp[5] / 6.0 +
                     mp[6] / 12.0 - mp[8] * 0.25;
    FP(d, 7, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 - mp[3] / 6.0 - mp[4] / 12.0 - mp[5] / 6.0 -
                     mp[6] / 12.0 + mp[8] * 0.25;
    FP(d, 8, i, j) = mp[0] / 9.0 + mp[1] / 18.0 + mp[2] / 36.0 + mp[3] / 6.0 + mp[4] / 12.0 - mp[5] / 6.0 -
                     mp[6] / 12.0 - mp[8] * 0.25;
}

// pull from fluid sources only; every interior node (fluid or solid) receives
// (case1 wraps the source column, fluid.F90:105-110)
__global__ void k2_stream(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0]) return;
    for (int a = 0; a < 9; a++) {
        const int ip = wxi(d, i - c_ex[a]), jp = j - c_ey[a];
        if (d.ob[IX(d, ip, jp)] == 0) F(d, a, i, j) = FP(d, a, ip, jp);
    }
}

// the four walls; corner nodes receive the same value from both of their walls.
// case1: only the two moving walls (fluid.F90:127-169)
__global__ void k2_walls(D2 d) {
    const int t = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (d.status[0]) return;
    const int nx = d.p.nx, ny = d.p.ny;
    if (d.p.variant == P2_SHEAR) {
        if (t > nx) return;
        const double uw = d.p.uwall, u0 = d.p.u0;
        F(d, 2, t, 1) = FP(d, 4, t, 1);
        if (d.p.moving_frame) {
            F(d, 5, t, 1) = FP(d, 7, t, 1) + (-uw - u0) / 6.0;
            F(d, 6, t, 1) = FP(d, 8, t, 1) - (-uw - u0) / 6.0;
        } else {
            F(d, 5, t, 1) = FP(d, 7, t, 1) + (-uw) / 6.0;
            F(d, 6, t, 1) = FP(d, 8, t, 1) - (-uw) / 6.0;
        }
        F(d, 4, t, ny) = FP(d, 2, t, ny);
        if (d.p.moving_frame) {
            F(d, 7, t, ny) = FP(d, 5, t, ny) - (uw - u0) / 6.0;
            F(d, 8, t, ny) = FP(d, 6, t, ny) + (uw - u0) / 6.0;
        } else {
            F(d, 7, t, ny) = FP(d, 5, t, ny) - (uw) / 6.0;
            F(d, 8, t, ny) = FP(d, 6, t, ny) + (uw) / 6.0;
        }
        return;
    }
    if (t <= ny) {
        F(d, 1, 1, t) = FP(d, 3, 1, t);
        F(d, 5, 1, t) = FP(d, 7, 1, t);
        F(d, 8, 1, t) = FP(d, 6, 1, t);
        F(d, 3, nx, t) = FP(d, 1, nx, t);
        F(d, 6, nx, t) = FP(d, 8, nx, t);
        F(d, 7, nx, t) = FP(d, 5, nx, t);
    }
    if (t <= nx) {
        F(d, 2, t, 1) = FP(d, 4, t, 1);
        F(d, 5, t, 1) = FP(d, 7, t, 1);
        F(d, 6, t, 1) = FP(d, 8, t, 1);
        F(d, 4, t, ny) = FP(d, 2, t, ny);
        F(d, 7, t, ny) = FP(d, 5, t, ny);
        F(d, 8, t, ny) = FP(d, 6, t, ny);
    }
}

// Sequential FP64 sums computed in parallel, bit for bit.  While the running
// sum s stays inside one binade [2^E, 2^(E+1)) and the addends are finite and
// non-negative, s is an integer S times u = 2^(E-52) with S in [2^52, 2^53),
// and RN(s + x) = (S + k) u where k is x/u rounded to an integer: down below
// one half, up above it, and on an exact half to the k that makes S + k even
// (ties to even).  Only the tie case reads the running sum, and only its
// parity, so an addend is a map from the incoming parity to (increment,
// outgoing parity); maps compose associatively, and an ordered tree reduction
// of a chunk's maps gives the chunk's sum.  A chunk that may leave the binade
// (or holds a negative or non-finite addend) is added one element at a time.
struct GridSeg {
    long long i0, i1;  // increment in units of u for incoming parity 0 / 1
    int o0, o1;        // outgoing parity for incoming parity 0 / 1
};

__device__ __forceinline__ GridSeg seg_identity() { return GridSeg{0, 0, 0, 1}; }

// a followed by b
__device__ __forceinline__ GridSeg seg_cat(const GridSeg& a, const GridSeg& b) {
    GridSeg r;
    r.i0 = a.i0 + (a.o0 ? b.i1 : b.i0);
    r.o0 = a.o0 ? b.o1 : b.o0;
    r.i1 = a.i1 + (a.o1 ? b.i1 : b.i0);
    r.o1 = a.o1 ? b.o1 : b.o0;
    return r;
}

__device__ __forceinline__ GridSeg seg_shfl_down(const GridSeg& g, int off) {
    GridSeg r;
    r.i0 = __shfl_down_sync(0xffffffffu, g.i0, off);
    r.i1 = __shfl_down_sync(0xffffffffu, g.i1, off);
    r.o0 = __shfl_down_sync(0xffffffffu, g.o0, off);
    r.o1 = __shfl_down_sync(0xffffffffu, g.o1, off);
    return r;
}

// ordered reduction over a warp: lane 0 ends with lane 0's map, then lane 1's, ...
__device__ __forceinline__ GridSeg seg_warp_reduce(GridSeg g) {
    for (int off = 1; off < 32; off <<= 1) {
        const GridSeg o = seg_shfl_down(g, off);
        if ((threadIdx.x & 31) + off < 32 && ((threadIdx.x & 31) & (2 * off - 1)) == 0)
            g = seg_cat(g, o);
    }
    return g;
}

constexpr long long MANT52 = (1LL << 52) - 1;
constexpr int NO_BINADE = 100000;

// the map of addend x (bits xb) on the grid of binade e (u = 2^(e-52)), from
// the bit pattern with integer operations only; false when x must be added the
// plain way (sign bit set, infinite or NaN, or x >= 2^(e+1)).  ub is an upper
// bound of the increment.
__device__ __forceinline__ bool seg_of(long long xb, int e, GridSeg& g, long long& ub) {
    if (xb < 0) return false;
    const int ex = (int)(xb >> 52);
    if (ex == 2047) return false;
    const long long M = (xb & MANT52) | (ex ? (1LL << 52) : 0);  // x = M 2^(max(ex,1)-1075)
    const int sh = max(ex, 1) - 1023 - e;                         // x / u = M 2^sh
    if (sh > 0) return false;
    long long m;
    int cls = 0;  // fraction of x / u: 0 below one half, 1 above, 2 exactly one half
    if (sh == 0) {
        m = M;
    } else if (sh >= -62) {
        const int k = -sh;
        m = M >> k;
        const long long rem = M & ((1LL << k) - 1), half = 1LL << (k - 1);
        cls = rem > half ? 1 : (rem == half ? 2 : 0);
    } else {
        m = 0;  // x < u / 2
    }
    if (cls == 2) {
        g.i0 = m + (m & 1);
        g.i1 = m + ((m + 1) & 1);
        g.o0 = g.o1 = 0;
        ub = m + 1;
    } else {
        const long long v = m + cls;
        g.i0 = g.i1 = v;
        g.o0 = (int)(v & 1);
        g.o1 = (int)((v + 1) & 1);
        ub = v;
    }
    return true;
}

// binade of a positive normal running sum, NO_BINADE when the grid path is off
__device__ __forceinline__ int binade_of(double acc) {
    const long long b = __double_as_longlong(acc);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    return (acc > 0.0 && e >= -900 && e <= 1000) ? e : NO_BINADE;
}

// acc + (the addends whose composed map is h and increment bound hb) on binade
// e; false when the sum may leave the binade
__device__ __forceinline__ bool grid_apply(double& acc, int e, const GridSeg& h, long long hb) {
    const long long S = (__double_as_longlong(acc) & MANT52) | (1LL << 52);
    if (!(hb < (1LL << 53) - S)) return false;
    const long long S1 = S + ((S & 1) ? h.i1 : h.i0);
    acc = __longlong_as_double(((long long)(e + 1023) << 52) | (S1 & MANT52));
    return true;
}

__device__ __forceinline__ long long warp_incl_scan(long long x) {
    const int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    return x;
}

__device__ __forceinline__ GridSeg seg_select(bool keep, const GridSeg& g) {
    return keep ? g : seg_identity();
}

// Warp 0 adds the addends [lo, hi) of sr (where sm is set) to acc (held by
// lane 0) in order, 32 at a time: the lanes up to the first addend that cannot
// take the grid path of the current binade (it is not finite and non-negative,
// or the sum may leave the binade) are added as one map, that addend the plain
// way, and the rest start over on the new binade.
__device__ void warp_sum_pieces(const double* sr, const unsigned char* sm, int lo, int hi,
                                double& acc) {
    const int lane = threadIdx.x & 31;
    for (int p = lo; p < hi; p += 32) {
        int lstart = 0;
        while (lstart < 32) {
            const double a0 = __shfl_sync(0xffffffffu, acc, 0);
            const int ep = binade_of(a0);
            const long long S = ep == NO_BINADE ? 0 : (__double_as_longlong(a0) & MANT52) | (1LL << 52);
            const int q = p + lane;
            const bool valid = lane >= lstart && q < hi && sm[q];
            GridSeg g = seg_identity();
            long long ub = 0;
            bool bad = false;
            if (valid) bad = ep == NO_BINADE || !seg_of(__double_as_longlong(sr[q]), ep, g, ub);
            const long long incl = warp_incl_scan(ub);
            const bool ok = !bad && (ep == NO_BINADE || incl < (1LL << 53) - S);
            const unsigned nb = __ballot_sync(0xffffffffu, !ok);
            const int lstar = nb ? __ffs(nb) - 1 : 32;
            const GridSeg h = seg_warp_reduce(seg_select(lane < lstar, g));
            const long long hb = __shfl_sync(0xffffffffu, incl, lstar > 0 ? lstar - 1 : 0);
            if (lane == 0) {
                if (ep != NO_BINADE && lstar > 0) grid_apply(acc, ep, h, hb);
                if (lstar < 32) acc = acc + sr[p + lstar];
            }
            lstart = lstar + 1;
        }
    }
}

// The sequential sum x_0 + x_1 + ... over the addends t = 0..total-1 that a
// fetch functor keeps (fetch(t, keep, x)), with the rounding of that order,
// in chunks of CH addends (EPT consecutive addends per thread of an SB-thread
// block):
//   k_gs_part  (one block per chunk) plain partial sums (any order) and counts;
//   k_gs_scan  (one block) their exclusive prefix: an estimate of the running
//              sum where each chunk starts, hence of its binade;
//   k_gs_map   (one block per chunk) the chunk's composed grid map on that
//              binade, with its increment bound;
//   k_gs_apply (one block) walks the chunks in order: a chunk whose binade
//              estimate is the exact running sum's binade, whose addends all
//              took the grid path and whose bound keeps the sum in the binade
//              is added as its map; any other chunk is added by chunk_split.
// chunk_split adds one chunk with the whole block: the warps up to the first
// one holding an addend that cannot take the grid path of the current binade
// are added as one map, that warp's addends by warp 0 (warp_sum_pieces), and
// the rest start over on the new binade.
constexpr int SB = 1024;  // threads of the ordered sweeps (one block)
constexpr int EPT = 4;    // addends per thread and chunk
constexpr int CH = SB * EPT;
constexpr long long UB_CAP = 1LL << 61;  // saturation of chunk increment bounds

struct SumShared {
    double sr[CH];
    unsigned char sm[CH];  // 1 = kept
    GridSeg wseg[SB / 32];
    long long wub[SB / 32];
    int wbad[SB / 32];
    double acc;  // the running sum
    int next;
};

// per-chunk records of the pipeline (nch entries each)
struct GsBuf {
    double *part, *pre;
    GridSeg* map;
    long long* ub;
    int *e, *flag, *cnt;  // flag: 0 map valid, 1 plain path needed, 2 no kept addend
};

// adds the chunk at base (this thread's addends fc/xc) to sh.acc; all threads
// call it; it ends with a barrier
__device__ void chunk_split(int base, int total, const bool (&fc)[EPT], const double (&xc)[EPT],
                            SumShared& sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int u = 0; u < EPT; u++) {
        sh.sm[threadIdx.x * EPT + u] = fc[u];
        sh.sr[threadIdx.x * EPT + u] = xc[u];
    }
    int startw = 0;
    for (;;) {
        const int e = binade_of(sh.acc);
        GridSeg g = seg_identity();
        long long ub = 0;  // at most 128 bounds below 2^53 per warp: no overflow
        bool bad = false;
        if (w >= startw) {
#pragma unroll
            for (int u = 0; u < EPT; u++) {
                if (!fc[u] || bad) continue;
                GridSeg gu;
                long long bu;
                if (e != NO_BINADE && seg_of(__double_as_longlong(xc[u]), e, gu, bu)) {
                    g = seg_cat(g, gu);
                    ub += bu;
                } else {
                    bad = true;
                }
            }
        }
        g = seg_warp_reduce(g);
        for (int off = 16; off > 0; off >>= 1) ub += __shfl_down_sync(0xffffffffu, ub, off);
        const int wb = __any_sync(0xffffffffu, bad);
        if (lane == 0) {
            sh.wseg[w] = g;
            sh.wub[w] = ub;
            sh.wbad[w] = wb;
        }
        __syncthreads();
        if (w == 0) {
            double acc = sh.acc;
            const long long S = e == NO_BINADE ? 0 : (__double_as_longlong(acc) & MANT52) | (1LL << 52);
            // the prefix grows by at most 2^60 a lane, so it cannot wrap before
            // the first lane past the bound, and only lanes before that are used
            const long long incl = warp_incl_scan(sh.wub[lane]);
            const bool ok = lane < startw ||
                            (!sh.wbad[lane] && e != NO_BINADE && incl < (1LL << 53) - S);
            const unsigned nb = __ballot_sync(0xffffffffu, !ok);
            const int wstar = nb ? __ffs(nb) - 1 : 32;
            const GridSeg h = seg_warp_reduce(seg_select(lane < wstar, sh.wseg[lane]));
            const long long hb = __shfl_sync(0xffffffffu, incl, wstar > 0 ? wstar - 1 : 0);
            if (lane == 0 && e != NO_BINADE && wstar > startw) grid_apply(acc, e, h, hb);
            if (wstar < 32) {
                const int lo = wstar * 32 * EPT;
                warp_sum_pieces(sh.sr, sh.sm, lo, min(lo + 32 * EPT, total - base), acc);
            }
            if (lane == 0) {
                sh.acc = acc;
                sh.next = wstar >= 31 ? 32 : wstar + 1;
            }
        }
        __syncthreads();
        startw = sh.next;
        if (startw >= 32) break;
    }
}

template <class Fetch>
__global__ void __launch_bounds__(SB) k_gs_part(Fetch fetch, int total, GsBuf b) {
    __shared__ double ws[SB / 32];
    __shared__ int wc[SB / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c = blockIdx.x;
    double v = 0.0;
    int n = 0;
#pragma unroll
    for (int u = 0; u < EPT; u++) {
        bool fl;
        double x;
        fetch(c * CH + threadIdx.x * EPT + u, fl, x);
        if (fl) {
            v += x;
            n++;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, off);
        n += __shfl_down_sync(0xffffffffu, n, off);
    }
    if (lane == 0) {
        ws[w] = v;
        wc[w] = n;
    }
    __syncthreads();
    if (w == 0) {
        v = ws[lane];
        n = wc[lane];
        for (int off = 16; off > 0; off >>= 1) {
            v += __shfl_down_sync(0xffffffffu, v, off);
            n += __shfl_down_sync(0xffffffffu, n, off);
        }
        if (lane == 0) {
            b.part[c] = v;
            b.cnt[c] = n;
        }
    }
}

__global__ void __launch_bounds__(SB) k_gs_scan(GsBuf b, int nch) {
    __shared__ double ws[SB / 32];
    __shared__ double carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    for (int base = 0; base < nch; base += SB) {
        const int c = base + threadIdx.x;
        const double own = c < nch ? b.part[c] : 0.0;
        double v = own;
        for (int off = 1; off < 32; off <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= off) v += y;
        }
        if (lane == 31) ws[w] = v;
        __syncthreads();
        if (w == 0) {
            double t = ws[lane];
            for (int off = 1; off < 32; off <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, t, off);
                if (lane >= off) t += y;
            }
            ws[lane] = t;
        }
        __syncthreads();
        const double incl = v + (w > 0 ? ws[w - 1] : 0.0) + carry;
        if (c < nch) b.pre[c] = incl - own;  // an estimate: any rounding will do
        __syncthreads();
        if (threadIdx.x == SB - 1) carry = incl;
        __syncthreads();
    }
}

template <class Fetch>
__global__ void __launch_bounds__(SB) k_gs_map(Fetch fetch, int total, GsBuf b) {
    __shared__ GridSeg wseg[SB / 32];
    __shared__ long long wub[SB / 32];
    __shared__ int wbad[SB / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c = blockIdx.x;
    const int e = binade_of(b.pre[c]);
    GridSeg g = seg_identity();
    long long ub = 0;
    bool bad = e == NO_BINADE;
#pragma unroll
    for (int u = 0; u < EPT; u++) {
        bool fl;
        double x;
        fetch(c * CH + threadIdx.x * EPT + u, fl, x);
        if (!fl || bad) continue;
        GridSeg gu;
        long long bu;
        if (seg_of(__double_as_longlong(x), e, gu, bu)) {
            g = seg_cat(g, gu);
            ub += bu;
        } else {
            bad = true;
        }
    }
    g = seg_warp_reduce(g);
    for (int off = 16; off > 0; off >>= 1) ub += __shfl_down_sync(0xffffffffu, ub, off);
    const int wb = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        wseg[w] = g;
        wub[w] = ub;
        wbad[w] = wb;
    }
    __syncthreads();
    if (w == 0) {
        const GridSeg h = seg_warp_reduce(wseg[lane]);
        long long hb = min(wub[lane], UB_CAP);
        for (int off = 16; off > 0; off >>= 1)
            hb = min(hb + __shfl_down_sync(0xffffffffu, hb, off), UB_CAP);  // both <= 2^61
        const int hbad = __any_sync(0xffffffffu, wbad[lane]);
        if (lane == 0) {
            b.map[c] = h;
            b.ub[c] = hb;
            b.e[c] = e;
            b.flag[c] = b.cnt[c] == 0 ? 2 : (hbad ? 1 : 0);
        }
    }
}

// the ordered walk; out[0] = the sum and out[1] = the count, or out[0] =
// sum / count when average is set; nothing when status[0] is set
template <class Fetch>
__global__ void __launch_bounds__(SB) k_gs_apply(Fetch fetch, int total, int nch, GsBuf b,
                                                 double* out, bool average, const int* status) {
    if (status && status[0]) return;
    __shared__ SumShared sh;
    __shared__ long long wn[SB / 32];
    __shared__ int s_fail;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long n = 0;
    for (int c = threadIdx.x; c < nch; c += SB) n += b.cnt[c];
    for (int off = 16; off > 0; off >>= 1) n += __shfl_down_sync(0xffffffffu, n, off);
    if (lane == 0) wn[w] = n;
    if (threadIdx.x == 0) sh.acc = 0.0;
    __syncthreads();
    int next = 0;
    for (;;) {
        if (w == 0) {
            double acc = sh.acc;  // every lane walks the same sums
            int fail = nch;
            for (int cb = next; cb < nch && fail == nch; cb += 32) {
                const int c = cb + lane;
                GridSeg g = seg_identity();
                long long ub = 0;
                int e = NO_BINADE, flag = 1;
                if (c < nch) {
                    g = b.map[c];
                    ub = b.ub[c];
                    e = b.e[c];
                    flag = b.flag[c];
                }
                const int lim = min(32, nch - cb);
                for (int l = 0; l < lim; l++) {
                    const GridSeg gl{__shfl_sync(0xffffffffu, g.i0, l), __shfl_sync(0xffffffffu, g.i1, l),
                                     __shfl_sync(0xffffffffu, g.o0, l), __shfl_sync(0xffffffffu, g.o1, l)};
                    const long long ubl = __shfl_sync(0xffffffffu, ub, l);
                    const int el = __shfl_sync(0xffffffffu, e, l);
                    const int fl = __shfl_sync(0xffffffffu, flag, l);
                    if (fl == 2) continue;  // nothing kept
                    const int ea = binade_of(acc);
                    if (fl != 0 || ea == NO_BINADE || el != ea || !grid_apply(acc, ea, gl, ubl)) {
                        fail = cb + l;
                        break;
                    }
                }
            }
            if (lane == 0) {
                sh.acc = acc;
                s_fail = fail;
            }
        }
        __syncthreads();
        const int fc = s_fail;
        if (fc >= nch) break;
        bool f4[EPT];
        double x4[EPT];
#pragma unroll
        for (int u = 0; u < EPT; u++) fetch(fc * CH + threadIdx.x * EPT + u, f4[u], x4[u]);
        chunk_split(fc * CH, total, f4, x4, sh);
        next = fc + 1;
    }
    if (threadIdx.x == 0) {
        long long cnt = 0;
        for (int q = 0; q < SB / 32; q++) cnt += wn[q];
        if (average) {
            out[0] = sh.acc / (double)cnt;
        } else {
            out[0] = sh.acc;
            out[1] = (double)cnt;
        }
    }
}

// the fluid densities of a 2-D mask in the reference's loop order (j outer)
struct RhoFetch {
    D2 d;
    const int* mask;
    int total;
    __device__ void operator()(int t, bool& fl, double& x) const {
        fl = false;
        x = 0.0;
        if (t < total) {
            const int nx = d.p.nx, j = 1 + t / nx, i = 1 + t % nx;
            fl = mask[IX(d, i, j)] == 0;
            x = d.rho[IX(d, i, j)];
        }
    }
};

struct ArrayFetch {
    const double* x;
    const int* keep;
    int total;
    __device__ void operator()(int t, bool& fl, double& v) const {
        fl = t < total && keep[t] != 0;
        v = t < total ? x[t] : 0.0;
    }
};

GsBuf gs_of(const D2& d) {
    return GsBuf{d.gs_part, d.gs_pre, (GridSeg*)d.gs_map, d.gs_ub, d.gs_e, d.gs_flag, d.gs_cnt};
}

int gs_chunks(long long total) { return (int)((total + CH - 1) / CH) > 0 ? (int)((total + CH - 1) / CH) : 1; }

template <class Fetch>
void gs_launch(const Fetch& f, int total, const GsBuf& b, double* out, bool average,
               const int* status, cudaStream_t s) {
    const int nch = gs_chunks(total);
    k_gs_part<<<nch, SB, 0, s>>>(f, total, b);
    k_gs_scan<<<1, SB, 0, s>>>(b, nch);
    k_gs_map<<<nch, SB, 0, s>>>(f, total, b);
    k_gs_apply<<<1, SB, 0, s>>>(f, total, nch, b, out, average, status);
}

// calQ / calQ2 from node (x, y) along direction a towards circle c
__device__ bool calq(const D2& d, int c, double x, double y, int a, double& x0, double& y0,
                     double& q) {
    const double xc = d.xc[3 * c], yc = d.xc[3 * c + 1], R = d.p.radius;
    if (!d.p.q_bisection) {
        const double ea = c_ex[a], eb = c_ey[a], ec = 0.0;
        const double ca = ea * ea + eb * eb + ec * ec;
        const double cb = 2.0 * (ea * (x - xc) + eb * (y - yc) + 0.0);
        const double cc = (x - xc) * (x - xc) + (y - yc) * (y - yc) + 0.0 - R * R;
        const double delta = cb * cb - 4.0 * ca * cc;
        if (delta < 0) return false;
        q = (-cb - sqrt(delta)) / (2.0 * ca);
        x0 = x + q * ea;
        y0 = y + q * eb;
    } else {
        const double epsR = (double)1e-9f;  // default-real literal 1e-9 (:106)
        double qq = 0.5, qt = 0.5;
        double px = x + qt * (double)c_ex[a], py = y + qt * (double)c_ey[a];
        auto dist = [&]() { return sqrt((px - xc) * (px - xc) + (py - yc) * (py - yc) + 0.0); };
        int guard = 0;
        while (fabs(dist() - R) >= epsR) {
            if (++guard > 200) return false;
            if (dist() > R) {
                qt = qt / 2.0;
                px = px + qt * (double)c_ex[a];
                py = py + qt * (double)c_ey[a];
                qq = qq + qt;
            } else if (dist() < R) {
                qt = qt / 2.0;
                px = px - qt * (double)c_ex[a];
                py = py - qt * (double)c_ey[a];
                qq = qq - qt;
            } else {
                return false;
            }
        }
        q = qq;
        x0 = px;
        y0 = py;
    }
    return !(q > 1.0 || q < 0.0);
}

// quadratic interpolated bounce-back (particle_bounceback.F90:37-97)
__global__ void k2_ibb(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0] || d.ob[IX(d, i, j)] != 0) return;
    const double ravg = d.ravg[0];
    for (int a = 1; a < 9; a++) {
        const int ip = i + c_ex[a], jp = j + c_ey[a];
        if (d.ob[IX(d, ip, jp)] != 1) continue;
        bool found = false;
        for (int c = 0; c < d.p.np; c++) {
            if (!inside(d, d.xc, c, (double)ip, (double)jp)) continue;
            found = true;
            double x0, y0, q;
            if (!calq(d, c, (double)i, (double)j, a, x0, y0, q)) {
                fail(d, S_Q, c);
                return;
            }
            const double Om = d.om[3 * c + 2];
            const double rot0 = -(y0 - d.xc[3 * c + 1]) * Om, rot1 = (x0 - d.xc[3 * c]) * Om;
            const int ra = c_r[a];
            const double eu = c_ex[ra] * (d.uc[3 * c] + rot0) + c_ey[ra] * (d.uc[3 * c + 1] + rot1);
            const int ex = c_ex[a], ey = c_ey[a];
            const int i1 = wxi(d, i - ex), i2 = wxi(d, i - 2 * ex);
            if (d.p.linear) {  // case1 particle_bounceback.F90:66-76
                if (q < 0.5) {
                    F(d, ra, i, j) = 2.0 * q * FP(d, a, i, j) + (1.0 - 2.0 * q) * FP(d, a, i1, j - ey) +
                                     6.0 * c_w[a] * ravg * eu;
                } else {
                    F(d, ra, i, j) = 0.5 / q * FP(d, a, i, j) + (1.0 - 0.50 / q) * FP(d, ra, i, j) +
                                     3.0 * c_w[a] * ravg / q * eu;
                }
            } else if (q < 0.5) {
                F(d, ra, i, j) = q * (1.0 + 2.0 * q) * FP(d, a, i, j) +
                                 (1.0 - 4.0 * q * q) * FP(d, a, i1, j - ey) -
                                 q * (1.0 - 2.0 * q) * FP(d, a, i2, j - 2 * ey) +
                                 6.0 * c_w[a] * ravg * eu;
            } else {
                F(d, ra, i, j) = FP(d, a, i, j) / q / (1.0 + 2.0 * q) +
                                 FP(d, ra, i, j) * (2.0 * q - 1.0) / q -
                                 FP(d, ra, i1, j - ey) * (2.0 * q - 1.0) / (2.0 * q + 1.0) +
                                 6.0 * c_w[a] * ravg / q / (1.0 + 2.0 * q) * eu;
            }
        }
        if (!found) {
            fail(d, S_NO_OWNER, -1);
            return;
        }
    }
}

__global__ void k2_macro(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0] || d.ob[IX(d, i, j)] != 0) return;
    double g[9];
    for (int a = 0; a < 9; a++) g[a] = F(d, a, i, j);
    const double r = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8];
    d.rho[IX(d, i, j)] = r;
    d.u[IX(d, i, j)] = (g[1] - g[3] + g[5] - g[6] - g[7] + g[8]) / r;
    d.v[IX(d, i, j)] = (g[2] - g[4] + g[5] + g[6] - g[7] - g[8]) / r;
}

// calForce (particle_force.F90:35-190): one thread per circle; its links are
// visited in the reference's global loop order restricted to its box
// calQ of every boundary link of the current mask, one thread per fluid node,
// for the force sums below (which visit a circle's links one at a time in the
// reference's loop order); the values are calq's, so the sums are unchanged
__global__ void k2_links(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0] || d.ob[IX(d, i, j)] != 0) return;
    for (int a = 1; a < 9; a++) {
        const int ip = i + c_ex[a], jp = j + c_ey[a];
        if (d.ob[IX(d, ip, jp)] != 1) continue;
        const size_t li = (size_t)IX(d, i, j) * 8 + (a - 1);
        int owner = -1;
        for (int c = 0; c < d.p.np && owner < 0; c++)
            if (inside(d, d.xc, c, (double)ip, (double)jp)) owner = c;
        d.lc[li] = owner;
        if (owner < 0) continue;
        double x0, y0, q;
        if (!calq(d, owner, (double)i, (double)j, a, x0, y0, q)) {
            fail(d, S_Q, owner);
            return;
        }
        d.lq[3 * li] = x0;
        d.lq[3 * li + 1] = y0;
        d.lq[3 * li + 2] = q;
    }
}

// one warp per circle: the lanes evaluate 32 consecutive candidate links (j
// outer, i, direction inner: the reference's loop order) at a time, and every
// lane then adds the valid ones in that order, so the sums are the sequential ones
__global__ void k2_force(D2 d) {
    const int c = blockIdx.x, lane = threadIdx.x;
    if (c >= d.p.np || d.status[0]) return;
    const P2Params& p = d.p;
    const double PI = p.pi, R0 = p.radius, ravg = d.ravg[0];
    const double xcc = d.xc[3 * c], ycc = d.xc[3 * c + 1];
    const int i0 = max(1, (int)floor(xcc - R0) - 2), i1 = min(p.nx, (int)ceil(xcc + R0) + 2);
    const int j0 = max(1, (int)floor(ycc - R0) - 2), j1 = min(p.ny, (int)ceil(ycc + R0) + 2);
    const int ni = max(0, i1 - i0 + 1), nj = max(0, j1 - j0 + 1);
    const long long ncand = (long long)ni * nj * 8;
    const double Om = d.om[3 * c + 2], U0 = d.uc[3 * c], U1 = d.uc[3 * c + 1];
    double fs0 = 0.0, fs1 = 0.0, ts = 0.0;
    for (long long base = 0; base < ncand; base += 32) {
        const long long k = base + lane;
        bool ok = false, bad = false;
        double Fx = 0.0, Fy = 0.0, T = 0.0;
        if (k < ncand) {
            const int a = 1 + (int)(k % 8);
            const int i = i0 + (int)((k / 8) % ni), j = j0 + (int)(k / 8 / ni);
            const int ip = i + c_ex[a], jp = j + c_ey[a];
            if (d.ob[IX(d, i, j)] == 0 && d.ob[IX(d, ip, jp)] == 1 &&
                inside(d, d.xc, c, (double)ip, (double)jp)) {
                double x0, y0, q;
                const size_t li = (size_t)IX(d, i, j) * 8 + (a - 1);
                if (d.lc[li] == c) {  // from k2_links
                    x0 = d.lq[3 * li];
                    y0 = d.lq[3 * li + 1];
                    q = d.lq[3 * li + 2];
                    ok = true;
                } else {
                    ok = calq(d, c, (double)i, (double)j, a, x0, y0, q);
                    bad = !ok;
                }
                (void)q;
                if (ok) {
                    const double rot0 = -(y0 - ycc) * Om, rot1 = (x0 - xcc) * Om;
                    const int ra = c_r[a];
                    Fx = (c_ex[a] - U0 - rot0) * FP(d, a, i, j) - (c_ex[ra] - U0 - rot0) * F(d, ra, i, j);
                    Fy = (c_ey[a] - U1 - rot1) * FP(d, a, i, j) - (c_ey[ra] - U1 - rot1) * F(d, ra, i, j);
                    const double rx = x0 - xcc, ry = y0 - ycc;
                    T = rx * Fy - ry * Fx;
                }
            }
        }
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) fail(d, S_Q, c);
            return;
        }
        for (unsigned v = __ballot_sync(0xffffffffu, ok); v; v &= v - 1) {
            const int l = __ffs(v) - 1;
            fs0 = fs0 + __shfl_sync(0xffffffffu, Fx, l);
            fs1 = fs1 + __shfl_sync(0xffffffffu, Fy, l);
            ts = ts + __shfl_sync(0xffffffffu, T, l);
        }
    }
    if (lane != 0) return;
    if (p.variant == P2_SHEAR) {  // case1 particle_force.F90:86-92: momentum exchange only
        d.force[3 * c] = fs0;
        d.force[3 * c + 1] = fs1;
        d.force[3 * c + 2] = 0.0;
        d.torque[3 * c] = 0.0;
        d.torque[3 * c + 1] = 0.0;
        d.torque[3 * c + 2] = ts;
        return;
    }
    const double gmag = fabs(-p.gravity);
    double fij[3] = {0.0, 0.0, 0.0}, fw[3] = {0.0, 0.0, 0.0};
    const double Rc = R0;
    // particle-particle springs (:100-125)
    const double scale_p = PI * (Rc * Rc) * (p.rho_solid - ravg) * gmag / p.stiff_particle;
    for (int c2 = 0; c2 < p.np; c2++) {
        if (c2 == c) continue;
        const double d0 = d.xc[3 * c] - d.xc[3 * c2];
        const double d1 = d.xc[3 * c + 1] - d.xc[3 * c2 + 1];
        const double d2 = 0.0;
        const double dij = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        const double R2 = R0, thr = p.threshold_particle;
        if (dij >= Rc + R2 + thr) {
        } else if (dij < Rc + R2 + thr && dij >= Rc + R2) {
            const double t = (dij - Rc - R2 - thr) / thr;
            fij[0] = fij[0] + scale_p * (t * t) * d0 / dij;
            fij[1] = fij[1] + scale_p * (t * t) * d1 / dij;
            fij[2] = fij[2] + scale_p * (t * t) * d2 / dij;
        } else {
            fail(d, S_OVERLAP, c);
            return;
        }
    }
    // particle-wall springs (:128-178): left, right, bottom (no top spring)
    const double scale_w = PI * (Rc * Rc) * (p.rho_solid - p.rho0) * gmag / p.stiff_wall;
    const double thw = p.threshold_wall;
    for (int ax = 0; ax < 2; ax++) {
        const int n_ax = ax == 0 ? p.nx : p.ny;
        const bool high = ax == 0;
        const double cpos = d.xc[3 * c + ax];
        double dw = cpos - Rc - 1.0;
        if (dw < 0) { fail(d, S_WALL, c); return; }
        if (dw < thw) fw[ax] = fw[ax] + scale_w * ((dw - thw) / thw) * ((dw - thw) / thw);
        if (high) {
            dw = (double)n_ax - cpos - Rc;
            if (dw < 0) { fail(d, S_WALL, c); return; }
            if (dw < thw) fw[ax] = fw[ax] - scale_w * ((dw - thw) / thw) * ((dw - thw) / thw);
        }
    }
    // totals (:184-190)
    d.force[3 * c] = fs0 + fij[0] + fw[0];
    d.force[3 * c + 1] = fs1 - (p.rho_solid - ravg) * PI * (R0 * R0) * gmag + fij[1] + fw[1];
    d.force[3 * c + 2] = 0.0;
    d.torque[3 * c] = 0.0;
    d.torque[3 * c + 1] = 0.0;
    d.torque[3 * c + 2] = ts;
}

// updateCenter (particle_update.F90:26-50): U += F/M, Omega += T/I, x += U_old + a/2
__global__ void k2_move(D2 d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.p.np || d.status[0]) return;
    const P2Params& p = d.p;
    for (int q = 0; q < 3; q++) {
        d.xco[3 * c + q] = d.xc[3 * c + q];
        d.uco[3 * c + q] = d.uc[3 * c + q];
        d.omo[3 * c + q] = d.om[3 * c + q];
    }
    if (p.variant == P2_SHEAR) {  // case1 particle_update.F90:21-35: prescribed motion
        d.uc[3 * c] = p.moving_frame ? 0.0 : p.u0;
        d.uc[3 * c + 1] = 0.0;
        d.om[3 * c + 2] = 0.0;
        d.xc[3 * c] = d.xco[3 * c] + d.uco[3 * c];
        d.xc[3 * c + 1] = d.xco[3 * c + 1] + d.uco[3 * c + 1];
        return;
    }
    const double PI = p.pi, R0 = p.radius, r = p.radius;
    const double ax = d.force[3 * c] / PI / (R0 * R0) / p.rho_solid;
    const double ay = d.force[3 * c + 1] / PI / (R0 * R0) / p.rho_solid;
    const double aom = d.torque[3 * c + 2] / (0.5 * p.rho_solid * PI * (r * r * r * r));
    d.uc[3 * c] = d.uco[3 * c] + ax;
    d.uc[3 * c + 1] = d.uco[3 * c + 1] + ay;
    d.om[3 * c + 2] = d.omo[3 * c + 2] + aom;
    d.xc[3 * c] = d.xco[3 * c] + d.uco[3 * c] + 0.5 * ax;
    d.xc[3 * c + 1] = d.xco[3 * c + 1] + d.uco[3 * c + 1] + 0.5 * ay;
}

// obst from the centres over 0..nx+1 x 0..ny+1 (particle_update.F90:80-93);
// interior solid nodes get rho_s and u = 0 (:94-102)
__global__ void k2_mask(D2 d, int* mask, bool set_macro) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > d.p.nx + 1 || d.status[0]) return;
    int o = 0;
    for (int c = 0; c < d.p.np; c++)
        if (inside(d, d.xc, c, (double)i, (double)j)) o = 1;
    mask[IX(d, i, j)] = o;
    if (set_macro && o == 1 && i >= 1 && i <= d.p.nx && j >= 1 && j <= d.p.ny) {
        d.rho[IX(d, i, j)] = d.p.rho_solid;
        d.u[IX(d, i, j)] = 0.0;
        d.v[IX(d, i, j)] = 0.0;
    }
}

// refill of nodes that left a circle (particle_update.F90:122-193) for one
// node; false when it failed (status set)
__device__ bool refill_node(const D2& d, int i, int j, double ra) {
    const P2Params& p = d.p;
    bool found = false;
    for (int c = 0; c < p.np; c++) {
        if (!inside(d, d.xco, c, (double)i, (double)j)) continue;
        found = true;
        const double xc = d.xc[3 * c], yc = d.xc[3 * c + 1];
        double out = 0.0;
        int ec = 0;
        for (int a = 1; a < 9; a++) {
            const double t = ((i - xc) * c_ex[a] + (j - yc) * c_ey[a]) /
                             sqrt((i - xc) * (i - xc) + (j - yc) * (j - yc));
            if (t > out) {
                out = t;
                ec = a;
            }
        }
        if (ec == 0) {
            fail(d, S_NO_DIR, c);
            return false;
        }
        const int e0 = c_ex[ec], e1 = c_ey[ec];
        const int i1 = wxi(d, i + e0), i2 = wxi(d, i + 2 * e0), i3 = wxi(d, i + 3 * e0);
        for (int a = 0; a < 9; a++) {
            if (p.linear)  // case1 particle_update.F90:115-119
                F(d, a, i, j) = 2.0 * F(d, a, i1, j + e1) - F(d, a, i2, j + 2 * e1);
            else
                F(d, a, i, j) = 3.0 * F(d, a, i1, j + e1) - 3.0 * F(d, a, i2, j + 2 * e1) +
                                F(d, a, i3, j + 3 * e1);
        }
        double G[9], m[9];
        for (int a = 0; a < 9; a++) G[a] = F(d, a, i, j);
        m[0] = G[0] + G[1] + G[2] + G[3] + G[4] + G[5] + G[6] + G[7] + G[8];
        m[1] = -4.0 * G[0] - G[1] - G[2] - G[3] - G[4] + 2.0 * G[5] + 2.0 * G[6] + 2.0 * G[7] + 2.0 * G[8];
        m[2] = 4.0 * G[0] - 2.0 * G[1] - 2.0 * G[2] - 2.0 * G[3] - 2.0 * G[4] + G[5] + G[6] + G[7] + G[8];
        if (p.variant == P2_SHEAR) {  // case1 :130,132: the first circle's (Uc, Vc)
            m[3] = ra * d.uc[0];
            m[5] = ra * d.uc[1];
        } else {
            m[3] = ra * (d.uc[3 * c] - (j - yc) * d.om[3 * c + 2]);
            m[5] = ra * (d.uc[3 * c + 1] + (i - xc) * d.om[3 * c + 2]);
        }
        m[4] = -2.0 * G[1] + 2.0 * G[3] + G[5] - G[6] - G[7] + G[8];
        m[6] = -2.0 * G[2] + 2.0 * G[4] + G[5] + G[6] - G[7] - G[8];
        m[7] = G[1] - G[2] + G[3] - G[4];
        m[8] = G[5] - G[6] + G[7] - G[8];
        G[0] = (m[0] - m[1] + m[2]) / 9.0;
        G[1] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[3] / 6.0 - m[4] / 6.0 + m[7] * 0.25;
        G[2] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 + m[5] / 6.0 - m[6] / 6.0 - m[7] * 0.25;
        G[3] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[3] / 6.0 + m[4] / 6.0 + m[7] * 0.25;
        G[4] = m[0] / 9.0 - m[1] / 36.0 - m[2] / 18.0 - m[5] / 6.0 + m[6] / 6.0 - m[7] * 0.25;
        G[5] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 + m[5] / 6.0 +
               m[6] / 12.0 + m[8] * 0.25;
        G[6] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 + m[5] / 6.0 +
               m[6] / 12.0 - m[8] * 0.25;
        G[7] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 - m[3] / 6.0 - m[4] / 12.0 - m[5] / 6.0 -
               m[6] / 12.0 + m[8] * 0.25;
        G[8] = m[0] / 9.0 + m[1] / 18.0 + m[2] / 36.0 + m[3] / 6.0 + m[4] / 12.0 - m[5] / 6.0 -
               m[6] / 12.0 - m[8] * 0.25;
        for (int a = 0; a < 9; a++) F(d, a, i, j) = G[a];
        const double r = G[0] + G[1] + G[2] + G[3] + G[4] + G[5] + G[6] + G[7] + G[8];
        d.rho[IX(d, i, j)] = r;
        d.u[IX(d, i, j)] = (G[1] - G[3] + G[5] - G[6] - G[7] + G[8]) / r;
        d.v[IX(d, i, j)] = (G[2] - G[4] + G[5] + G[6] - G[7] - G[8]) / r;
    }
    if (!found) {
        fail(d, S_NO_OWNER, -1);
        return false;
    }
    return true;
}

// The refill sweep in the reference's order: each refill may read an earlier
// one, so one thread refills.  The nodes to refill (left a circle: solid
// before, fluid now) are listed by k2_refill_find in any order; k2_refill sorts
// the list by node index and refills in that order.  A list longer than
// RF_CAP is replaced by refill_scan, which finds the nodes chunk by chunk with
// an ordered block compaction.
constexpr int RF_CAP = 4096;

__global__ void k2_refill_find(D2 d) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx || d.status[0]) return;
    if (d.ob[IX(d, i, j)] == 1 && d.on[IX(d, i, j)] == 0) {
        const int pos = atomicAdd(d.rf_count, 1);
        if (pos < RF_CAP) d.rf_list[pos] = (j - 1) * d.p.nx + (i - 1);
    }
}

__device__ void refill_scan(const D2& d) {
    __shared__ int list[SB];
    __shared__ int wcount[SB / 32];
    __shared__ int nlist, stop;
    const int nx = d.p.nx;
    const long long total = (long long)nx * d.p.ny;
    const double ra = d.ravg[0];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) stop = 0;
    auto left = [&](long long t) {  // solid before, fluid now
        if (t >= total) return false;
        const int j = 1 + (int)(t / nx), i = 1 + (int)(t % nx);
        return d.ob[IX(d, i, j)] == 1 && d.on[IX(d, i, j)] == 0;
    };
    // chunks of EPT sub-chunks of SB nodes; flags of the next chunk are read ahead
    bool fnext[EPT];
#pragma unroll
    for (int u = 0; u < EPT; u++) fnext[u] = left((long long)u * SB + threadIdx.x);
    for (long long cbase = 0; cbase < total; cbase += CH) {
        bool fcur[EPT];
        bool any = false;
#pragma unroll
        for (int u = 0; u < EPT; u++) {
            fcur[u] = fnext[u];
            any = any || fcur[u];
            fnext[u] = left(cbase + CH + (long long)u * SB + threadIdx.x);
        }
        if (!__syncthreads_or(any)) continue;  // most chunks have none
        for (int u = 0; u < EPT; u++) {
            const long long t = cbase + (long long)u * SB + threadIdx.x;
            const bool flag = fcur[u];
            if (!__syncthreads_or(flag)) continue;
            const unsigned bal = __ballot_sync(0xffffffffu, flag);
            if (lane == 0) wcount[w] = __popc(bal);
            __syncthreads();
            if (threadIdx.x == 0) {
                int acc = 0;
                for (int q = 0; q < SB / 32; q++) {
                    const int c = wcount[q];
                    wcount[q] = acc;
                    acc += c;
                }
                nlist = acc;
            }
            __syncthreads();
            if (flag) list[wcount[w] + __popc(bal & ((1u << lane) - 1u))] = (int)t;
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int q = 0; q < nlist; q++) {
                    const int node = list[q];
                    if (!refill_node(d, 1 + node % nx, 1 + node / nx, ra)) {
                        stop = 1;
                        break;
                    }
                }
            }
            __syncthreads();
            if (stop) return;
        }
    }
}

__global__ void __launch_bounds__(SB) k2_refill(D2 d) {
    if (d.status[0]) return;
    const int cnt = d.rf_count[0];
    if (cnt > RF_CAP) {
        refill_scan(d);
        return;
    }
    __shared__ int keys[RF_CAP];
    int n2 = 1;
    while (n2 < cnt) n2 <<= 1;
    for (int q = threadIdx.x; q < n2; q += SB) keys[q] = q < cnt ? d.rf_list[q] : 0x7fffffff;
    __syncthreads();
    for (int k = 2; k <= n2; k <<= 1)  // bitonic sort, ascending
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int q = threadIdx.x; q < n2; q += SB) {
                const int r = q ^ jj;
                if (r > q) {
                    const int a = keys[q], b = keys[r];
                    if ((a > b) == ((q & k) == 0)) {
                        keys[q] = b;
                        keys[r] = a;
                    }
                }
            }
            __syncthreads();
        }
    if (threadIdx.x == 0) {
        const int nx = d.p.nx;
        const double ra = d.ravg[0];
        for (int q = 0; q < cnt; q++)
            if (!refill_node(d, 1 + keys[q] % nx, 1 + keys[q] / nx, ra)) return;
    }
}

// initial.F90:103-188 with the centres given by the caller: mask, rho = rho_s
// (solid) or rho0, u = 0, f = omega on fluid nodes, ghosts omega*rho0
__global__ void k2_init_fields(D2 d) {
    const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x), j = -2 + (int)blockIdx.y;
    if (i > d.p.nx + 3) return;
    const int nx = d.p.nx, ny = d.p.ny;
    const bool interior = i >= 1 && i <= nx && j >= 1 && j <= ny;
    const bool ghost = !interior && i >= -1 && i <= nx + 2 && j >= -1 && j <= ny + 2;
    if (interior) {
        const bool solid = d.ob[IX(d, i, j)] == 1;
        d.rho[IX(d, i, j)] = solid ? d.p.rho_solid : d.p.rho0;
        double uu = 0.0;
        if (d.p.variant == P2_SHEAR) {  // case1 initial.F90:96-127
            const bool mf = d.p.moving_frame;
            uu = mf ? 0.0 : d.p.u0;
            if (j == 1) uu = mf ? -d.p.uwall - d.p.u0 : -d.p.uwall;
            if (j == ny) uu = mf ? d.p.uwall - d.p.u0 : d.p.uwall;
        }
        d.u[IX(d, i, j)] = uu;
        d.v[IX(d, i, j)] = 0.0;
        if (!solid) {
            const double vv = 0.0, us2 = uu * uu + vv * vv;
            for (int a = 0; a < 9; a++) {
                const double un = uu * c_ex[a] + vv * c_ey[a];
                F(d, a, i, j) = c_w[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
            }
        }
    } else if (ghost && d.p.variant != P2_SHEAR) {  // case1 ghosts stay 0 (initial.F90:140)
        for (int a = 0; a < 9; a++) {
            F(d, a, i, j) = c_w[a] * d.p.rho0;
            FP(d, a, i, j) = c_w[a] * d.p.rho0;
        }
    }
}

// owner index of every interior node (-1 fluid)
__global__ void k2_owner(D2 d, int* out) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > d.p.nx) return;
    int o = -1;
    if (d.ob[IX(d, i, j)] == 1)
        for (int c = 0; c < d.p.np && o < 0; c++)
            if (inside(d, d.xc, c, (double)i, (double)j)) o = c;
    out[(i - 1) + d.p.nx * (j - 1)] = o;
}

}  // namespace

struct P2Ctx {
    D2 d{};
    cudaStream_t s = nullptr;
    bool own_stream = false;
    std::vector<double> centers;  // np x 3
    long long itc = 0;
    long long bytes = 0;
    int* owner_tmp = nullptr;
};

namespace {

int ck(cudaError_t e, const char* what, std::string& err) {
    if (e == cudaSuccess) return MGLC_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return MGLC_ERR_CUDA;
}

template <typename T>
int dal(P2Ctx* c, T** p, size_t n, std::string& err) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        err = std::string("device allocation: ") + cudaGetErrorString(e);
        return MGLC_ERR_NOMEM;
    }
    c->bytes += (long long)(n * sizeof(T));
    return cudaMemsetAsync(*p, 0, n * sizeof(T), c->s) == cudaSuccess ? MGLC_OK : MGLC_ERR_CUDA;
}

dim3 rows_grid(const D2& d) { return dim3((d.p.nx + 127) / 128, d.p.ny); }

}  // namespace

int p2d_create(const P2Params& p, const double* centers_xy, P2Ctx** out, std::string& err) {
    P2Ctx* c = new P2Ctx();
    *out = c;
    c->d.p = p;
    c->d.X = p.nx + 6;
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
        err = "stream creation failed";
        return MGLC_ERR_CUDA;
    }
    c->own_stream = true;
    const size_t cells = (size_t)(p.nx + 6) * (p.ny + 6), np3 = 3 * (size_t)(p.np > 0 ? p.np : 1);
    D2& d = c->d;
    int rc = 0;
    if ((rc = dal(c, &d.f, 9 * cells, err)) || (rc = dal(c, &d.fp, 9 * cells, err)) ||
        (rc = dal(c, &d.rho, cells, err)) || (rc = dal(c, &d.u, cells, err)) ||
        (rc = dal(c, &d.v, cells, err)) || (rc = dal(c, &d.ob, cells, err)) ||
        (rc = dal(c, &d.on, cells, err)))
        return rc;
    double** pa[] = {&d.xc, &d.uc, &d.om, &d.xco, &d.uco, &d.omo, &d.force, &d.torque};
    for (double** a : pa)
        if ((rc = dal(c, a, np3, err))) return rc;
    if ((rc = dal(c, &d.lc, 8 * cells, err)) || (rc = dal(c, &d.lq, 24 * cells, err))) return rc;
    const size_t nch = (size_t)gs_chunks((long long)p.nx * p.ny);
    GridSeg* gmap = nullptr;
    if ((rc = dal(c, &d.gs_part, nch, err)) || (rc = dal(c, &d.gs_pre, nch, err)) ||
        (rc = dal(c, &gmap, nch, err)) || (rc = dal(c, &d.gs_ub, nch, err)) ||
        (rc = dal(c, &d.gs_e, nch, err)) || (rc = dal(c, &d.gs_flag, nch, err)) ||
        (rc = dal(c, &d.gs_cnt, nch, err)))
        return rc;
    d.gs_map = gmap;
    if ((rc = dal(c, &d.rf_count, 1, err)) || (rc = dal(c, &d.rf_list, RF_CAP, err))) return rc;
    if ((rc = dal(c, &d.ravg, 2, err)) || (rc = dal(c, &d.status, 2, err)) ||
        (rc = dal(c, &c->owner_tmp, (size_t)p.nx * p.ny, err)))
        return rc;
    c->centers.assign(3 * (size_t)p.np, 0.0);
    for (int q = 0; q < p.np; q++) {
        c->centers[3 * q] = centers_xy[2 * q];
        c->centers[3 * q + 1] = centers_xy[2 * q + 1];
    }
    return ck(cudaStreamSynchronize(c->s), "create", err);
}

void p2d_destroy(P2Ctx* c) {
    if (!c) return;
    D2& d = c->d;
    void* ps[] = {d.f, d.fp, d.rho, d.u, d.v, d.ob, d.on, d.xc, d.uc, d.om, d.xco, d.uco, d.omo,
                  d.force, d.torque, d.ravg, d.status, d.lc, d.lq, c->owner_tmp,
                  d.gs_part, d.gs_pre, d.gs_map, d.gs_ub, d.gs_e, d.gs_flag, d.gs_cnt,
                  d.rf_count, d.rf_list};
    if (c->s) cudaStreamSynchronize(c->s);
    for (void* p : ps)
        if (p) cudaFree(p);
    if (c->own_stream && c->s) cudaStreamDestroy(c->s);
    delete c;
}

int p2d_set_stream(P2Ctx* c, cudaStream_t s) {
    if (c->own_stream && c->s) cudaStreamSynchronize(c->s);
    if (!s) return MGLC_OK;  // keep the current stream
    if (c->own_stream) cudaStreamDestroy(c->s);
    c->s = s;
    c->own_stream = false;
    return MGLC_OK;
}

int p2d_initial(P2Ctx* c, std::string& err) {
    D2& d = c->d;
    const size_t cells = (size_t)d.X * (d.p.ny + 6), np3 = 3 * (size_t)(d.p.np > 0 ? d.p.np : 1);
    int rc = 0;
    for (auto& pr : {std::make_pair((void*)d.f, 9 * cells * 8), std::make_pair((void*)d.fp, 9 * cells * 8),
                     std::make_pair((void*)d.ob, cells * 4), std::make_pair((void*)d.on, cells * 4),
                     std::make_pair((void*)d.uc, np3 * 8), std::make_pair((void*)d.om, np3 * 8),
                     std::make_pair((void*)d.force, np3 * 8), std::make_pair((void*)d.torque, np3 * 8),
                     std::make_pair((void*)d.status, (size_t)8)})
        if ((rc = ck(cudaMemsetAsync(pr.first, 0, pr.second, c->s), "reset", err))) return rc;
    if (d.p.np > 0) {
        if ((rc = ck(cudaMemcpyAsync(d.xc, c->centers.data(), sizeof(double) * 3 * d.p.np,
                                     cudaMemcpyHostToDevice, c->s), "centres", err)))
            return rc;
        if ((rc = ck(cudaMemcpyAsync(d.xco, d.xc, sizeof(double) * 3 * d.p.np, cudaMemcpyDeviceToDevice,
                                     c->s), "centres", err)))
            return rc;
    }
    if (d.p.variant == P2_SHEAR && d.p.np > 0) {  // case1 initial.F90:61-70
        std::vector<double> uc(3 * (size_t)d.p.np, 0.0);
        for (int q = 0; q < d.p.np; q++) uc[3 * q] = d.p.moving_frame ? 0.0 : d.p.u0;
        if ((rc = ck(cudaMemcpyAsync(d.uc, uc.data(), sizeof(double) * uc.size(),
                                     cudaMemcpyHostToDevice, c->s), "velocities", err)))
            return rc;
        if ((rc = ck(cudaStreamSynchronize(c->s), "velocities", err))) return rc;
    }
    k2_mask<<<dim3((d.p.nx + 2 + 127) / 128, d.p.ny + 2), 128, 0, c->s>>>(d, d.ob, false);
    k2_init_fields<<<dim3((d.p.nx + 6 + 127) / 128, d.p.ny + 6), 128, 0, c->s>>>(d);
    c->itc = 0;
    return ck(cudaStreamSynchronize(c->s), "initial", err);
}

int p2d_step(P2Ctx* c, int nsteps, std::string& err) {
    D2& d = c->d;
    const dim3 g = rows_grid(d);
    const int nw = d.p.nx > d.p.ny ? d.p.nx : d.p.ny;
    const int pg = (d.p.np + 63) / 64;
    const size_t cells = (size_t)d.X * (d.p.ny + 6);
    for (int n = 0; n < nsteps; n++) {
        k2_collide<<<g, 128, 0, c->s>>>(d);
        k2_stream<<<g, 128, 0, c->s>>>(d);
        k2_walls<<<(nw + 127) / 128, 128, 0, c->s>>>(d);
        gs_launch(RhoFetch{d, d.ob, d.p.nx * d.p.ny}, d.p.nx * d.p.ny, gs_of(d), d.ravg, true,
                  d.status, c->s);
        k2_ibb<<<g, 128, 0, c->s>>>(d);
        k2_macro<<<g, 128, 0, c->s>>>(d);
        if (d.p.np > 0) {
            k2_links<<<g, 128, 0, c->s>>>(d);
            k2_force<<<d.p.np, 32, 0, c->s>>>(d);
            k2_move<<<pg, 64, 0, c->s>>>(d);
        }
        k2_mask<<<dim3((d.p.nx + 2 + 127) / 128, d.p.ny + 2), 128, 0, c->s>>>(d, d.on, true);
        gs_launch(RhoFetch{d, d.on, d.p.nx * d.p.ny}, d.p.nx * d.p.ny, gs_of(d), d.ravg, true,
                  d.status, c->s);
        cudaMemsetAsync(d.rf_count, 0, sizeof(int), c->s);
        k2_refill_find<<<g, 128, 0, c->s>>>(d);
        k2_refill<<<1, SB, 0, c->s>>>(d);
        cudaMemcpyAsync(d.ob, d.on, cells * sizeof(int), cudaMemcpyDeviceToDevice, c->s);
        c->itc++;
    }
    int st[2] = {0, 0};
    int rc = ck(cudaGetLastError(), "particle step launch", err);
    if (!rc) rc = ck(cudaMemcpyAsync(st, d.status, sizeof st, cudaMemcpyDeviceToHost, c->s), "status", err);
    if (!rc) rc = ck(cudaStreamSynchronize(c->s), "particle step", err);
    if (rc) return rc;
    if (st[0]) {
        static const char* what[] = {"", "no circle owns a solid boundary node",
                                     "interpolation fraction q outside [0,1]",
                                     "particle-particle interpenetration",
                                     "particle penetrates a wall",
                                     "no refill direction for a node leaving a circle"};
        char buf[200];
        std::snprintf(buf, sizeof buf, "%s (circle %d); the state is frozen at that step",
                      what[st[0] < 6 ? st[0] : 0], st[1]);
        err = buf;
        return MGLC_ERR_PARTICLE;
    }
    return MGLC_OK;
}

namespace {
// interior of a padded device array, row by row (x fastest)
template <typename T>
int get_interior(P2Ctx* c, const T* dev, int per, T* host, std::string& err) {
    const D2& d = c->d;
    const size_t pitch = sizeof(T) * per * d.X;
    const T* first = dev + (size_t)per * (3 + (size_t)d.X * 3);  // node (1, 1)
    cudaError_t e = cudaMemcpy2DAsync(host, sizeof(T) * per * d.p.nx, first, pitch,
                                      sizeof(T) * per * d.p.nx, d.p.ny, cudaMemcpyDeviceToHost, c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    return ck(e, "copy to host", err);
}
}  // namespace

int p2d_get_f(P2Ctx* c, double* f, std::string& err) { return get_interior(c, c->d.f, 9, f, err); }

int p2d_get_macros(P2Ctx* c, double* rho, double* u, double* v, double* w, std::string& err) {
    int rc = 0;
    if (rho && (rc = get_interior(c, c->d.rho, 1, rho, err))) return rc;
    if (u && (rc = get_interior(c, c->d.u, 1, u, err))) return rc;
    if (v && (rc = get_interior(c, c->d.v, 1, v, err))) return rc;
    if (w) std::memset(w, 0, sizeof(double) * (size_t)c->d.p.nx * c->d.p.ny);
    return MGLC_OK;
}

int p2d_state(P2Ctx* c, double* xc, double* uc, double* omega, double* force, double* torque,
              std::string& err) {
    const D2& d = c->d;
    const size_t b = sizeof(double) * 3 * d.p.np;
    const double* src[] = {d.xc, d.uc, d.om, d.force, d.torque};
    double* dst[] = {xc, uc, omega, force, torque};
    for (int q = 0; q < 5; q++)
        if (dst[q] && b) {
            int rc = ck(cudaMemcpyAsync(dst[q], src[q], b, cudaMemcpyDeviceToHost, c->s), "state", err);
            if (rc) return rc;
        }
    return ck(cudaStreamSynchronize(c->s), "state", err);
}

int p2d_mask(P2Ctx* c, int* owner, std::string& err) {
    const D2& d = c->d;
    k2_owner<<<rows_grid(d), 128, 0, c->s>>>(d, c->owner_tmp);
    cudaError_t e = cudaMemcpyAsync(owner, c->owner_tmp, sizeof(int) * (size_t)d.p.nx * d.p.ny,
                                    cudaMemcpyDeviceToHost, c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    return ck(e, "mask", err);
}

long long p2d_itc(const P2Ctx* c) { return c->itc; }
long long p2d_device_bytes(const P2Ctx* c) { return c->bytes; }

double p2d_rho_avg(P2Ctx* c) {
    double r = 0.0;
    cudaMemcpyAsync(&r, c->d.ravg, sizeof r, cudaMemcpyDeviceToHost, c->s);
    cudaStreamSynchronize(c->s);
    return r;
}

}  // namespace mglc

extern "C" int mglc_sequential_sum(const double* x, const int* keep, int n, double* sum,
                                   long long* count) {
    if (n < 0 || !x || !keep || !sum || !count) return MGLC_ERR_INVALID;
    const size_t m = n > 0 ? (size_t)n : 1, nch = (size_t)mglc::gs_chunks(n);
    double *dx = nullptr, *dout = nullptr, *part = nullptr, *pre = nullptr;
    int *dk = nullptr, *ge = nullptr, *gf = nullptr, *gc = nullptr;
    mglc::GridSeg* gmap = nullptr;
    long long* gub = nullptr;
    cudaError_t e = cudaMalloc(&dx, m * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dk, m * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&dout, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&part, nch * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&pre, nch * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&gmap, nch * sizeof(mglc::GridSeg));
    if (e == cudaSuccess) e = cudaMalloc(&gub, nch * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&ge, nch * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&gf, nch * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&gc, nch * sizeof(int));
    if (e == cudaSuccess && n > 0) e = cudaMemcpy(dx, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n > 0) e = cudaMemcpy(dk, keep, (size_t)n * sizeof(int), cudaMemcpyHostToDevice);
    double out[2] = {0.0, 0.0};
    if (e == cudaSuccess) {
        const mglc::GsBuf b{part, pre, gmap, gub, ge, gf, gc};
        mglc::gs_launch(mglc::ArrayFetch{dx, dk, n}, n, b, dout, false, nullptr, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof out, cudaMemcpyDeviceToHost);
    void* ps[] = {dx, dk, dout, part, pre, gmap, gub, ge, gf, gc};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (e != cudaSuccess) return MGLC_ERR_CUDA;
    *sum = out[0];
    *count = (long long)out[1];
    return MGLC_OK;
}
