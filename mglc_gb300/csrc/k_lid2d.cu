// k_lid2d.cu -- D2Q9 MRT lid-driven cavity, the reference's 2-D step
// (MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked, main.f90:69-89):
//
//   collision (evolution.f90:1-71), streaming (:75-94), bounceback
//   (bounceback.f90:1-45), macro (evolution.f90:98-112), check (:115-150).
//
// One fused kernel per step, one thread per node: it forms rho, u, v from the
// populations it loads (the previous step's macro, same statements; the step
// after initial()/load reads the stored fields instead), collides, and pushes
// each post-collision population to its neighbour, or reflects it into the
// opposite direction of the same node when the neighbour is outside (halfway
// bounce-back; a population leaving through the top row gets the lid term
// -rho*Uwall/6 * e_x, which also decides the two top corners, as the
// reference's top-wall loop runs last).
//
// Layout: two population buffers (ping-pong), SoA planes f[a][j][i] so that
// each of the 18 loads and stores of a warp is a contiguous row segment.  All
// arithmetic is FP64 in the reference's expression order and this file is
// compiled without FMA contraction (device and host), so every value rounds
// as the reference's statement does.  check() sums on the host in the
// reference's (j, i) loop order for the same reason.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mglc.h"
#include "lid2d.cuh"

namespace mglc {

namespace {

__device__ __constant__ int l2_ex[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
__device__ __constant__ int l2_ey[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
__device__ __constant__ int l2_op[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

// Quotients by the collision's constant divisors d = 6, 9, 12, 18, 36, rounded
// exactly as IEEE division rounds them, from one multiply and one fused
// multiply-add: x/d = RN(x*h + RN(x*l)) with h = 1/d rounded down and
// l = 1/d - h rounded to nearest (a two-term reciprocal; Brisebarre, Muller and
// Raina, "Accelerating correctly rounded floating-point division when the
// divisor is known in advance", IEEE Trans. Computers 53(8), 2004).  Why the
// rounding is the division's: d = 3*2^k or 9*2^k, so for normal x the exact
// x/d lies at least ulp(x/d)/18 from every rounding midpoint (d times a
// midpoint is an odd multiple of 2^(e-53), x an even one), while h + l is 1/d
// to about 2^-106 relative, putting x*h + RN(x*l) within ~2^-104 relative of
// x/d: no midpoint between them.  Zeros and infinities keep their signs
// because l > 0, NaN stays NaN.  Inputs below 2^-900 in magnitude (x*l could
// lose bits to underflow) take the true division: a node whose divided
// values are not all normal-or-zero runs the division variant.
constexpr double RH6 = 0x1.5555555555555p-3, RL6 = 0x1.5555555555555p-57;
constexpr double RH9 = 0x1.c71c71c71c71cp-4, RL9 = 0x1.c71c71c71c71cp-58;
constexpr double RH12 = 0x1.5555555555555p-4, RL12 = 0x1.5555555555555p-58;
constexpr double RH18 = 0x1.c71c71c71c71cp-5, RL18 = 0x1.c71c71c71c71cp-59;
constexpr double RH36 = 0x1.c71c71c71c71cp-6, RL36 = 0x1.c71c71c71c71cp-60;

template <bool FAST>
__device__ __forceinline__ double dv(double x, double d, double h, double l) {
    return FAST ? __fma_rn(x, h, __dmul_rn(x, l)) : x / d;
}

// |x| >= 2^-900 (infinities and NaN included) or x == +-0
__device__ __forceinline__ bool rcp_ok(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return ((b >> 52) & 0x7ff) >= 123 || (b << 1) == 0;
}

// f_post from m_post, evolution.f90:55-68, each quotient as its own rounded value
template <bool FAST>
__device__ __forceinline__ void l2_post(const double* mp, double* fp) {
    const double q0 = dv<FAST>(mp[0], 9.0, RH9, RL9), q1a = dv<FAST>(mp[1], 36.0, RH36, RL36),
                 q1b = dv<FAST>(mp[1], 18.0, RH18, RL18), q2a = dv<FAST>(mp[2], 18.0, RH18, RL18),
                 q2b = dv<FAST>(mp[2], 36.0, RH36, RL36), q3 = dv<FAST>(mp[3], 6.0, RH6, RL6),
                 q4 = dv<FAST>(mp[4], 6.0, RH6, RL6), q4b = dv<FAST>(mp[4], 12.0, RH12, RL12),
                 q5 = dv<FAST>(mp[5], 6.0, RH6, RL6), q6 = dv<FAST>(mp[6], 6.0, RH6, RL6),
                 q6b = dv<FAST>(mp[6], 12.0, RH12, RL12), q7 = mp[7] * 0.25, q8 = mp[8] * 0.25;
    fp[0] = dv<FAST>(mp[0] - mp[1] + mp[2], 9.0, RH9, RL9);
    fp[1] = q0 - q1a - q2a + q3 - q4 + q7;
    fp[2] = q0 - q1a - q2a + q5 - q6 - q7;
    fp[3] = q0 - q1a - q2a - q3 + q4 + q7;
    fp[4] = q0 - q1a - q2a - q5 + q6 - q7;
    fp[5] = q0 + q1b + q2b + q3 + q4b + q5 + q6b + q8;
    fp[6] = q0 + q1b + q2b - q3 - q4b + q5 + q6b - q8;
    fp[7] = q0 + q1b + q2b - q3 - q4b - q5 - q6b + q8;
    fp[8] = q0 + q1b + q2b + q3 + q4b - q5 - q6b - q8;
}

struct L2K {
    const double* __restrict__ fin;
    double* __restrict__ fout;
    const double *rho, *u, *v;  // stored fields, read by the first step only
    long long n;                // nx * ny
    int nx, ny;
    double snu, sq, uwall;
};

// initial.f90:40-68: rho0, u = U0 on the top row, equilibrium populations
__global__ void k_l2_initial(double* __restrict__ f, double* __restrict__ rho,
                             double* __restrict__ u, double* __restrict__ v, long long n, int nx,
                             int ny, double u0, double rho0) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int j = (int)(c / nx);
    const double r = rho0, uu = (j == ny - 1) ? u0 : 0.0, vv = 0.0;
    rho[c] = r;
    u[c] = uu;
    v[c] = vv;
    const double us2 = uu * uu + vv * vv;
    for (int a = 0; a < 9; a++) {
        const double om = a == 0 ? 4.0 / 9.0 : (a <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
        const double un = uu * (double)l2_ex[a] + vv * (double)l2_ey[a];
        f[(size_t)a * n + c] = r * om * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
    }
}

template <bool FIRST>
__global__ void __launch_bounds__(128) k_l2_step(L2K k) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= k.n) return;
    const int j = (int)(c / k.nx), i = (int)(c - (long long)j * k.nx);
    const size_t n = (size_t)k.n;
    double f[9];
#pragma unroll
    for (int a = 0; a < 9; a++) f[a] = k.fin[a * n + c];
    double r, u, v;
    if (FIRST) {
        r = k.rho[c];
        u = k.u[c];
        v = k.v[c];
    } else {  // macro, evolution.f90:103-107
        r = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
        u = (f[1] - f[3] + f[5] - f[6] - f[7] + f[8]) / r;
        v = (f[2] - f[4] + f[5] + f[6] - f[7] - f[8]) / r;
    }
    // collision, evolution.f90:16-68
    double m[9], meq[9], s[9], mp[9], fp[9];
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
    m[1] = -4.0 * f[0] - f[1] - f[2] - f[3] - f[4] + 2.0 * (f[5] + f[6] + f[7] + f[8]);
    m[2] = 4.0 * f[0] - 2.0 * (f[1] + f[2] + f[3] + f[4]) + f[5] + f[6] + f[7] + f[8];
    m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
    m[4] = -2.0 * f[1] + 2.0 * f[3] + f[5] - f[6] - f[7] + f[8];
    m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    m[6] = -2.0 * f[2] + 2.0 * f[4] + f[5] + f[6] - f[7] - f[8];
    m[7] = f[1] - f[2] + f[3] - f[4];
    m[8] = f[5] - f[6] + f[7] - f[8];
    meq[0] = r;
    meq[1] = r * (-2.0 + 3.0 * (u * u + v * v));
    meq[2] = r * (1.0 - 3.0 * (u * u + v * v));
    meq[3] = r * u;
    meq[4] = -r * u;
    meq[5] = r * v;
    meq[6] = -r * v;
    meq[7] = r * (u * u - v * v);
    meq[8] = r * (u * v);
    s[0] = 0.0;
    s[1] = k.snu;
    s[2] = k.snu;
    s[3] = 0.0;
    s[4] = k.sq;
    s[5] = 0.0;
    s[6] = k.sq;
    s[7] = k.snu;
    s[8] = k.snu;
#pragma unroll
    for (int a = 0; a < 9; a++) mp[a] = m[a] - s[a] * (m[a] - meq[a]);
    const bool fast = rcp_ok(mp[0]) && rcp_ok(mp[1]) && rcp_ok(mp[2]) && rcp_ok(mp[3]) &&
                      rcp_ok(mp[4]) && rcp_ok(mp[5]) && rcp_ok(mp[6]) &&
                      rcp_ok(mp[0] - mp[1] + mp[2]);
    if (fast)
        l2_post<true>(mp, fp);
    else
        l2_post<false>(mp, fp);
    // streaming + bounceback, evolution.f90:81-90 and bounceback.f90:6-42
#pragma unroll
    for (int a = 0; a < 9; a++) {
        const int di = i + l2_ex[a], dj = j + l2_ey[a];
        if (di >= 0 && di < k.nx && dj >= 0 && dj < k.ny) {
            k.fout[a * n + (size_t)dj * k.nx + di] = fp[a];
        } else {
            double val = fp[a];
            if (dj >= k.ny) {  // top wall, bounceback.f90:37-41
                if (l2_ex[a] > 0) val = fp[a] - r * (k.uwall) / 6.0;
                else if (l2_ex[a] < 0) val = fp[a] - r * (-k.uwall) / 6.0;
            }
            k.fout[l2_op[a] * n + c] = val;
        }
    }
}

// macro, evolution.f90:98-112 (or the stored fields before the first step)
__global__ void k_l2_macro(const double* __restrict__ f, const double* __restrict__ srho,
                           const double* __restrict__ su, const double* __restrict__ sv,
                           int stored, long long n, double* __restrict__ rho,
                           double* __restrict__ u, double* __restrict__ v) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= n) return;
    double r, uu, vv;
    if (stored) {
        r = srho[c];
        uu = su[c];
        vv = sv[c];
    } else {
        double q[9];
        for (int a = 0; a < 9; a++) q[a] = f[(size_t)a * n + c];
        r = q[0] + q[1] + q[2] + q[3] + q[4] + q[5] + q[6] + q[7] + q[8];
        uu = (q[1] - q[3] + q[5] - q[6] - q[7] + q[8]) / r;
        vv = (q[2] - q[4] + q[5] + q[6] - q[7] - q[8]) / r;
    }
    if (rho) rho[c] = r;
    if (u) u[c] = uu;
    if (v) v[c] = vv;
}

}  // namespace

struct L2Ctx {
    L2Params p{};
    long long n = 0;
    cudaStream_t s = nullptr;
    bool own_stream = false;
    double* f[2] = {nullptr, nullptr};
    int cur = 0;
    double *rho = nullptr, *u = nullptr, *v = nullptr;  // stored fields (first step)
    double *mr = nullptr, *mu = nullptr, *mv = nullptr;  // macro output scratch
    std::vector<double> up, vp;                          // check(): previous fields
    bool first_pending = false;
    bool initialised = false;
    long long itc = 0;
    long long bytes = 0;
};

namespace {

int ck(cudaError_t e, const char* what, std::string& err) {
    if (e == cudaSuccess) return MGLC_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return MGLC_ERR_CUDA;
}

int dal(L2Ctx* c, double** p, size_t n, std::string& err) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(double));
    if (e != cudaSuccess) {
        err = std::string("device allocation: ") + cudaGetErrorString(e);
        return MGLC_ERR_NOMEM;
    }
    c->bytes += (long long)(n * sizeof(double));
    return cudaMemsetAsync(*p, 0, n * sizeof(double), c->s) == cudaSuccess ? MGLC_OK
                                                                             : MGLC_ERR_CUDA;
}

unsigned blocks_of(long long n) { return (unsigned)((n + 127) / 128); }

}  // namespace

int l2d_create(const L2Params& p, L2Ctx** out, std::string& err) {
    L2Ctx* c = new L2Ctx();
    *out = c;
    c->p = p;
    c->n = (long long)p.nx * p.ny;
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
        err = "stream creation failed";
        return MGLC_ERR_CUDA;
    }
    c->own_stream = true;
    const size_t n = (size_t)c->n;
    int rc = 0;
    if ((rc = dal(c, &c->f[0], 9 * n, err)) || (rc = dal(c, &c->f[1], 9 * n, err)) ||
        (rc = dal(c, &c->rho, n, err)) || (rc = dal(c, &c->u, n, err)) ||
        (rc = dal(c, &c->v, n, err)) || (rc = dal(c, &c->mr, n, err)) ||
        (rc = dal(c, &c->mu, n, err)) || (rc = dal(c, &c->mv, n, err)))
        return rc;
    c->up.assign(n, 0.0);
    c->vp.assign(n, 0.0);
    return ck(cudaStreamSynchronize(c->s), "create", err);
}

void l2d_destroy(L2Ctx* c) {
    if (!c) return;
    if (c->s) cudaStreamSynchronize(c->s);
    double* ps[] = {c->f[0], c->f[1], c->rho, c->u, c->v, c->mr, c->mu, c->mv};
    for (double* q : ps)
        if (q) cudaFree(q);
    if (c->own_stream && c->s) cudaStreamDestroy(c->s);
    delete c;
}

int l2d_set_stream(L2Ctx* c, cudaStream_t s) {
    if (c->own_stream && c->s) cudaStreamSynchronize(c->s);
    if (!s) return MGLC_OK;
    if (c->own_stream) cudaStreamDestroy(c->s);
    c->s = s;
    c->own_stream = false;
    return MGLC_OK;
}

int l2d_initial(L2Ctx* c, std::string& err) {
    c->cur = 0;
    k_l2_initial<<<blocks_of(c->n), 128, 0, c->s>>>(c->f[0], c->rho, c->u, c->v, c->n, c->p.nx,
                                                     c->p.ny, c->p.u0, c->p.rho0);
    int rc = ck(cudaGetLastError(), "initial launch", err);
    if (rc) return rc;
    std::fill(c->up.begin(), c->up.end(), 0.0);  // initial.f90:43-44
    std::fill(c->vp.begin(), c->vp.end(), 0.0);
    c->first_pending = true;
    c->initialised = true;
    c->itc = 0;
    return MGLC_OK;
}

int l2d_load(L2Ctx* c, const double* f, const double* rho, const double* u, const double* v,
             std::string& err) {
    const bool given = rho || u || v;
    if (given && !(rho && u && v)) {
        err = "rho, u and v are given together or not at all";
        return MGLC_ERR_INVALID;
    }
    const size_t n = (size_t)c->n;
    std::vector<double> soa(9 * n);
    for (size_t q = 0; q < n; q++)
        for (int a = 0; a < 9; a++) soa[(size_t)a * n + q] = f[9 * q + a];
    c->cur = 0;
    int rc = ck(cudaMemcpyAsync(c->f[0], soa.data(), 9 * n * sizeof(double),
                                cudaMemcpyHostToDevice, c->s), "load f", err);
    if (!rc && given) {
        if ((rc = ck(cudaMemcpyAsync(c->rho, rho, n * 8, cudaMemcpyHostToDevice, c->s), "load", err)) ||
            (rc = ck(cudaMemcpyAsync(c->u, u, n * 8, cudaMemcpyHostToDevice, c->s), "load", err)) ||
            (rc = ck(cudaMemcpyAsync(c->v, v, n * 8, cudaMemcpyHostToDevice, c->s), "load", err)))
            return rc;
    }
    if (!rc) rc = ck(cudaStreamSynchronize(c->s), "load", err);
    if (rc) return rc;
    c->first_pending = given;
    c->initialised = true;
    c->itc = 0;
    return MGLC_OK;
}

int l2d_step(L2Ctx* c, int nsteps, std::string& err) {
    if (!c->initialised) {
        err = "call mglc_initial or mglc_load_state first";
        return MGLC_ERR_STATE;
    }
    L2K k{};
    k.rho = c->rho;
    k.u = c->u;
    k.v = c->v;
    k.n = c->n;
    k.nx = c->p.nx;
    k.ny = c->p.ny;
    k.snu = c->p.snu;
    k.sq = c->p.sq;
    k.uwall = c->p.u0;
    for (int t = 0; t < nsteps; t++) {
        k.fin = c->f[c->cur];
        k.fout = c->f[c->cur ^ 1];
        if (c->first_pending)
            k_l2_step<true><<<blocks_of(c->n), 128, 0, c->s>>>(k);
        else
            k_l2_step<false><<<blocks_of(c->n), 128, 0, c->s>>>(k);
        c->first_pending = false;
        c->cur ^= 1;
        c->itc++;
    }
    return ck(cudaGetLastError(), "lid2d step launch", err);
}

int l2d_get_f(L2Ctx* c, double* f, std::string& err) {
    const size_t n = (size_t)c->n;
    std::vector<double> soa(9 * n);
    int rc = ck(cudaMemcpyAsync(soa.data(), c->f[c->cur], 9 * n * 8, cudaMemcpyDeviceToHost, c->s),
                "get f", err);
    if (!rc) rc = ck(cudaStreamSynchronize(c->s), "get f", err);
    if (rc) return rc;
    for (size_t q = 0; q < n; q++)
        for (int a = 0; a < 9; a++) f[9 * q + a] = soa[(size_t)a * n + q];
    return MGLC_OK;
}

namespace {
int l2_macro_launch(L2Ctx* c, double* rho, double* u, double* v, std::string& err) {
    k_l2_macro<<<blocks_of(c->n), 128, 0, c->s>>>(c->f[c->cur], c->rho, c->u, c->v,
                                                   c->first_pending ? 1 : 0, c->n, rho, u, v);
    return ck(cudaGetLastError(), "macro launch", err);
}
}  // namespace

int l2d_get_macros_device(L2Ctx* c, double* rho, double* u, double* v, double* w,
                          std::string& err) {
    if (!c->initialised) {
        err = "call mglc_initial or mglc_load_state first";
        return MGLC_ERR_STATE;
    }
    int rc = l2_macro_launch(c, rho, u, v, err);
    if (!rc && w) rc = ck(cudaMemsetAsync(w, 0, (size_t)c->n * 8, c->s), "zero w", err);
    return rc ? rc : ck(cudaStreamSynchronize(c->s), "macros", err);
}

int l2d_get_macros(L2Ctx* c, double* rho, double* u, double* v, double* w, std::string& err) {
    if (!c->initialised) {
        err = "call mglc_initial or mglc_load_state first";
        return MGLC_ERR_STATE;
    }
    const size_t n = (size_t)c->n;
    int rc = l2_macro_launch(c, c->mr, c->mu, c->mv, err);
    double* outs[3] = {rho, u, v};
    double* devs[3] = {c->mr, c->mu, c->mv};
    for (int q = 0; q < 3 && !rc; q++)
        if (outs[q])
            rc = ck(cudaMemcpyAsync(outs[q], devs[q], n * 8, cudaMemcpyDeviceToHost, c->s),
                    "get macros", err);
    if (!rc) rc = ck(cudaStreamSynchronize(c->s), "get macros", err);
    if (!rc && w) std::memset(w, 0, n * sizeof(double));
    return rc;
}

// evolution.f90:115-150: error1/error2 summed in the reference's loop order
int l2d_check(L2Ctx* c, double* error_u, std::string& err) {
    const size_t n = (size_t)c->n;
    std::vector<double> u(n), v(n);
    int rc = l2d_get_macros(c, nullptr, u.data(), v.data(), nullptr, err);
    if (rc) return rc;
    double e1 = 0.0, e2 = 0.0;
    for (size_t q = 0; q < n; q++) {
        e1 = e1 + (u[q] - c->up[q]) * (u[q] - c->up[q]) + (v[q] - c->vp[q]) * (v[q] - c->vp[q]);
        e2 = e2 + u[q] * u[q] + v[q] * v[q];
    }
    c->up.swap(u);
    c->vp.swap(v);
    if (error_u) *error_u = std::sqrt(e1) / std::sqrt(e2);
    return MGLC_OK;
}

long long l2d_itc(const L2Ctx* c) { return c->itc; }
long long l2d_device_bytes(const L2Ctx* c) { return c->bytes; }

}  // namespace mglc
