// static_residual.cu -- residual of check() that allocates no device memory.
//
// Who needs this: a host that cannot call cudaMalloc itself -- for example a
// Fortran/OpenACC program or a serving process whose device memory is owned
// entirely by another runtime's fixed pool, or a latency-critical loop that
// must not pay cudaMalloc's implicit device synchronisation.  Such a caller
// keeps its velocity fields in memory it already owns and asks only for the
// reference's residual (errorU, errorT).  The per-block partial sums this
// reduction needs live in a file-scope static __device__ array instead of a
// cudaMalloc'd buffer; every GPU that loads the library holds that array
// (512 KiB + 32 B) until the process exits.
//
// Limits and sharing: at most kMaxCells = 67,108,864 cells per call (larger n
// is rejected with MGLC_ERR_INVALID).  All calls in the process share the one
// array per device and it keeps the last call's contents; every slot a call
// reads is written earlier in the same call, so nothing needs clearing, but
// calls that overlap on the GPU (concurrent streams) race on the array and
// must be serialised by the caller.  The array's device address belongs to a
// CUDA context: the first call in each context on a device looks it up
// (cudaGetSymbolAddress, with that device current) and keeps it under the
// context's unique id, so a new context (after cudaDeviceReset, or a host
// runtime that makes its own) gets its own lookup; make that first call
// before any stream capture.  Each call waits for its stream to finish
// (cudaStreamSynchronize) before it returns the sums.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/mglc.h"

namespace {

constexpr int kBlock = 256;
constexpr int kCellsPerThread = 16;
constexpr long long kCellsPerBlock = (long long)kBlock * kCellsPerThread;  // 4096
constexpr int kMaxBlocks = 16384;
constexpr long long kMaxCells = kCellsPerBlock * kMaxBlocks;  // 67,108,864
constexpr int kMaxDevices = 64;

// 4 partial sums per block, then the 4 final sums
static __device__ __align__(256) double g_residual_scratch[kMaxBlocks * 4 + 4];

std::mutex g_setup_mu;
// one cached address per device, valid for the context whose id it records
struct ScratchSlot {
    bool valid;
    unsigned long long ctx_id;
    double* ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// driver entry points for the current context's unique id (CUDA 12.0+),
// looked up through the runtime so the library needs no libcuda link
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// One block per tile of kCellsPerBlock cells; each block writes its own four
// partial-sum slots (sum (u-up)^2+(v-vp)^2[+(w-wp)^2], sum |u|^2, sum |T-Tp|,
// sum |T|) and moves the current fields into the previous ones, like check().
__global__ void __launch_bounds__(kBlock)
    k_residual_tiles(long long n, const double* __restrict__ u, const double* __restrict__ v,
                     const double* __restrict__ w, const double* __restrict__ T, double* up,
                     double* vp, double* wp, double* Tp, int with_w, double* scratch) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const long long c0 = (long long)blockIdx.x * kCellsPerBlock;
    long long c1 = c0 + kCellsPerBlock;
    if (c1 > n) c1 = n;
    for (long long c = c0 + threadIdx.x; c < c1; c += kBlock) {
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
    __shared__ double sh[kBlock / 32][4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 4; k++) sh[wid][k] = acc[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) {
            double t = 0.0;
            for (int q = 0; q < kBlock / 32; q++) t += sh[q][k];
            scratch[4 * blockIdx.x + k] = t;
        }
}

// One warp sums the partials in a fixed order into the four final slots.
__global__ void k_residual_finish(int nblocks, double* scratch) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += 32)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] += scratch[4 * b + k];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 4; k++) scratch[4 * kMaxBlocks + k] = acc[k];
}

int set_error(char* buf, int len, int code, const char* msg) {
    if (buf && len > 0) std::snprintf(buf, (size_t)len, "%s", msg);
    return code;
}

// Device address of the static scratch in the current context.
int symbol_address(double** out, char* errbuf, int errlen) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_residual_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        char m[256];
        std::snprintf(m, sizeof m, "cudaGetSymbolAddress of the static residual scratch failed: %s",
                      cudaGetErrorString(e));
        return set_error(errbuf, errlen, MGLC_ERR_CUDA, m);
    }
    *out = (double*)p;
    return MGLC_OK;
}

// The scratch address for the current device's current context, looked up
// once per context (a context's id is unique for the life of the process).
int scratch_for_current_device(double** out, char* errbuf, int errlen) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char m[256];
        std::snprintf(m, sizeof m, "cudaGetDevice failed: %s", cudaGetErrorString(e));
        return set_error(errbuf, errlen, MGLC_ERR_CUDA, m);
    }
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(errbuf, errlen, MGLC_ERR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
        if (e != cudaSuccess || qa != cudaDriverEntryPointSuccess ||
            qb != cudaDriverEntryPointSuccess || !a || !b) {
            cudaGetLastError();
            return set_error(errbuf, errlen, MGLC_ERR_CUDA,
                             "the CUDA driver lacks cuCtxGetCurrent/cuCtxGetId (CUDA 12.0 or later needed)");
        }
        g_ctx_get_current = (CtxGetCurrentFn)a;
        g_ctx_get_id = (CtxGetIdFn)b;
    }
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0)
        return set_error(errbuf, errlen, MGLC_ERR_CUDA, "cuCtxGetCurrent failed");
    double* fresh = nullptr;
    if (!ctx) {
        // nothing current on this thread yet: the runtime call makes the
        // device's primary context current, then the context is known
        int rc = symbol_address(&fresh, errbuf, errlen);
        if (rc != MGLC_OK) return rc;
        if (g_ctx_get_current(&ctx) != 0 || !ctx)
            return set_error(errbuf, errlen, MGLC_ERR_CUDA, "no current CUDA context on this thread");
    }
    unsigned long long id = 0;
    if (g_ctx_get_id(ctx, &id) != 0)
        return set_error(errbuf, errlen, MGLC_ERR_CUDA, "cuCtxGetId failed");
    ScratchSlot& slot = g_scratch[dev];
    if (!slot.valid || slot.ctx_id != id) {
        if (!fresh) {
            int rc = symbol_address(&fresh, errbuf, errlen);
            if (rc != MGLC_OK) return rc;
        }
        slot.ptr = fresh;
        slot.ctx_id = id;
        slot.valid = true;
    }
    *out = slot.ptr;
    return MGLC_OK;
}

}  // namespace

extern "C" int mglc_residual_noalloc(long long n, const double* u, const double* v,
                                     const double* w, const double* T, double* up, double* vp,
                                     double* wp, double* Tp, int with_w, void* cuda_stream,
                                     double* error_u, double* error_t, char* errbuf,
                                     int errbuf_len) {
    if (errbuf && errbuf_len > 0) errbuf[0] = '\0';
    if (n < 1) return set_error(errbuf, errbuf_len, MGLC_ERR_INVALID, "n must be at least 1");
    if (n > kMaxCells) {
        char m[256];
        std::snprintf(m, sizeof m,
                      "n = %lld cells exceeds the static scratch limit of %lld cells "
                      "(use mglc_check on a context instead)",
                      n, kMaxCells);
        return set_error(errbuf, errbuf_len, MGLC_ERR_INVALID, m);
    }
    if (!u || !v || !w || !up || !vp || !wp)
        return set_error(errbuf, errbuf_len, MGLC_ERR_INVALID, "u, v, w, up, vp, wp are required");
    if ((T == nullptr) != (Tp == nullptr))
        return set_error(errbuf, errbuf_len, MGLC_ERR_INVALID, "T and Tp must be given together");
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch, errbuf, errbuf_len);
    if (rc != MGLC_OK) return rc;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    const int nb = (int)((n + kCellsPerBlock - 1) / kCellsPerBlock);
    cudaGetLastError();  // an earlier, unrelated launch error must not be taken for ours
    k_residual_tiles<<<nb, kBlock, 0, s>>>(n, u, v, w, T, up, vp, wp, Tp, with_w, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_residual_finish<<<1, 32, 0, s>>>(nb, scratch);
        e = cudaGetLastError();
    }
    double sums[4] = {0.0, 0.0, 0.0, 0.0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sums, scratch + 4 * kMaxBlocks, sizeof sums, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char m[256];
        std::snprintf(m, sizeof m, "residual kernels failed: %s", cudaGetErrorString(e));
        return set_error(errbuf, errbuf_len, MGLC_ERR_CUDA, m);
    }
    const double eu = std::sqrt(sums[0]) / std::sqrt(sums[1]);
    const double et = T ? sums[2] / sums[3] : 0.0;
    if (error_u) *error_u = eu;
    if (error_t) *error_t = et;
    // a zero velocity field (sum |u|^2 = 0) or zero temperature field gives
    // 0/0 or x/0, like a non-finite field: the ratios are written as computed
    // and the call reports MGLC_ERR_NUMERIC
    if (!std::isfinite(eu) || !std::isfinite(et))
        return set_error(errbuf, errbuf_len, MGLC_ERR_NUMERIC,
                         "residual not finite (a non-finite field, or sum |u|^2 or sum |T| is zero)");
    return MGLC_OK;
}
