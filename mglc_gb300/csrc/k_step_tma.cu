// k_step_tma.cu -- the lid-driven-cavity step with its population loads
// staged through shared memory by the bulk-copy engine (cp.async.bulk +
// mbarrier), for the FP32 and 16-bit storage forms.
//
// The arithmetic is lid_cell_from's (step_cell.cuh), so every bit of the
// result equals the one-thread-per-cell kernel's; only the loads change.  A
// persistent CTA walks a contiguous range of tiles (x-row segments of up to
// 128 cells); one thread issues, NSTAGE - 1 tiles ahead, the 19 bulk copies
// of a tile (one per population plane, 16-byte aligned rows) into a
// shared-memory stage, completing on that stage's mbarrier.  The threads read
// their cell's populations from shared memory (fixed offsets from one base),
// collide and push to global memory as before.  Loads no longer cost each
// thread 19 address computations and 19 long-latency global loads, and the
// copies of later tiles are in flight while a tile is computed.
//
// Every wait is bounded: a stage that has not completed after about a second
// sets the context's step status word, the CTA waits (again bounded) for its
// remaining copies and returns, and the host reports the status at its next
// read of the state.
#include "step_cell.cuh"

namespace mglc {

constexpr int TMA_T = 128;                    // cells per tile = threads per CTA
constexpr int TMA_NSTAGE = 4;                 // shared-memory stages
constexpr long long TMA_WAIT_CYCLES = 2000000000LL;  // about 1 s at 2 GHz
constexpr int TMA_STATUS_TIMEOUT = 1;

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase with the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    if (mbar_test(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (clock64() - t0 > TMA_WAIT_CYCLES) return false;
        __nanosleep(64);
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// tile t of a lattice with nseg x-segments per row -> (i0, j, k), advanced
// incrementally (no divisions inside the loops)
struct TileIt {
    int seg, j, k;
    __device__ void start(int t, int nseg, int ny) {
        seg = t % nseg;
        const int r = t / nseg;
        j = r % ny;
        k = r / ny;
    }
    __device__ void next(int nseg, int ny) {
        if (++seg == nseg) {
            seg = 0;
            if (++j == ny) {
                j = 0;
                ++k;
            }
        }
    }
};

// resident CTAs per SM the register allocation is held to
#ifndef MGLC_TMA_MINB
#define MGLC_TMA_MINB 1
#endif

template <typename S, typename IDX, bool SR>
__global__ void __launch_bounds__(TMA_T, MGLC_TMA_MINB)
    k_lid_step_tma(const S* __restrict__ fin, S* __restrict__ fout, StepK<typename St<S>::C> K,
                   IDX P, int ntiles, int* status) {
    __shared__ __align__(128) S sm[TMA_NSTAGE][Q19][TMA_T];
    __shared__ __align__(8) unsigned long long bar[TMA_NSTAGE];
    const int tid = threadIdx.x;
    const int nx = K.nx, ny = K.ny;
    const int nseg = (nx + TMA_T - 1) / TMA_T;
    // this CTA's contiguous range of tiles
    const int t0 = (int)((long long)blockIdx.x * ntiles / gridDim.x);
    const int t1 = (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x);
    const int nt = t1 - t0;
    if (tid == 0) {
        for (int s = 0; s < TMA_NSTAGE; s++) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    TileIt prod;  // producer position (thread 0 only)
    auto issue = [&](int n) {  // tile t0 + n into stage n % NSTAGE
        const int st = (int)(n % TMA_NSTAGE);
        const int i0 = prod.seg * TMA_T;
        const int w = min(TMA_T, nx - i0);
        const unsigned bytes = (unsigned)(w * sizeof(S));
        const IDX c0 = (IDX)i0 + (IDX)nx * ((IDX)prod.j + (IDX)ny * (IDX)prod.k);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[st], bytes * Q19);
#pragma unroll
        for (int q = 0; q < Q19; q++) bulk_g2s(&sm[st][q][0], fin + ((IDX)q * P + c0), bytes, &bar[st]);
        prod.next(nseg, ny);
    };
    if (tid == 0) {
        prod.start(t0, nseg, ny);
        for (int n = 0; n < TMA_NSTAGE - 1 && n < nt; n++) issue(n);
    }
    TileIt cur;
    cur.start(t0, nseg, ny);
    bool failed = false;
    int n = 0;
    for (; n < nt; n++) {
        if (tid == 0 && n + TMA_NSTAGE - 1 < nt) issue(n + TMA_NSTAGE - 1);
        const int st = (int)(n % TMA_NSTAGE);
        const bool ok = mbar_wait(&bar[st], (unsigned)((n / TMA_NSTAGE) & 1));
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const int i = cur.seg * TMA_T + tid;
        S raw[Q19];
        if (i < nx) {
#pragma unroll
            for (int q = 0; q < Q19; q++) raw[q] = sm[st][q][tid];
        }
        __syncthreads();  // stage st is free for tile n + NSTAGE
        if (i < nx)
            lid_cell_from<S, false, IDX, SR>(i, cur.j, cur.k, raw, fout, K, P, nullptr, nullptr,
                                             nullptr, nullptr, K.seed);
        cur.next(nseg, ny);
    }
    if (failed && tid == 0) {
        atomicExch(status, TMA_STATUS_TIMEOUT);
        // copies issued for tiles n .. n + NSTAGE - 1: wait (bounded) before leaving
        for (int m = n; m < nt && m < n + TMA_NSTAGE; m++)
            mbar_wait(&bar[m % TMA_NSTAGE], (unsigned)((m / TMA_NSTAGE) & 1));
    }
}

// Usable when every bulk copy starts and ends on 16 bytes: rows of a multiple
// of 16 bytes (nx * sizeof(S) % 16 == 0, so every plane and tile offset is
// aligned too) and 16-byte aligned buffers.
bool lid_tma_ok(const Geom& g, size_t elem, const void* fin, const void* fout) {
    return ((size_t)g.nx * elem) % 16 == 0 && ((uintptr_t)fin % 16) == 0 &&
           ((uintptr_t)fout % 16) == 0;
}

template <typename S>
static cudaError_t go(const void* fin, void* fout, const LidStepArgs& a, int* status,
                      cudaStream_t s) {
    using C = typename St<S>::C;
    StepK<C> K = make_k<C>(a.g, a.cd, a.u0, a.rho0, a.scale, a.inv_scale);
    K.seed = a.seed;
    K.sr = a.sr;
    const int nseg = (a.g.nx + TMA_T - 1) / TMA_T;
    const long long ntl = (long long)nseg * a.g.ny * a.g.nz;  // below 2^31: ny, nz <= 65535
    if (ntl >= (1ll << 31)) return cudaErrorInvalidValue;
    const int ntiles = (int)ntl;
    static int ctas[8][2][2] = {};  // per device ordinal: resident CTAs per SM, cached
    int dev = 0;
    cudaGetDevice(&dev);
    const bool small = (long long)Q19 * a.g.plane < (1ll << 31);
    const bool sr = sizeof(S) == 2 && a.sr;
    int& per_sm = ctas[dev & 7][small][sr];
    if (per_sm == 0) {
        cudaError_t e;
        if (small)
            e = sr ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lid_step_tma<S, unsigned, sizeof(S) == 2>, TMA_T, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lid_step_tma<S, unsigned, false>, TMA_T, 0);
        else
            e = sr ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lid_step_tma<S, long long, sizeof(S) == 2>, TMA_T, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lid_step_tma<S, long long, false>, TMA_T, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (long long)sms * per_sm;
    const int grid = (int)(ntiles < want ? ntiles : want);
    if (small) {
        if (sr) k_lid_step_tma<S, unsigned, sizeof(S) == 2><<<grid, TMA_T, 0, s>>>((const S*)fin, (S*)fout, K, (unsigned)a.g.plane, ntiles, status);
        else k_lid_step_tma<S, unsigned, false><<<grid, TMA_T, 0, s>>>((const S*)fin, (S*)fout, K, (unsigned)a.g.plane, ntiles, status);
    } else {
        if (sr) k_lid_step_tma<S, long long, sizeof(S) == 2><<<grid, TMA_T, 0, s>>>((const S*)fin, (S*)fout, K, (long long)a.g.plane, ntiles, status);
        else k_lid_step_tma<S, long long, false><<<grid, TMA_T, 0, s>>>((const S*)fin, (S*)fout, K, (long long)a.g.plane, ntiles, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_lid_step_tma(int form, const void* fin, void* fout, const LidStepArgs& a,
                                int* status, cudaStream_t s) {
    switch (form) {
        case FORM_FP32: return go<float>(fin, fout, a, status, s);
        case FORM_FP16: return go<__half>(fin, fout, a, status, s);
        case FORM_BF16: return go<__nv_bfloat16>(fin, fout, a, status, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace mglc
