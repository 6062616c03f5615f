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
__global__ void __launch_bounds__(128)
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

// Pairwise exchange (q, x) <-> (opp(q), x - e_q) for the nine directions with
// opp(q) > q: the streaming half of a step, without collision.  The pair is
// owned by the thread of x, so the exchange is race-free; where x - e_q is
// outside, slot q of x already holds the reflected population.
template <typename S, typename IDX>
__global__ void __launch_bounds__(128) k_aa_swap(S* f, int nx, int ny, int nz, IDX P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const IDX cell = (IDX)i + (IDX)nx * ((IDX)j + (IDX)ny * (IDX)k);
    const IDX sy = (IDX)nx, sz = (IDX)nx * (IDX)ny;
    const unsigned bm = face_mask(i, j, k, nx, ny, nz);
#pragma unroll
    for (int q = 1; q < Q19; q++) {
        if (opp19(q) < q) continue;
        const int dx = ex19(q), dy = ey19(q), dz = ez19(q);
        if ((bm & leave_bits(-dx, -dy, -dz)) != 0) continue;
        S* a = f + ((IDX)q * P + cell);
        S* b = f + ((IDX)opp19(q) * P + cell - (IDX)(dx + dy * (int)sy) - (IDX)dz * sz);
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

template <typename S>
cudaError_t swap_go(const Geom& g, void* f, cudaStream_t s) {
    const dim3 b = aa_block(g.nx), gr((g.nx + b.x - 1) / b.x, g.ny, g.nz);
    if ((long long)Q19 * g.plane < (1ll << 31))
        k_aa_swap<S, unsigned><<<gr, b, 0, s>>>((S*)f, g.nx, g.ny, g.nz, (unsigned)g.plane);
    else
        k_aa_swap<S, long long><<<gr, b, 0, s>>>((S*)f, g.nx, g.ny, g.nz, (long long)g.plane);
    return cudaGetLastError();
}

}  // namespace

// first: the step reads the stored macroscopic fields (after initial/load; the
// layout is then the post-stream one, so first implies an even step)
cudaError_t launch_lid_step_aa(int form, bool first, bool odd, void* f, const LidStepArgs& a,
                               cudaStream_t s) {
    if (first && odd) return cudaErrorInvalidValue;
    switch (form) {
        case FORM_FP64: return lid_go_aa<double>(first, odd, f, a, s);
        case FORM_FP32: return lid_go_aa<float>(first, odd, f, a, s);
        case FORM_FP16: return lid_go_aa<__half>(first, odd, f, a, s);
        case FORM_BF16: return lid_go_aa<__nv_bfloat16>(first, odd, f, a, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_aa_swap(int form, const Geom& g, void* f, cudaStream_t s) {
    switch (form) {
        case FORM_FP64: return swap_go<double>(g, f, s);
        case FORM_FP32: return swap_go<float>(g, f, s);
        case FORM_FP16: return swap_go<__half>(g, f, s);
        case FORM_BF16: return swap_go<__nv_bfloat16>(g, f, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace mglc
