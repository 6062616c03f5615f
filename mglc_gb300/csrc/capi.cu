// capi.cu -- the C-ABI of libmglc_gb300.so (declared in include/mglc.h).
//
// A context owns every device buffer of one solve: two population buffers
// (ping-pong, SoA planes), the macroscopic fields the first collision after
// initial()/load reads, the previous fields of the residual check, the
// carried body force (thermal), and a small reduction scratch.  All work runs
// on the context's stream.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mglc.h"
#include "kernels.cuh"
#include "particles.cuh"
#include "particles2d.cuh"
#include "lid2d.cuh"

using namespace mglc;

namespace {
// NVTX range around an entry point (visible in Nsight timelines; a no-op
// unless a tool is attached)
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};
}  // namespace

struct mglc_ctx {
    int kind = 0, form = FORM_FP64;
    bool fx64 = false;  // MGLC_FX64: FP64 storage (form FP64), Q55 fixed-point lid collision
    P2Ctx* p2d = nullptr;  // MGLC_KIND_PARTICLE2D: the D2Q9 case4 state
    L2Ctx* l2d = nullptr;  // MGLC_KIND_LID2D: the D2Q9 lid-driven cavity
    bool sr = false;       // MGLC_FP16S / MGLC_BF16S: stochastic rounding of the 16-bit stores
    bool in_place = false; // lid: AA pattern on one population buffer (f[1] unused)
    bool swapped = false;  // in place: the buffer holds an even step's output (swap pending)
    Geom geom{};
    long long n = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // constants
    double tauf = 0, snu = 0, sq = 0, u0 = 0, rho0 = 1.0;
    int top_layer_u0 = 1;
    double viscosity = 0, diffusivity = 0, para_a = 0, gbeta = 0, omega_rot = 0, qd = 0, qnu = 0;
    double t_hot = 0, t_cold = 0, t_ref = 0;
    int bc_y = 1, bc_z = 0;
    float scale = 1.0f, inv_scale = 1.0f;
    // device buffers
    void* f[2] = {nullptr, nullptr};
    void* g[2] = {nullptr, nullptr};
    int cur = 0;
    void* F = nullptr;  // carried force, 3 planes (thermal)
    double *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *T = nullptr;
    double *up = nullptr, *vp = nullptr, *wp = nullptr, *Tp = nullptr;
    double* partials = nullptr;  // reduction scratch
    double* red_out = nullptr;   // 4 doubles
    double* stage = nullptr;     // layout staging for host copies: two halves, so the
    size_t stage_bytes = 0;      // copy of one chunk overlaps the conversion of the other
    cudaStream_t copy_stream = nullptr;               // host copies of the staged chunks
    cudaEvent_t stage_ready[2] = {nullptr, nullptr};  // a half holds a copied / converted chunk
    cudaEvent_t stage_free[2] = {nullptr, nullptr};   // a half's chunk has been used
    long long device_bytes = 0;
    // state flags
    bool first_pending = false;  // next step reads the stored macroscopic fields
    bool macros_valid = false;   // rho,u,v,w(,T) arrays describe the current state
    long long itc = 0;
    bool initialised = false;
    std::string err;
    // moving particles
    PartParams pp{};
    PartDev pd{};
    std::vector<double> centers0;
};

namespace {

int fail(mglc_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_fail(mglc_ctx* c, cudaError_t e, const char* what) {
    return fail(c, MGLC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                                    \
    do {                                                  \
        cudaError_t e_ = (expr);                          \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

int dalloc(mglc_ctx* c, void** p, size_t bytes, const char* what) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(c, MGLC_ERR_NOMEM, "cudaMalloc(%zu bytes) for %s failed: %s", bytes, what,
                    cudaGetErrorString(e));
    }
    c->device_bytes += (long long)bytes;
    return MGLC_OK;
}

void release(mglc_ctx* c) {
    void* ptrs[] = {c->f[0], c->f[1], c->g[0], c->g[1], c->F, c->rho, c->u, c->v, c->w, c->T,
                    c->up, c->vp, c->wp, c->Tp, c->partials, c->red_out, c->stage};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    PartDev& d = c->pd;
    void* pptrs[] = {d.owner_cur, d.owner_new, d.xc, d.uc, d.om, d.xc_old, d.uc_old, d.om_old,
                     d.flink, d.tlink, d.corr, d.ftot, d.ttot, d.prep_sum, d.prep_cnt,
                     d.partials, d.n_fluid, d.rho_avg, d.status};
    for (void* p : pptrs)
        if (p) cudaFree(p);
    for (int h = 0; h < 2; h++) {
        if (c->stage_ready[h]) cudaEventDestroy(c->stage_ready[h]);
        if (c->stage_free[h]) cudaEventDestroy(c->stage_free[h]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

bool valid_form(int f) { return f >= FORM_FP64 && f <= FORM_BF16; }
// MGLC_FP16S / MGLC_BF16S: the 16-bit storage forms with stochastic rounding
bool sr_form(int f) { return f == MGLC_FP16S || f == MGLC_BF16S; }
int storage_of(int f) { return f == MGLC_FP16S ? FORM_FP16 : (f == MGLC_BF16S ? FORM_BF16 : f); }

// FP16 deviations are scaled so that typical |f - w rho0| (1e-5 .. 1e-1)
// stays in the normal FP16 range
constexpr float FP16_SCALE = 256.0f;

int alloc_common(mglc_ctx* c, bool thermal) {
    const long long n = c->n;
    const size_t pb = form_bytes(c->form);
    int rc;
    for (int b = 0; b < (c->in_place ? 1 : 2); b++)
        if ((rc = dalloc(c, &c->f[b], (size_t)Q19 * n * pb, "populations f"))) return rc;
    if (thermal) {
        // temperature populations in the arithmetic type (FP64 or FP32)
        const size_t gb = c->form == FORM_FP64 ? 8 : 4;
        for (int b = 0; b < (c->in_place ? 1 : 2); b++)
            if ((rc = dalloc(c, &c->g[b], (size_t)Q7 * n * gb, "populations g"))) return rc;
        const size_t cb = c->form == FORM_FP64 ? 8 : 4;
        if ((rc = dalloc(c, &c->F, 3 * n * cb, "carried force"))) return rc;
        CK(cudaMemsetAsync(c->F, 0, 3 * n * cb, c->stream), "memset F");
    }
    double** fields[] = {&c->rho, &c->u, &c->v, &c->w, &c->up, &c->vp, &c->wp};
    for (double** fp : fields)
        if ((rc = dalloc(c, (void**)fp, n * sizeof(double), "macroscopic field"))) return rc;
    if (thermal) {
        if ((rc = dalloc(c, (void**)&c->T, n * sizeof(double), "temperature"))) return rc;
        if ((rc = dalloc(c, (void**)&c->Tp, n * sizeof(double), "temperature"))) return rc;
    }
    if ((rc = dalloc(c, (void**)&c->partials, (size_t)reduce_blocks(n) * 4 * sizeof(double),
                     "reduction scratch")))
        return rc;
    if ((rc = dalloc(c, (void**)&c->red_out, 4 * sizeof(double), "reduction result"))) return rc;
    return MGLC_OK;
}

int create_stream(mglc_ctx* c) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamCreate");
    c->own_stream = true;
    return MGLC_OK;
}

int ensure_stage(mglc_ctx* c, size_t want) {
    if (!c->copy_stream) {
        CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "copy stream");
        for (int h = 0; h < 2; h++) {
            CK(cudaEventCreateWithFlags(&c->stage_ready[h], cudaEventDisableTiming), "stage event");
            CK(cudaEventCreateWithFlags(&c->stage_free[h], cudaEventDisableTiming), "stage event");
        }
    }
    if (c->stage_bytes >= want) return MGLC_OK;
    if (c->stage) {
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        CK(cudaStreamSynchronize(c->copy_stream), "synchronize");
        cudaFree(c->stage);
        c->device_bytes -= (long long)c->stage_bytes;
        c->stage = nullptr;
        c->stage_bytes = 0;
    }
    int rc = dalloc(c, (void**)&c->stage, want, "layout staging");
    if (rc == MGLC_OK) c->stage_bytes = want;
    return rc;
}

// cells per staged chunk: whole x-y planes, about 128 MB of FP64 AoS data
long long chunk_cells(const mglc_ctx* c, int Q) {
    const long long plane = (long long)c->geom.nx * c->geom.ny;
    long long kc = (128ll << 20) / ((long long)Q * 8 * plane);
    if (kc < 1) kc = 1;
    if (kc > c->geom.nz) kc = c->geom.nz;
    return kc * plane;
}

// storage form of a population set: f in the context's form, g in FP64/FP32
int pop_form(const mglc_ctx* c, int Q) {
    if (Q == Q19) return c->form;
    return c->form == FORM_FP64 ? FORM_FP64 : FORM_FP32;
}

// Host AoS populations -> device SoA form, through the two staging halves:
// the copy of chunk n (copy stream) overlaps the conversion of chunk n - 1
// (context stream); events order each half's copy after its previous
// conversion and each conversion after its copy.
int upload_pops(mglc_ctx* c, int Q, const double* host, void* dev, bool shifted) {
    const long long cc = chunk_cells(c, Q);
    int rc = ensure_stage(c, 2 * (size_t)cc * Q * sizeof(double));
    if (rc) return rc;
    // the copy stream starts after everything already queued on the context's stream
    CK(cudaEventRecord(c->stage_free[0], c->stream), "event");
    CK(cudaEventRecord(c->stage_free[1], c->stream), "event");
    int n = 0;
    for (long long c0 = 0; c0 < c->n; c0 += cc, n++) {
        const int h = n & 1;
        double* half = c->stage + (size_t)h * cc * Q;
        long long nc = std::min(cc, c->n - c0);
        CK(cudaStreamWaitEvent(c->copy_stream, c->stage_free[h], 0), "wait");
        CK(cudaMemcpyAsync(half, host + (size_t)c0 * Q, (size_t)nc * Q * sizeof(double),
                           cudaMemcpyHostToDevice, c->copy_stream),
           "copy populations to device");
        CK(cudaEventRecord(c->stage_ready[h], c->copy_stream), "event");
        CK(cudaStreamWaitEvent(c->stream, c->stage_ready[h], 0), "wait");
        CK(launch_aos_to_soa(pop_form(c, Q), Q, c->geom, c0, nc, half, dev, c->rho0,
                             Q == Q19 ? c->scale : 1.0f, shifted, c->stream),
           "aos_to_soa");
        CK(cudaEventRecord(c->stage_free[h], c->stream), "event");
    }
    // the host array may be reused once this returns: wait for its copies (the
    // last conversions stay queued on the context's stream)
    CK(cudaStreamSynchronize(c->copy_stream), "synchronize");
    return MGLC_OK;
}

// Device SoA form -> host AoS, the reverse pipeline: the conversion of chunk
// n (context stream) overlaps the copy of chunk n - 1 (copy stream).
int download_pops(mglc_ctx* c, int Q, const void* dev, double* host, bool shifted) {
    const long long cc = chunk_cells(c, Q);
    int rc = ensure_stage(c, 2 * (size_t)cc * Q * sizeof(double));
    if (rc) return rc;
    CK(cudaEventRecord(c->stage_free[0], c->copy_stream), "event");
    CK(cudaEventRecord(c->stage_free[1], c->copy_stream), "event");
    int n = 0;
    for (long long c0 = 0; c0 < c->n; c0 += cc, n++) {
        const int h = n & 1;
        double* half = c->stage + (size_t)h * cc * Q;
        long long nc = std::min(cc, c->n - c0);
        CK(cudaStreamWaitEvent(c->stream, c->stage_free[h], 0), "wait");
        CK(launch_soa_to_aos(pop_form(c, Q), Q, c->geom, c0, nc, dev, half, c->rho0,
                             Q == Q19 ? c->inv_scale : 1.0f, shifted, c->stream),
           "soa_to_aos");
        CK(cudaEventRecord(c->stage_ready[h], c->stream), "event");
        CK(cudaStreamWaitEvent(c->copy_stream, c->stage_ready[h], 0), "wait");
        CK(cudaMemcpyAsync(host + (size_t)c0 * Q, half, (size_t)nc * Q * sizeof(double),
                           cudaMemcpyDeviceToHost, c->copy_stream),
           "copy populations to host");
        CK(cudaEventRecord(c->stage_free[h], c->copy_stream), "event");
    }
    CK(cudaStreamSynchronize(c->copy_stream), "synchronize");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MGLC_OK;
}

bool thermal(const mglc_ctx* c) { return c->kind == MGLC_KIND_THERMAL; }

// in place: restore the post-stream layout after an even step (pairwise swap)
int natural_layout(mglc_ctx* c) {
    if (!c->in_place || !c->swapped) return MGLC_OK;
    CK(launch_aa_swap(c->form, c->geom, c->f[0], thermal(c) ? c->g[0] : nullptr, c->stream),
       "in-place layout swap");
    c->swapped = false;
    return MGLC_OK;
}

// bring rho,u,v,w(,T) up to date with the current populations
int refresh_macros(mglc_ctx* c) {
    if (c->macros_valid) return MGLC_OK;
    int rc0 = natural_layout(c);
    if (rc0) return rc0;
    if (c->kind == MGLC_KIND_PARTICLE) {
        CK(launch_particle_macro(c->form, c->first_pending, c->f[c->cur], c->pp, c->pd, c->rho,
                                 c->u, c->v, c->w, c->stream),
           "particle macro");
        c->macros_valid = true;
        return MGLC_OK;
    }
    CK(launch_macro(c->form, thermal(c), c->geom, c->f[c->cur], thermal(c) ? c->g[c->cur] : nullptr,
                    c->F, c->rho0, c->inv_scale, c->rho, c->u, c->v, c->w, c->T, c->stream),
       "macro");
    c->macros_valid = true;
    return MGLC_OK;
}

int check_geom(mglc_ctx* c, int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2)
        return fail(c, MGLC_ERR_INVALID, "grid %dx%dx%d: each axis needs at least 2 nodes", nx, ny, nz);
    if (ny > 65535 || nz > 65535)
        return fail(c, MGLC_ERR_INVALID, "grid %dx%dx%d: ny and nz are limited to 65535", nx, ny, nz);
    return MGLC_OK;
}

}  // namespace

extern "C" {

int mglc_lid_create(const mglc_lid_params* p, mglc_ctx** out) {
    if (!p || !out) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    int rc = check_geom(c, p->total_nx, p->total_ny, p->total_nz);
    if (!rc && !valid_form(p->precision) && p->precision != MGLC_FX64 && !sr_form(p->precision))
        rc = fail(c, MGLC_ERR_INVALID, "unknown precision %d", p->precision);
    if (!rc && !(p->reynolds > 0.0)) rc = fail(c, MGLC_ERR_INVALID, "reynolds must be positive");
    if (rc) {
        *out = c;  // caller reads the message, then destroys
        return rc;
    }
    c->kind = MGLC_KIND_LID;
    c->in_place = p->in_place != 0;
    c->fx64 = p->precision == MGLC_FX64;
    c->sr = sr_form(p->precision);
    c->form = c->fx64 ? FORM_FP64 : storage_of(p->precision);
    c->geom = {p->total_nx, p->total_ny, p->total_nz,
               (long long)p->total_nx * p->total_ny * p->total_nz};
    c->n = c->geom.plane;
    c->u0 = p->u0;
    c->rho0 = p->rho0;
    c->top_layer_u0 = p->top_layer_u0;
    // commondata.f90:9,42
    c->tauf = p->u0 * (double)p->total_nx / p->reynolds * 3.0 + 0.5;
    c->snu = 1.0 / c->tauf;
    c->sq = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
    if (c->form == FORM_FP16) {
        c->scale = FP16_SCALE;
        c->inv_scale = 1.0f / FP16_SCALE;
    }
    if ((rc = create_stream(c)) || (rc = alloc_common(c, false))) {
        *out = c;
        return rc;
    }
    *out = c;
    return MGLC_OK;
}

int mglc_thermal_create(const mglc_thermal_params* p, mglc_ctx** out) {
    if (!p || !out) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    int rc = check_geom(c, p->total_nx, p->total_ny, p->total_nz);
    if (!rc && !valid_form(p->precision) && !sr_form(p->precision) && p->precision != MGLC_FX64)
        rc = fail(c, MGLC_ERR_INVALID, "unknown precision %d", p->precision);
    if (!rc && !(p->rayleigh > 0.0 && p->prandtl > 0.0 && p->mach > 0.0))
        rc = fail(c, MGLC_ERR_INVALID, "rayleigh, prandtl and mach must be positive");
    if (rc) {
        *out = c;
        return rc;
    }
    c->kind = MGLC_KIND_THERMAL;
    c->in_place = p->in_place != 0;
    c->sr = sr_form(p->precision);
    c->fx64 = p->precision == MGLC_FX64;
    c->form = c->fx64 ? FORM_FP64 : storage_of(p->precision);
    c->geom = {p->total_nx, p->total_ny, p->total_nz,
               (long long)p->total_nx * p->total_ny * p->total_nz};
    c->n = c->geom.plane;
    // bouyancy3d_mpi.F90:34-54,80-81
    const int nz = p->total_nz;
    c->tauf = 0.5 + p->mach * (double)nz * std::sqrt(3.0 * p->prandtl / p->rayleigh);
    c->viscosity = (c->tauf - 0.5) / 3.0;
    c->diffusivity = c->viscosity / p->prandtl;
    c->omega_rot = p->ekman > 0.0 ? c->viscosity / 2.0 / p->ekman / (double)(nz * nz) : 0.0;
    c->para_a = 42.0 * std::sqrt(3.0) * c->diffusivity - 6.0;
    c->gbeta = p->rayleigh * c->viscosity * c->diffusivity / (double)nz / (double)(nz * nz);
    c->snu = 1.0 / c->tauf;
    c->sq = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
    c->qd = 3.0 - std::sqrt(3.0);
    c->qnu = 4.0 * std::sqrt(3.0) - 6.0;
    c->t_hot = p->t_hot;
    c->t_cold = p->t_cold;
    c->t_ref = p->t_ref;
    c->bc_y = p->bc_y_const_t ? 1 : 0;
    c->bc_z = p->bc_z_const_t ? 1 : 0;
    c->rho0 = 1.0;
    if (c->form == FORM_FP16) {
        c->scale = FP16_SCALE;
        c->inv_scale = 1.0f / FP16_SCALE;
    }
    if ((rc = create_stream(c)) || (rc = alloc_common(c, true))) {
        *out = c;
        return rc;
    }
    *out = c;
    return MGLC_OK;
}

void mglc_destroy(mglc_ctx* c) {
    if (!c) return;
    if (c->p2d) p2d_destroy(c->p2d);
    c->p2d = nullptr;
    if (c->l2d) l2d_destroy(c->l2d);
    c->l2d = nullptr;
    if (c->stream) cudaStreamSynchronize(c->stream);
    release(c);
    delete c;
}

const char* mglc_last_error(const mglc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mglc_set_stream(mglc_ctx* c, void* s) {
    if (!c) return MGLC_ERR_INVALID;
    if (c->p2d) return p2d_set_stream(c->p2d, (cudaStream_t)s);
    if (c->l2d) return l2d_set_stream(c->l2d, (cudaStream_t)s);
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (s) {
        c->stream = (cudaStream_t)s;
        c->own_stream = false;
        return MGLC_OK;
    }
    return create_stream(c);
}

int mglc_get_info(const mglc_ctx* c, mglc_info* o) {
    if (!c || !o) return MGLC_ERR_INVALID;
    std::memset(o, 0, sizeof *o);
    o->kind = c->kind;
    o->precision = c->fx64 ? MGLC_FX64
                 : c->sr ? (c->form == FORM_FP16 ? MGLC_FP16S : MGLC_BF16S) : c->form;
    o->nx = c->geom.nx;
    o->ny = c->geom.ny;
    o->nz = c->geom.nz;
    o->itc = c->itc;
    o->tauf = c->tauf;
    o->snu = c->snu;
    o->sq = c->sq;
    o->viscosity = (c->kind == MGLC_KIND_LID || c->kind == MGLC_KIND_LID2D) ? (c->tauf - 0.5) / 3.0
                                                                              : c->viscosity;
    o->diffusivity = c->diffusivity;
    o->para_a = c->para_a;
    o->gbeta = c->gbeta;
    o->omega_rot = c->omega_rot;
    const double pb = (double)form_bytes(c->form);
    if (c->p2d) {
        o->itc = p2d_itc(c->p2d);
        o->bytes_per_cell_step = 2.0 * 9 * 8.0 + 4.0;  // f pulled from fp, the mask read
        o->device_bytes = p2d_device_bytes(c->p2d);
        return MGLC_OK;
    }
    if (c->l2d) {
        o->itc = l2d_itc(c->l2d);
        o->bytes_per_cell_step = 2.0 * 9 * 8.0;
        o->device_bytes = l2d_device_bytes(c->l2d);
        return MGLC_OK;
    }
    if (c->kind == MGLC_KIND_LID) {
        o->bytes_per_cell_step = 2.0 * Q19 * pb;
    } else if (c->kind == MGLC_KIND_PARTICLE) {
        o->bytes_per_cell_step = 2.0 * Q19 * pb + 4.0;  // populations + owner mask read
    } else {
        const double cb = c->form == FORM_FP64 ? 8.0 : 4.0;
        // carried force: read and written once per step (F_z only without rotation);
        // g is kept in the arithmetic type
        const double carried = 2.0 * (c->omega_rot != 0.0 ? 3.0 : 1.0) * cb;
        o->bytes_per_cell_step = 2.0 * Q19 * pb + 2.0 * Q7 * cb + carried;
    }
    o->device_bytes = c->device_bytes;
    return MGLC_OK;
}

int particle_initial(mglc_ctx* c);

int mglc_initial(mglc_ctx* c) {
    Range nvtx_range("mglc_initial");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (c->kind == MGLC_KIND_PARTICLE) return particle_initial(c);
    if (c->p2d) {
        int rc = p2d_initial(c->p2d, c->err);
        c->initialised = rc == MGLC_OK;
        return rc;
    }
    if (c->l2d) {
        int rc = l2d_initial(c->l2d, c->err);
        c->initialised = rc == MGLC_OK;
        return rc;
    }
    const long long n = c->n;
    const Geom& g = c->geom;
    // rho = rho0, u = v = w = 0 (and T); lid top layer u = U0; hot/cold walls
    std::vector<double> hr(n, c->kind == MGLC_KIND_LID ? c->rho0 : 1.0), hu(n, 0.0), hz(n, 0.0);
    std::vector<double> ht;
    if (c->kind == MGLC_KIND_LID && c->top_layer_u0) {
        const long long top = (long long)g.nx * g.ny * (g.nz - 1);
        for (long long q = 0; q < (long long)g.nx * g.ny; q++) hu[top + q] = c->u0;
    }
    if (thermal(c)) {
        ht.assign(n, 0.0);
        if (c->bc_y)
            for (int k = 0; k < g.nz; k++)
                for (int i = 0; i < g.nx; i++) {
                    ht[i + (long long)g.nx * (0 + (long long)g.ny * k)] = c->t_hot;
                    ht[i + (long long)g.nx * ((g.ny - 1) + (long long)g.ny * k)] = c->t_cold;
                }
        if (c->bc_z)
            for (int j = 0; j < g.ny; j++)
                for (int i = 0; i < g.nx; i++) {
                    ht[i + (long long)g.nx * j] = c->t_hot;
                    ht[i + (long long)g.nx * (j + (long long)g.ny * (g.nz - 1))] = c->t_cold;
                }
    }
    const size_t b = n * sizeof(double);
    CK(cudaMemcpyAsync(c->rho, hr.data(), b, cudaMemcpyHostToDevice, c->stream), "copy rho");
    CK(cudaMemcpyAsync(c->u, hu.data(), b, cudaMemcpyHostToDevice, c->stream), "copy u");
    CK(cudaMemcpyAsync(c->v, hz.data(), b, cudaMemcpyHostToDevice, c->stream), "copy v");
    CK(cudaMemcpyAsync(c->w, hz.data(), b, cudaMemcpyHostToDevice, c->stream), "copy w");
    CK(cudaMemsetAsync(c->up, 0, b, c->stream), "zero up");
    CK(cudaMemsetAsync(c->vp, 0, b, c->stream), "zero vp");
    CK(cudaMemsetAsync(c->wp, 0, b, c->stream), "zero wp");
    if (thermal(c)) {
        CK(cudaMemcpyAsync(c->T, ht.data(), b, cudaMemcpyHostToDevice, c->stream), "copy T");
        CK(cudaMemsetAsync(c->Tp, 0, b, c->stream), "zero Tp");
    }
    CK(launch_equilibrium(c->form, thermal(c), g, c->rho, c->u, c->v, c->w, c->T, c->para_a,
                          c->rho0, c->scale, c->f[0], thermal(c) ? c->g[0] : nullptr, c->stream),
       "equilibrium");
    CK(cudaStreamSynchronize(c->stream), "synchronize");  // host vectors go out of scope
    c->cur = 0;
    c->swapped = false;
    c->itc = 0;
    c->first_pending = true;
    c->macros_valid = true;
    c->initialised = true;
    return MGLC_OK;
}

int mglc_load_state(mglc_ctx* c, const double* f, const double* g, const double* rho,
                    const double* u, const double* v, const double* w, const double* T) {
    Range nvtx_range("mglc_load_state");
    if (!c || !c->kind || !f) return c ? fail(c, MGLC_ERR_INVALID, "f is required") : MGLC_ERR_INVALID;
    if (c->p2d) return fail(c, MGLC_ERR_UNSUPPORTED, "2-D particle contexts start from mglc_initial");
    if (c->l2d) {
        int rc = l2d_load(c->l2d, f, rho, u, v, c->err);
        c->initialised = c->initialised || rc == MGLC_OK;
        return rc;
    }
    if (thermal(c) && !g) return fail(c, MGLC_ERR_INVALID, "thermal contexts need g");
    const bool shifted = c->form != FORM_FP64;
    int rc;
    c->swapped = false;  // the upload writes the post-stream layout
    if ((rc = upload_pops(c, Q19, f, c->f[0], shifted))) return rc;
    if (thermal(c) && (rc = upload_pops(c, Q7, g, c->g[0], false))) return rc;
    const size_t b = c->n * sizeof(double);
    const bool any = rho || u || v || w || T;
    if (any) {
        if (!(u && v && w) || (thermal(c) && !T))
            return fail(c, MGLC_ERR_INVALID, "u, v, w (and T) must be given together");
        if (rho) {
            CK(cudaMemcpyAsync(c->rho, rho, b, cudaMemcpyHostToDevice, c->stream), "copy rho");
        } else {
            // reference reload path keeps rho = 1 (bouyancy3d_mpi.F90:556,598-611)
            std::vector<double> ones(c->n, c->rho0);
            CK(cudaMemcpyAsync(c->rho, ones.data(), b, cudaMemcpyHostToDevice, c->stream), "copy rho");
            CK(cudaStreamSynchronize(c->stream), "synchronize");
        }
        CK(cudaMemcpyAsync(c->u, u, b, cudaMemcpyHostToDevice, c->stream), "copy u");
        CK(cudaMemcpyAsync(c->v, v, b, cudaMemcpyHostToDevice, c->stream), "copy v");
        CK(cudaMemcpyAsync(c->w, w, b, cudaMemcpyHostToDevice, c->stream), "copy w");
        if (thermal(c)) CK(cudaMemcpyAsync(c->T, T, b, cudaMemcpyHostToDevice, c->stream), "copy T");
        c->macros_valid = true;
    } else {
        if (thermal(c)) {
            const size_t cb = c->form == FORM_FP64 ? 8 : 4;
            CK(cudaMemsetAsync(c->F, 0, 3 * c->n * cb, c->stream), "zero F");
        }
        c->cur = 0;
        c->macros_valid = false;
        if ((rc = refresh_macros(c))) return rc;
    }
    CK(cudaMemsetAsync(c->up, 0, b, c->stream), "zero up");
    CK(cudaMemsetAsync(c->vp, 0, b, c->stream), "zero vp");
    CK(cudaMemsetAsync(c->wp, 0, b, c->stream), "zero wp");
    if (thermal(c)) CK(cudaMemsetAsync(c->Tp, 0, b, c->stream), "zero Tp");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    c->cur = 0;
    c->itc = 0;
    c->first_pending = true;
    c->initialised = true;
    return MGLC_OK;
}

int mglc_get_f(mglc_ctx* c, double* f, double* g) {
    Range nvtx_range("mglc_get_f");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->p2d) return f ? p2d_get_f(c->p2d, f, c->err) : MGLC_OK;
    if (c->l2d) return f ? l2d_get_f(c->l2d, f, c->err) : MGLC_OK;
    const bool shifted = c->form != FORM_FP64;
    int rc;
    if ((rc = natural_layout(c))) return rc;
    if (f && (rc = download_pops(c, Q19, c->f[c->cur], f, shifted))) return rc;
    if (g && thermal(c) && (rc = download_pops(c, Q7, c->g[c->cur], g, false))) return rc;
    return MGLC_OK;
}

int mglc_step(mglc_ctx* c, int nsteps) {
    Range nvtx_range("mglc_step");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (nsteps < 0) return fail(c, MGLC_ERR_INVALID, "nsteps must be >= 0");
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->p2d) return p2d_step(c->p2d, nsteps, c->err);
    if (c->l2d) return l2d_step(c->l2d, nsteps, c->err);
    if (c->kind == MGLC_KIND_PARTICLE) {
        for (int s = 0; s < nsteps; s++) {
            const int nxt = c->cur ^ 1;
            cudaError_t e = launch_particle_step(c->form, c->first_pending, c->f[c->cur],
                                                 c->f[nxt], c->pp, c->pd, c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "particle step launch");
            std::swap(c->pd.owner_cur, c->pd.owner_new);
            c->cur = nxt;
            c->first_pending = false;
            c->macros_valid = false;
            c->itc++;
        }
        // particle failures (overlap, wall penetration, ...) are reported here
        int st[3] = {0, 0, 0};
        CK(cudaMemcpyAsync(st, c->pd.status, sizeof st, cudaMemcpyDeviceToHost, c->stream),
           "read particle status");
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        if (st[0]) {
            static const char* what[] = {"", "no particle owns a solid boundary node",
                                         "interpolation fraction q outside [0,1]",
                                         "particle-particle interpenetration",
                                         "particle penetrates a wall",
                                         "no refill direction for a node leaving a particle",
                                         "too many nodes left one particle in one step",
                                         "particle state diverged (not finite, or a centre moved "
                                         "half the periodic length or more in one step)"};
            return fail(c, MGLC_ERR_PARTICLE, "%s (particle %d, other %d); the state is frozen at that step",
                        what[st[0] < 8 ? st[0] : 0], st[1], st[2]);
        }
        return MGLC_OK;
    }
    for (int s = 0; s < nsteps; s++) {
        const int nxt = c->cur ^ 1;
        cudaError_t e;
        if (c->kind == MGLC_KIND_LID) {
            LidStepArgs a;
            a.g = c->geom;
            a.cd = make_mrt_coef(c->snu, c->sq);
            a.u0 = c->u0;
            a.rho0 = c->rho0;
            a.scale = c->scale;
            a.inv_scale = c->inv_scale;
            a.seed = (unsigned)c->itc;
            a.sr = c->sr ? 1 : 0;
            a.rho = c->rho; a.u = c->u; a.v = c->v; a.w = c->w;
            if (c->in_place) {
                e = launch_lid_step_aa(c->fx64 ? FORM_FX64 : c->form, c->first_pending, c->swapped,
                                       c->f[0], a, c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "step kernel launch");
                c->swapped = !c->swapped;
                c->first_pending = false;
                c->macros_valid = false;
                c->itc++;
                continue;
            }
            e = launch_lid_step(c->fx64 ? FORM_FX64 : c->form, c->first_pending, c->f[c->cur],
                                c->f[nxt], a, c->stream);
        } else {
            ThermalStepArgs a;
            a.g = c->geom;
            a.cd = make_mrt_coef(c->snu, c->sq);
            a.gbeta = c->gbeta; a.omega_rot = c->omega_rot; a.t_ref = c->t_ref;
            a.para_a = c->para_a; a.qd = c->qd; a.qnu = c->qnu;
            a.t_hot = c->t_hot; a.t_cold = c->t_cold; a.rho0 = c->rho0;
            a.bc_y = c->bc_y; a.bc_z = c->bc_z;
            a.scale = c->scale; a.inv_scale = c->inv_scale;
            a.seed = (unsigned)c->itc;
            a.sr = c->sr ? 1 : 0;
            a.rho = c->rho; a.u = c->u; a.v = c->v; a.w = c->w; a.T = c->T;
            if (c->in_place) {
                e = launch_thermal_step_aa(c->fx64 ? FORM_FX64 : c->form, c->first_pending,
                                           c->swapped, c->f[0], c->g[0], c->F, a, c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "step kernel launch");
                c->swapped = !c->swapped;
                c->first_pending = false;
                c->macros_valid = false;
                c->itc++;
                continue;
            }
            e = launch_thermal_step(c->fx64 ? FORM_FX64 : c->form, c->first_pending, c->f[c->cur], c->f[nxt], c->g[c->cur],
                                    c->g[nxt], c->F, a, c->stream);
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "step kernel launch");
        c->cur = nxt;
        c->first_pending = false;
        c->macros_valid = false;
        c->itc++;
    }
    return MGLC_OK;
}

int mglc_get_macros_device(mglc_ctx* c, double* rho, double* u, double* v, double* w, double* T) {
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (c->p2d) return fail(c, MGLC_ERR_UNSUPPORTED, "not available for 2-D particle contexts");
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->l2d) return l2d_get_macros_device(c->l2d, rho, u, v, w, c->err);
    int rc = refresh_macros(c);
    if (rc) return rc;
    const size_t b = c->n * sizeof(double);
    if (rho) CK(cudaMemcpyAsync(rho, c->rho, b, cudaMemcpyDeviceToDevice, c->stream), "copy rho");
    if (u) CK(cudaMemcpyAsync(u, c->u, b, cudaMemcpyDeviceToDevice, c->stream), "copy u");
    if (v) CK(cudaMemcpyAsync(v, c->v, b, cudaMemcpyDeviceToDevice, c->stream), "copy v");
    if (w) CK(cudaMemcpyAsync(w, c->w, b, cudaMemcpyDeviceToDevice, c->stream), "copy w");
    if (T && thermal(c)) CK(cudaMemcpyAsync(T, c->T, b, cudaMemcpyDeviceToDevice, c->stream), "copy T");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MGLC_OK;
}

int mglc_get_macros(mglc_ctx* c, double* rho, double* u, double* v, double* w, double* T) {
    Range nvtx_range("mglc_get_macros");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->p2d) return p2d_get_macros(c->p2d, rho, u, v, w, c->err);
    if (c->l2d) return l2d_get_macros(c->l2d, rho, u, v, w, c->err);
    int rc = refresh_macros(c);
    if (rc) return rc;
    const size_t b = c->n * sizeof(double);
    if (rho) CK(cudaMemcpyAsync(rho, c->rho, b, cudaMemcpyDeviceToHost, c->stream), "copy rho");
    if (u) CK(cudaMemcpyAsync(u, c->u, b, cudaMemcpyDeviceToHost, c->stream), "copy u");
    if (v) CK(cudaMemcpyAsync(v, c->v, b, cudaMemcpyDeviceToHost, c->stream), "copy v");
    if (w) CK(cudaMemcpyAsync(w, c->w, b, cudaMemcpyDeviceToHost, c->stream), "copy w");
    if (T && thermal(c)) CK(cudaMemcpyAsync(T, c->T, b, cudaMemcpyDeviceToHost, c->stream), "copy T");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MGLC_OK;
}

int mglc_check(mglc_ctx* c, double* error_u, double* error_t) {
    Range nvtx_range("mglc_check");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (c->p2d) return fail(c, MGLC_ERR_UNSUPPORTED, "not available for 2-D particle contexts");
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->l2d) {
        double eu = 0.0;
        int rc = l2d_check(c->l2d, &eu, c->err);
        if (rc) return rc;
        if (error_u) *error_u = eu;
        if (error_t) *error_t = 0.0;
        if (!std::isfinite(eu))
            return fail(c, MGLC_ERR_NUMERIC, "non-finite velocity field at step %lld",
                        l2d_itc(c->l2d));
        return MGLC_OK;
    }
    int rc = refresh_macros(c);
    if (rc) return rc;
    CK(launch_residual(c->n, c->u, c->v, c->w, thermal(c) ? c->T : nullptr, c->up, c->vp, c->wp,
                       c->Tp, thermal(c), c->partials, c->red_out, c->stream),
       "residual");
    double e[4];
    CK(cudaMemcpyAsync(e, c->red_out, sizeof e, cudaMemcpyDeviceToHost, c->stream), "copy residual");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    const double eu = std::sqrt(e[0]) / std::sqrt(e[1]);
    if (error_u) *error_u = eu;
    if (error_t) *error_t = thermal(c) ? e[2] / e[3] : 0.0;
    if (!std::isfinite(e[0]) || !std::isfinite(e[1]))
        return fail(c, MGLC_ERR_NUMERIC, "non-finite velocity field at step %lld", c->itc);
    return MGLC_OK;
}

int mglc_totals(mglc_ctx* c, double* mass, double* energy, double* heat) {
    Range nvtx_range("mglc_totals");
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    if (c->p2d) return fail(c, MGLC_ERR_UNSUPPORTED, "not available for 2-D particle contexts");
    if (c->l2d) {  // host sums of the 2-D fields
        mglc_info in;
        mglc_get_info(c, &in);
        const size_t n = (size_t)in.nx * in.ny;
        std::vector<double> r(n), u(n), v(n);
        int rc = l2d_get_macros(c->l2d, r.data(), u.data(), v.data(), nullptr, c->err);
        if (rc) return rc;
        double m = 0.0, e = 0.0;
        for (size_t q = 0; q < n; q++) {
            m += r[q];
            e += 0.5 * r[q] * (u[q] * u[q] + v[q] * v[q]);
        }
        if (mass) *mass = m;
        if (energy) *energy = e;
        if (heat) *heat = 0.0;
        if (!std::isfinite(m) || !std::isfinite(e))
            return fail(c, MGLC_ERR_NUMERIC, "non-finite totals at step %lld", l2d_itc(c->l2d));
        return MGLC_OK;
    }
    int rc = refresh_macros(c);
    if (rc) return rc;
    CK(launch_totals(c->n, c->rho, c->u, c->v, c->w, thermal(c) ? c->T : nullptr, c->partials,
                     c->red_out, c->stream),
       "totals");
    double e[3];
    CK(cudaMemcpyAsync(e, c->red_out, sizeof e, cudaMemcpyDeviceToHost, c->stream), "copy totals");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (mass) *mass = e[0];
    if (energy) *energy = e[1];
    if (heat) *heat = e[2];
    if (!std::isfinite(e[0]) || !std::isfinite(e[1]))
        return fail(c, MGLC_ERR_NUMERIC, "non-finite totals at step %lld", c->itc);
    return MGLC_OK;
}

int mglc_nusselt(mglc_ctx* c, double* nu_vol, double* re_vol, double* nu_hot, double* nu_cold) {
    if (!c || !c->kind) return MGLC_ERR_INVALID;
    if (!thermal(c)) return fail(c, MGLC_ERR_STATE, "mglc_nusselt needs a thermal context");
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial or mglc_load_state first");
    int rc = refresh_macros(c);
    if (rc) return rc;
    const int axis = c->bc_y ? 1 : (c->bc_z ? 2 : 0);
    CK(launch_thermal_stats(c->geom, c->u, c->v, c->w, c->T, axis, c->partials, c->red_out,
                            c->stream),
       "thermal statistics");
    double e[4];
    CK(cudaMemcpyAsync(e, c->red_out, sizeof e, cudaMemcpyDeviceToHost, c->stream), "copy stats");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    const Geom& g = c->geom;
    const double ncell = (double)g.nx * g.ny * g.nz;
    // RaNu.F90:23,47
    if (nu_vol) *nu_vol = e[0] / ncell * (double)g.nz / c->diffusivity + 1.0;
    if (re_vol) *re_vol = std::sqrt(e[1] / ncell) * (double)g.nz / c->viscosity;
    const double dT = c->t_hot - c->t_cold;
    double L = 0.0, nwall = 0.0;
    if (axis == 1) { L = g.ny; nwall = (double)g.nx * g.nz; }
    if (axis == 2) { L = g.nz; nwall = (double)g.nx * g.ny; }
    // dT/dn at the hot wall = (9T1 - T2 - 8Th)/3, heat leaves the hot wall: Nu = -L/dT * dT/dn
    if (nu_hot) *nu_hot = axis ? -L / dT * ((e[2] / nwall - 8.0 * c->t_hot) / 3.0) : 0.0;
    if (nu_cold) *nu_cold = axis ? L / dT * ((e[3] / nwall - 8.0 * c->t_cold) / 3.0) : 0.0;
    return MGLC_OK;
}

int mglc_particle_create(const mglc_particle_params* p, const double* centers, int np,
                         mglc_ctx** out) {
    if (!p || !out || (np > 0 && !centers)) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    *out = c;
    int rc = check_geom(c, p->total_nx, p->total_ny, p->total_nz);
    if (rc) return rc;
    if (p->precision != FORM_FP64 && p->precision != FORM_FP32)
        return fail(c, MGLC_ERR_INVALID, "particle flows support MGLC_FP64 and MGLC_FP32");
    if (!(p->tauf > 0.5)) return fail(c, MGLC_ERR_INVALID, "tauf must exceed 0.5");
    if (!(p->radius > 0.5)) return fail(c, MGLC_ERR_INVALID, "radius must exceed 0.5");
    if (np < 0 || np > 65536) return fail(c, MGLC_ERR_INVALID, "np must be in [0, 65536]");
    {   // the per-particle node boxes (2 ceil(R) + 6 wide) must not wrap onto themselves
        const int need = 2 * (int)std::ceil(p->radius) + 6;
        if (p->total_nx < need || p->total_ny < 8 || p->total_nz < 8)
            return fail(c, MGLC_ERR_INVALID, "grid %dx%dx%d too small for radius %g (nx >= %d, ny, nz >= 8)",
                        p->total_nx, p->total_ny, p->total_nz, p->radius, need);
    }
    if (!(p->threshold_wall > 0.0 && p->threshold_particle > 0.0))
        return fail(c, MGLC_ERR_INVALID, "spring thresholds must be positive");
    for (int q = 0; q < np; q++) {
        const double* X = centers + 3 * q;
        if (!(X[0] >= 0.5 && X[0] <= p->total_nx + 0.5 && X[1] >= 0.5 && X[1] <= p->total_ny + 0.5 &&
              X[2] >= 0.5 && X[2] <= p->total_nz + 0.5))
            return fail(c, MGLC_ERR_INVALID, "centre of particle %d lies outside the domain", q);
    }
    c->kind = MGLC_KIND_PARTICLE;
    c->form = p->precision;
    c->geom = {p->total_nx, p->total_ny, p->total_nz,
               (long long)p->total_nx * p->total_ny * p->total_nz};
    c->n = c->geom.plane;
    c->rho0 = p->rho0;
    c->tauf = p->tauf;
    // case4 commondata.F90:33-34
    c->snu = 1.0 / p->tauf;
    c->sq = 8.0 * (2.0 * p->tauf - 1.0) / (8.0 * p->tauf - 1.0);
    PartParams& pp = c->pp;
    pp.nx = p->total_nx; pp.ny = p->total_ny; pp.nz = p->total_nz;
    pp.periodic_x = p->periodic_x ? 1 : 0;
    pp.np = np;
    pp.rho0 = p->rho0; pp.rho_solid = p->rho_solid; pp.radius = p->radius;
    pp.pi = 4.0 * std::atan(1.0);
    for (int q = 0; q < 3; q++) {
        pp.gravity[q] = p->gravity[q];
        pp.body_force[q] = p->body_force[q];
    }
    pp.thr_wall = p->threshold_wall; pp.thr_part = p->threshold_particle;
    pp.scale_wall = p->spring_scale_wall; pp.scale_part = p->spring_scale_particle;
    pp.snu = c->snu; pp.sq = c->sq;
    c->centers0.assign(centers, centers + 3 * (size_t)np);
    if ((rc = create_stream(c))) return rc;
    const size_t pb = form_bytes(c->form), n = (size_t)c->n;
    for (int b = 0; b < 2; b++)
        if ((rc = dalloc(c, &c->f[b], Q19 * n * pb, "populations f"))) return rc;
    double** fields[] = {&c->rho, &c->u, &c->v, &c->w, &c->up, &c->vp, &c->wp};
    for (double** fp : fields)
        if ((rc = dalloc(c, (void**)fp, n * sizeof(double), "macroscopic field"))) return rc;
    if ((rc = dalloc(c, (void**)&c->partials, (size_t)reduce_blocks(c->n) * 4 * sizeof(double), "reduction scratch")))
        return rc;
    if ((rc = dalloc(c, (void**)&c->red_out, 4 * sizeof(double), "reduction result"))) return rc;
    PartDev& d = c->pd;
    if ((rc = dalloc(c, (void**)&d.owner_cur, n * sizeof(int), "owner mask"))) return rc;
    if ((rc = dalloc(c, (void**)&d.owner_new, n * sizeof(int), "owner mask"))) return rc;
    const size_t v3 = sizeof(double) * 3 * (size_t)(np > 0 ? np : 1);
    double** p3[] = {&d.xc, &d.uc, &d.om, &d.xc_old, &d.uc_old, &d.om_old, &d.ftot, &d.ttot};
    for (double** a : p3)
        if ((rc = dalloc(c, (void**)a, v3, "particle state"))) return rc;
    // per-particle, per-slab partial sums of the boundary-link kernel
    if ((rc = dalloc(c, (void**)&d.flink, PART_NSLAB * v3, "link sums"))) return rc;
    if ((rc = dalloc(c, (void**)&d.tlink, PART_NSLAB * v3, "link sums"))) return rc;
    if ((rc = dalloc(c, (void**)&d.corr, PART_NSLAB * v3 / 3, "link sums"))) return rc;
    if ((rc = dalloc(c, (void**)&d.prep_sum, v3 / 3, "particle sums"))) return rc;
    if ((rc = dalloc(c, (void**)&d.prep_cnt, sizeof(int) * (size_t)(np > 0 ? np : 1), "particle sums"))) return rc;
    d.nblocks = particle_bulk_blocks(pp);
    // bulk partials (2 per warp) and the 2 x 32 stage-two sums of the finish kernel
    if ((rc = dalloc(c, (void**)&d.partials, sizeof(double) * (2 * (size_t)d.nblocks + 64), "bulk partials"))) return rc;
    if ((rc = dalloc(c, (void**)&d.n_fluid, 2 * sizeof(long long), "fluid count"))) return rc;
    if ((rc = dalloc(c, (void**)&d.rho_avg, 4 * sizeof(double), "average density"))) return rc;
    if ((rc = dalloc(c, (void**)&d.status, 3 * sizeof(int), "particle status"))) return rc;
    return MGLC_OK;
}

int particle_initial(mglc_ctx* c) {
    PartDev& d = c->pd;
    const int np = c->pp.np;
    const size_t v3 = sizeof(double) * 3 * (size_t)(np > 0 ? np : 1);
    if (np > 0)
        CK(cudaMemcpyAsync(d.xc, c->centers0.data(), sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream),
           "copy centres");
    CK(cudaMemsetAsync(d.uc, 0, v3, c->stream), "zero velocities");
    CK(cudaMemsetAsync(d.om, 0, v3, c->stream), "zero rotation");
    CK(cudaMemsetAsync(d.ftot, 0, v3, c->stream), "zero forces");
    CK(cudaMemsetAsync(d.ttot, 0, v3, c->stream), "zero torques");
    CK(cudaMemsetAsync(d.status, 0, 3 * sizeof(int), c->stream), "zero status");
    CK(cudaMemsetAsync(d.rho_avg, 0, 4 * sizeof(double), c->stream), "zero average");
    const size_t b = c->n * sizeof(double);
    CK(cudaMemsetAsync(c->up, 0, b, c->stream), "zero up");
    CK(cudaMemsetAsync(c->vp, 0, b, c->stream), "zero vp");
    CK(cudaMemsetAsync(c->wp, 0, b, c->stream), "zero wp");
    CK(launch_particle_init(c->form, c->f[0], c->pp, d, c->stream), "particle initial");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    c->cur = 0;
    c->itc = 0;
    c->first_pending = true;
    c->macros_valid = false;
    c->initialised = true;
    return MGLC_OK;
}

int mglc_particle2d_create(const mglc_particle2d_params* p, const double* centers, int np,
                           mglc_ctx** out) {
    if (!p || !out || (np > 0 && !centers)) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    *out = c;
    if (p->total_nx < 8 || p->total_ny < 8) return fail(c, MGLC_ERR_INVALID, "the 2-D lattice needs nx, ny >= 8");
    if (np < 0 || np > 65536) return fail(c, MGLC_ERR_INVALID, "np must be in [0, 65536]");
    if (!(p->tauf > 0.5)) return fail(c, MGLC_ERR_INVALID, "tauf must exceed 0.5");
    if (!(p->radius > 0.5)) return fail(c, MGLC_ERR_INVALID, "radius must exceed 0.5");
    if (!(p->stiff_wall > 0.0 && p->stiff_particle > 0.0 && p->threshold_wall > 0.0 &&
          p->threshold_particle > 0.0))
        return fail(c, MGLC_ERR_INVALID, "spring stiffnesses and thresholds must be positive");
    for (int q = 0; q < np; q++) {
        const double x = centers[2 * q], y = centers[2 * q + 1];
        if (!(x - p->radius > 1.0 && y - p->radius > 1.0 && x + p->radius < p->total_nx &&
              y + p->radius < p->total_ny))
            return fail(c, MGLC_ERR_INVALID, "circle %d does not fit inside the walls", q);
    }
    P2Params pp{};
    pp.nx = p->total_nx; pp.ny = p->total_ny; pp.np = np;
    pp.q_bisection = p->q_bisection ? 1 : 0;
    pp.tauf = p->tauf; pp.rho0 = p->rho0; pp.rho_solid = p->rho_solid; pp.radius = p->radius;
    pp.gravity = p->gravity;
    pp.threshold_wall = p->threshold_wall; pp.stiff_wall = p->stiff_wall;
    pp.threshold_particle = p->threshold_particle; pp.stiff_particle = p->stiff_particle;
    // commondata.F90:33-34
    pp.snu = 1.0 / p->tauf;
    pp.sq = 8.0 * (2.0 * p->tauf - 1.0) / (8.0 * p->tauf - 1.0);
    pp.pi = 4.0 * std::atan(1.0);
    c->kind = MGLC_KIND_PARTICLE2D;
    c->form = FORM_FP64;
    c->geom = {p->total_nx, p->total_ny, 1, (long long)p->total_nx * p->total_ny};
    c->n = c->geom.plane;
    c->tauf = pp.tauf;
    c->snu = pp.snu;
    c->sq = pp.sq;
    return p2d_create(pp, centers, &c->p2d, c->err);
}

int mglc_shear2d_create(const mglc_shear2d_params* p, const double* centers, int np,
                        mglc_ctx** out) {
    if (!p || !out || (np > 0 && !centers)) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    *out = c;
    if (p->total_nx < 8 || p->total_ny < 8) return fail(c, MGLC_ERR_INVALID, "the 2-D lattice needs nx, ny >= 8");
    if (np < 0 || np > 65536) return fail(c, MGLC_ERR_INVALID, "np must be in [0, 65536]");
    if (!(p->tauf > 0.5)) return fail(c, MGLC_ERR_INVALID, "tauf must exceed 0.5");
    if (!(p->radius > 0.5)) return fail(c, MGLC_ERR_INVALID, "radius must exceed 0.5");
    for (int q = 0; q < np; q++) {
        const double x = centers[2 * q], y = centers[2 * q + 1];
        if (!(x - p->radius > 3.0 && x + p->radius < p->total_nx - 2.0 && y - p->radius > 1.0 &&
              y + p->radius < p->total_ny))
            return fail(c, MGLC_ERR_INVALID,
                        "circle %d must fit between the walls and clear the periodic boundary", q);
    }
    P2Params pp{};
    pp.nx = p->total_nx; pp.ny = p->total_ny; pp.np = np;
    pp.q_bisection = 1;  // case1 calls calQ (particle_bounceback.F90:59)
    pp.tauf = p->tauf; pp.rho0 = p->rho0; pp.rho_solid = p->rho_solid; pp.radius = p->radius;
    // commondata.F90:32
    pp.snu = 1.0 / p->tauf;
    pp.sq = 8.0 * (2.0 * p->tauf - 1.0) / (8.0 * p->tauf - 1.0);
    pp.pi = 4.0 * std::atan(1.0);
    pp.variant = P2_SHEAR;
    pp.moving_frame = p->moving_frame ? 1 : 0;
    pp.linear = p->linear ? 1 : 0;
    pp.u0 = p->u0;
    pp.uwall = p->uwall;
    c->kind = MGLC_KIND_PARTICLE2D;
    c->form = FORM_FP64;
    c->geom = {p->total_nx, p->total_ny, 1, (long long)p->total_nx * p->total_ny};
    c->n = c->geom.plane;
    c->tauf = pp.tauf;
    c->snu = pp.snu;
    c->sq = pp.sq;
    return p2d_create(pp, centers, &c->p2d, c->err);
}

int mglc_lid2d_create(const mglc_lid2d_params* p, mglc_ctx** out) {
    if (!p || !out) return MGLC_ERR_INVALID;
    *out = nullptr;
    mglc_ctx* c = new mglc_ctx();
    *out = c;
    if (p->total_nx < 2 || p->total_ny < 2 || (long long)p->total_nx * p->total_ny > (1LL << 31))
        return fail(c, MGLC_ERR_INVALID, "the 2-D lattice needs 2 <= nx, ny and nx*ny <= 2^31");
    if (p->precision != MGLC_FP64)
        return fail(c, MGLC_ERR_UNSUPPORTED, "the 2-D lid cavity is built for MGLC_FP64");
    if (!(p->reynolds > 0.0)) return fail(c, MGLC_ERR_INVALID, "reynolds must be positive");
    L2Params lp{};
    lp.nx = p->total_nx;
    lp.ny = p->total_ny;
    lp.u0 = p->u0;
    lp.rho0 = p->rho0;
    // commondata.f90:9,30
    lp.tauf = p->u0 * (double)p->total_nx / p->reynolds * 3.0 + 0.5;
    lp.snu = 1.0 / lp.tauf;
    lp.sq = 8.0 * (2.0 * lp.tauf - 1.0) / (8.0 * lp.tauf - 1.0);
    if (!(lp.tauf > 0.5)) return fail(c, MGLC_ERR_INVALID, "tauf must exceed 0.5");
    c->kind = MGLC_KIND_LID2D;
    c->form = FORM_FP64;
    c->geom = {p->total_nx, p->total_ny, 1, (long long)p->total_nx * p->total_ny};
    c->n = c->geom.plane;
    c->u0 = p->u0;
    c->rho0 = p->rho0;
    c->tauf = lp.tauf;
    c->snu = lp.snu;
    c->sq = lp.sq;
    return l2d_create(lp, &c->l2d, c->err);
}

int mglc_particle_state(mglc_ctx* c, double* xc, double* uc, double* omega, double* force,
                        double* torque) {
    if (c && c->p2d) return p2d_state(c->p2d, xc, uc, omega, force, torque, c->err);
    if (!c || c->kind != MGLC_KIND_PARTICLE)
        return c ? fail(c, MGLC_ERR_STATE, "mglc_particle_state needs a particle context") : MGLC_ERR_INVALID;
    const size_t b = sizeof(double) * 3 * (size_t)c->pp.np;
    if (b == 0) return MGLC_OK;
    if (xc) CK(cudaMemcpyAsync(xc, c->pd.xc, b, cudaMemcpyDeviceToHost, c->stream), "copy centres");
    if (uc) CK(cudaMemcpyAsync(uc, c->pd.uc, b, cudaMemcpyDeviceToHost, c->stream), "copy velocities");
    if (omega) CK(cudaMemcpyAsync(omega, c->pd.om, b, cudaMemcpyDeviceToHost, c->stream), "copy rotation");
    if (force) CK(cudaMemcpyAsync(force, c->pd.ftot, b, cudaMemcpyDeviceToHost, c->stream), "copy forces");
    if (torque) CK(cudaMemcpyAsync(torque, c->pd.ttot, b, cudaMemcpyDeviceToHost, c->stream), "copy torques");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MGLC_OK;
}

int mglc_get_mask(mglc_ctx* c, int* owner) {
    if (c && c->p2d && owner) {
        if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial first");
        return p2d_mask(c->p2d, owner, c->err);
    }
    if (!c || c->kind != MGLC_KIND_PARTICLE || !owner)
        return c ? fail(c, MGLC_ERR_STATE, "mglc_get_mask needs a particle context and a buffer") : MGLC_ERR_INVALID;
    if (!c->initialised) return fail(c, MGLC_ERR_STATE, "call mglc_initial first");
    CK(cudaMemcpyAsync(owner, c->pd.owner_cur, sizeof(int) * (size_t)c->n, cudaMemcpyDeviceToHost, c->stream),
       "copy mask");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MGLC_OK;
}

}  // extern "C"

#ifdef MGLC_BOUNDS_CHECK
// Bounds-checked builds only (no counterpart in the reference, not declared in
// mglc.h): out-of-range element indices counted by the step kernels of every
// translation unit since the library loaded on the current device.
extern "C" unsigned long long mglc_oob_hits_k_step();
extern "C" unsigned long long mglc_oob_hits_k_step_aa();
extern "C" unsigned long long mglc_oob_hits_k_serve();
extern "C" unsigned long long mglc_debug_bounds_hits() {
    return mglc_oob_hits_k_step() + mglc_oob_hits_k_step_aa() + mglc_oob_hits_k_serve();
}
#endif
