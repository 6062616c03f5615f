// serve.cu -- the solve server (continuous batching of cavity solves).
//
// Requests (lid-driven or heated cavities of uneven sizes and Re/Ra) arrive
// over time.  Each admitted request becomes a resident solve whose
// populations live in a device arena sized by an HBM budget; a request waits
// until a slot and enough arena memory are free (admission by footprint).
// Every iteration replays one CUDA graph: a memset of the queue counters,
// K launches of the persistent tile-queue step kernel (all active solves
// advance together), the residual kernel and a copy of the residuals to
// pinned host memory.  Between iterations solves retire -- when
// max|u - u_prev|/U over the last K steps drops below the tolerance, or at
// the step cap -- and waiting requests take their place.  The tile shape
// (threads per CTA, x-rows per tile, CTAs per SM) is chosen once by timing
// candidates on a synthetic mix.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mglc.h"
#include "serve.cuh"

using namespace mglc;

namespace {

// first-fit arena over one device allocation, 256-byte granules
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    void reset(char* b, size_t n) {
        base = b;
        size = n;
        used = peak = 0;
        free_.clear();
        free_[0] = n;
    }
    static size_t round(size_t n) { return (n + 255) & ~size_t(255); }
    bool alloc(size_t n, size_t* off) {
        n = round(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                const size_t rest = it->second - n, o2 = it->first + n;
                free_.erase(it);
                if (rest) free_[o2] = rest;
                used += n;
                peak = std::max(peak, used);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = round(n);
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Req {
    long long id = 0;
    mglc_request r{};
    int state = 0;  // 0 pending arrival, 1 waiting, 2 active, 3 retired
    int slot = -1;
    size_t off = 0, bytes = 0;
    long long steps = 0;
    double resid = 1e30;
    double admit_s = 0, finish_s = 0;
    int converged = 0;
    ServeSolve sv{};
    std::vector<float> fields;
};

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct mglc_server {
    mglc_server_params p{};
    cudaStream_t stream = nullptr;
    char* arena_mem = nullptr;
    Arena arena;
    ServeTable* tab_host = nullptr;  // pinned
    ServeTable* tab_dev = nullptr;
    unsigned* counters = nullptr;   // 2K + 24: per-step queue counters (iteration, autotuner)
    unsigned* resid_dev = nullptr;  // SERVE_MAX_ACTIVE
    unsigned* resid_host = nullptr; // pinned
    float* fields_dev = nullptr;    // staging for retired solves' fields
    size_t fields_bytes = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t done = nullptr;
    bool sr = false;  // stochastic rounding of the 16-bit stores
    bool in_place = false;  // AA pattern: one population buffer per solve
    cudaStream_t side = nullptr;        // heated-solve branch of the captured step
    cudaEvent_t fork = nullptr, join = nullptr;
    int block = 256, rows = 2, ctas_per_sm = 4, nsm = 152;
    bool tuned = false;
    std::vector<Req> reqs;
    std::vector<int> active;  // indices into reqs, in table order
    std::deque<int> waiting;
    double t0 = -1.0;
    mglc_server_stats stats{};
    std::string err;
};

namespace {

int sfail(mglc_server* s, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (s) s->err = buf;
    return code;
}
#define SCK(expr, what)                                                              \
    do {                                                                             \
        cudaError_t e_ = (expr);                                                     \
        if (e_ != cudaSuccess) return sfail(s, MGLC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
    } while (0)

size_t pop_bytes(const mglc_server* s) { return s->p.precision == MGLC_FP32 ? 4 : 2; }

// device footprint of a solve of n^3 cells
size_t footprint(const mglc_server* s, int kind, int n) {
    const size_t c = (size_t)n * n * n;
    const size_t nb = s->in_place ? 1 : 2;                          // buffers per population set
    size_t b = nb * 19 * c * pop_bytes(s) + 3 * c * 4 + 5 * 256;    // f, uprev
    if (kind == MGLC_KIND_THERMAL) b += nb * 7 * c * 4 + c * 4;     // g, F_z
    return b;
}

// constants of a request, as the one-solve contexts derive them
void fill_solve(const mglc_server* s, const mglc_request& r, ServeSolve* sv) {
    const int n = r.n;
    sv->kind = r.kind;
    sv->nx = sv->ny = sv->nz = n;
    sv->plane = (unsigned)((size_t)n * n * n);
    StepK<float>& K = sv->K;
    std::memset(&K, 0, sizeof K);
    K.nx = K.ny = K.nz = n;
    K.rho0 = 1.0f;
    const bool fp16 = s->p.precision == MGLC_FP16;
    K.sr = s->sr ? 1 : 0;
    K.scale = fp16 ? 256.0f : 1.0f;
    K.inv_scale = fp16 ? 1.0f / 256.0f : 1.0f;
    if (r.kind == MGLC_KIND_LID) {
        const double u0 = 0.1;
        const double tauf = u0 * (double)n / r.reynolds * 3.0 + 0.5;
        const double snu = 1.0 / tauf, sq = 8.0 * (2.0 * tauf - 1.0) / (8.0 * tauf - 1.0);
        K.c = cast_coef<float>(make_mrt_coef(snu, sq));
        K.u0 = (float)u0;
        sv->uref = (float)u0;
    } else {
        const double Pr = 0.71, Ma = 0.1;
        const double tauf = 0.5 + Ma * (double)n * std::sqrt(3.0 * Pr / r.rayleigh);
        const double nu = (tauf - 0.5) / 3.0, kappa = nu / Pr;
        const double para_a = 42.0 * std::sqrt(3.0) * kappa - 6.0;
        const double gbeta = r.rayleigh * nu * kappa / (double)n / (double)(n * n);
        const double snu = 1.0 / tauf, sq = 8.0 * (2.0 * tauf - 1.0) / (8.0 * tauf - 1.0);
        K.c = cast_coef<float>(make_mrt_coef(snu, sq));
        K.gbeta = (float)gbeta;
        K.omega_rot = 0.0f;
        K.t_ref = 0.0f;
        K.para_a = (float)para_a;
        K.qd = (float)(3.0 - std::sqrt(3.0));
        K.qnu = (float)(4.0 * std::sqrt(3.0) - 6.0);
        K.chot = (float)((6.0 + para_a) / 21.0 * 0.5);
        K.ccold = (float)((6.0 + para_a) / 21.0 * -0.5);
        K.bc_y = 1;
        K.bc_z = 0;
        sv->uref = (float)std::sqrt(gbeta * (double)n * 1.0);  // free-fall velocity, dT = 1
    }
}

// place a solve's buffers at arena offset off
void place(mglc_server* s, Req& q) {
    char* b = s->arena_mem + q.off;
    const size_t c = q.sv.plane, pb = pop_bytes(s);
    auto take = [&](size_t n) { char* p = b; b += Arena::round(n); return p; };
    q.sv.f[0] = take(19 * c * pb);
    q.sv.f[1] = s->in_place ? q.sv.f[0] : take(19 * c * pb);
    q.sv.uprev = (float*)take(3 * c * 4);
    if (q.sv.kind == MGLC_KIND_THERMAL) {
        q.sv.g[0] = (float*)take(7 * c * 4);
        q.sv.g[1] = s->in_place ? q.sv.g[0] : (float*)take(7 * c * 4);
        q.sv.F = (float*)take(c * 4);
    } else {
        q.sv.g[0] = q.sv.g[1] = nullptr;
        q.sv.F = nullptr;
    }
}

int tiles_of(const mglc_server* s, const ServeSolve& sv) { return (sv.ny * sv.nz + s->rows - 1) / s->rows; }

// rebuild the host table from the active list (lid solves first) and upload it
int upload_table(mglc_server* s) {
    ServeTable* t = s->tab_host;
    std::stable_sort(s->active.begin(), s->active.end(), [&](int a, int b) {
        return s->reqs[a].r.kind < s->reqs[b].r.kind;  // MGLC_KIND_LID (1) before THERMAL (2)
    });
    t->n_active = (int)s->active.size();
    t->rows_per_tile = s->rows;
    int tile = 0;
    t->lid_tiles = 0;
    for (int a = 0; a < t->n_active; a++) {
        Req& q = s->reqs[s->active[a]];
        q.slot = a;
        q.sv.tile0 = tile;
        q.sv.ntiles = tiles_of(s, q.sv);
        q.sv.step0 = (unsigned)q.steps;  // the device copy advances by K per iteration too
        tile += q.sv.ntiles;
        if (q.r.kind == MGLC_KIND_LID) t->lid_tiles = tile;
        t->s[a] = q.sv;
    }
    t->total_tiles = tile;
    const size_t bytes = offsetof(ServeTable, s) + sizeof(ServeSolve) * (size_t)std::max(1, t->n_active);
    SCK(cudaMemcpyAsync(s->tab_dev, t, bytes, cudaMemcpyHostToDevice, s->stream), "upload solve table");
    return MGLC_OK;
}

// one step of every resident solve as an iteration issues it: the heated
// kernel on the side stream beside the lid kernel, joined before the next step
cudaError_t issue_step(mglc_server* s, int k, unsigned* c_lid, unsigned* c_heat, int grid,
                       int blk) {
    const int sr = s->sr ? 1 : 0;
    cudaError_t e = cudaEventRecord(s->fork, s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->side, s->fork, 0);
    if (e == cudaSuccess)
        e = launch_serve_step(s->p.precision, sr, s->in_place ? 1 : 0, 1, s->tab_dev, k, c_heat, grid, blk, s->side);
    if (e == cudaSuccess)
        e = launch_serve_step(s->p.precision, sr, s->in_place ? 1 : 0, 0, s->tab_dev, k, c_lid, grid, blk, s->stream);
    if (e == cudaSuccess) e = cudaEventRecord(s->join, s->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->join, 0);
    return e;
}

int build_graph(mglc_server* s) {
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    const int K = s->p.steps_per_iteration;
    const int grid = s->nsm * s->ctas_per_sm;
    cudaGraph_t g;
    SCK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    // counters: [0, K) lid steps, [K, 2K) heated steps, 2K residual
    cudaError_t e = cudaMemsetAsync(s->counters, 0, sizeof(unsigned) * (2 * K + 1), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->resid_dev, 0, sizeof(unsigned) * SERVE_MAX_ACTIVE, s->stream);
    for (int k = 0; k < K && e == cudaSuccess; k++)
        e = issue_step(s, k, s->counters + k, s->counters + K + k, grid, s->block);
    if (e == cudaSuccess)
        e = launch_serve_resid(s->p.precision, s->tab_dev, s->counters + 2 * K, s->resid_dev, K, grid,
                               s->block, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->resid_host, s->resid_dev, sizeof(unsigned) * SERVE_MAX_ACTIVE,
                            cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        cudaGetLastError();
        return sfail(s, MGLC_ERR_CUDA, "graph capture failed: %s",
                     cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return sfail(s, MGLC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    return MGLC_OK;
}

// Choose threads per CTA, rows per tile and CTAs per SM by timing steps of a
// synthetic mix (one solve of each size, lid and heated alternating), issued
// as an iteration issues them (heated beside lid): per candidate two warm-up
// steps and eight timed ones, the best of two passes over all candidates.
// NVTX range of one serving iteration (a no-op unless a tool is attached)
struct IterRange {
    IterRange() { nvtxRangePushA("serve iteration"); }
    ~IterRange() { nvtxRangePop(); }
};

int autotune(mglc_server* s) {
    static const int sizes[] = {32, 48, 64, 96, 128};
    std::vector<Req> mix;
    size_t need = 0;
    for (int q = 0; q < 5; q++) {
        Req r;
        r.r.kind = (q % 2) ? MGLC_KIND_THERMAL : MGLC_KIND_LID;
        r.r.n = sizes[q];
        r.r.reynolds = 400.0;
        r.r.rayleigh = 1e4;
        fill_solve(s, r.r, &r.sv);
        r.bytes = footprint(s, r.r.kind, r.r.n);
        need += Arena::round(r.bytes);
        mix.push_back(r);
    }
    if (need > s->arena.size / 2) {  // budget too small to probe: keep the defaults
        s->tuned = true;
        return MGLC_OK;
    }
    for (auto& r : mix) {
        if (!s->arena.alloc(r.bytes, &r.off)) break;
        place(s, r);
        SCK(launch_serve_init(s->p.precision, r.sv, 0.5, -0.5, s->stream), "init probe");
    }
    const std::vector<Req> saved_reqs = s->reqs;
    const std::vector<int> saved_active = s->active;
    s->reqs = mix;
    s->active.clear();
    for (size_t q = 0; q < mix.size(); q++) s->active.push_back((int)q);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    int bb = s->block, br = s->rows, bc = s->ctas_per_sm;
    const int blocks[] = {128, 256};
    const int rowsv[] = {1, 2, 4, 8};
    const int ctas[] = {2, 4, 8};
    constexpr int kWarm = 2, kTimed = 8, kSteps = kWarm + kTimed;  // counters: 2 * kSteps
    for (int pass = 0; pass < 2; pass++)
        for (int blk : blocks)
            for (int rw : rowsv)
                for (int cp : ctas) {
                    s->block = blk;
                    s->rows = rw;
                    s->ctas_per_sm = cp;
                    if (upload_table(s)) break;
                    cudaStreamSynchronize(s->stream);  // the pinned table is rewritten next round
                    const int grid = s->nsm * cp;
                    cudaMemsetAsync(s->counters, 0, sizeof(unsigned) * 2 * kSteps, s->stream);
                    for (int k = 0; k < kSteps; k++) {
                        if (k == kWarm) cudaEventRecord(a, s->stream);
                        issue_step(s, k, s->counters + k, s->counters + kSteps + k, grid, blk);
                    }
                    cudaEventRecord(b, s->stream);
                    cudaEventSynchronize(b);
                    float ms = 0;
                    cudaEventElapsedTime(&ms, a, b);
                    if (ms < best) {
                        best = ms;
                        bb = blk;
                        br = rw;
                        bc = cp;
                    }
                }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    SCK(cudaStreamSynchronize(s->stream), "autotune");
    for (auto& r : mix) s->arena.release(r.off, r.bytes);
    s->arena.peak = 0;
    s->reqs = saved_reqs;
    s->active = saved_active;
    s->block = bb;
    s->rows = br;
    s->ctas_per_sm = bc;
    s->tuned = true;
    return MGLC_OK;
}

int admit(mglc_server* s, double t) {
    bool changed = false;
    while (!s->waiting.empty() && (int)s->active.size() < std::min(s->p.max_active, SERVE_MAX_ACTIVE)) {
        Req& q = s->reqs[s->waiting.front()];
        q.bytes = footprint(s, q.r.kind, q.r.n);
        if (!s->arena.alloc(q.bytes, &q.off)) break;  // wait for memory (FIFO)
        fill_solve(s, q.r, &q.sv);
        place(s, q);
        SCK(launch_serve_init(s->p.precision, q.sv, 0.5, -0.5, s->stream), "init solve");
        q.state = 2;
        q.admit_s = t;
        s->active.push_back(s->waiting.front());
        s->waiting.pop_front();
        changed = true;
    }
    s->stats.peak_active = std::max(s->stats.peak_active, (int)s->active.size());
    s->stats.peak_device_bytes = std::max<long long>(s->stats.peak_device_bytes, (long long)s->arena.peak);
    if (changed) return upload_table(s);
    return MGLC_OK;
}

}  // namespace

extern "C" {

int mglc_server_create(const mglc_server_params* p, mglc_server** out) {
    if (!p || !out) return MGLC_ERR_INVALID;
    mglc_server* s = new mglc_server();
    *out = s;
    s->p = *p;
    if (p->precision != MGLC_FP16 && p->precision != MGLC_FP32 && p->precision != MGLC_BF16 &&
        p->precision != MGLC_FP16S && p->precision != MGLC_BF16S)
        return sfail(s, MGLC_ERR_INVALID, "the server stores populations as FP16, BF16 or FP32");
    // FP16S / BF16S: 16-bit storage with stochastic rounding; from here on the
    // precision field holds the storage form
    s->sr = p->precision == MGLC_FP16S || p->precision == MGLC_BF16S;
    s->in_place = p->in_place != 0;
    if (p->precision == MGLC_FP16S) s->p.precision = MGLC_FP16;
    if (p->precision == MGLC_BF16S) s->p.precision = MGLC_BF16;
    if (p->steps_per_iteration < 2 || p->steps_per_iteration % 2)
        return sfail(s, MGLC_ERR_INVALID, "steps_per_iteration must be even and >= 2");
    if (p->max_active < 1) return sfail(s, MGLC_ERR_INVALID, "max_active must be >= 1");
    if (p->hbm_budget_bytes < (1ll << 24)) return sfail(s, MGLC_ERR_INVALID, "hbm_budget_bytes below 16 MiB");
    int dev = 0;
    SCK(cudaGetDevice(&dev), "cudaGetDevice");
    SCK(cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
    SCK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream");
    cudaError_t e = cudaMalloc((void**)&s->arena_mem, (size_t)p->hbm_budget_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return sfail(s, MGLC_ERR_NOMEM, "arena of %lld bytes: %s", p->hbm_budget_bytes, cudaGetErrorString(e));
    }
    s->arena.reset(s->arena_mem, (size_t)p->hbm_budget_bytes);
    SCK(cudaMallocHost((void**)&s->tab_host, sizeof(ServeTable)), "pinned table");
    std::memset(s->tab_host, 0, sizeof(ServeTable));
    SCK(cudaMalloc((void**)&s->tab_dev, sizeof(ServeTable)), "device table");
    SCK(cudaMalloc((void**)&s->counters, sizeof(unsigned) * (2 * p->steps_per_iteration + 24)),
        "counters");
    SCK(cudaMalloc((void**)&s->resid_dev, sizeof(unsigned) * SERVE_MAX_ACTIVE), "residuals");
    SCK(cudaMallocHost((void**)&s->resid_host, sizeof(unsigned) * SERVE_MAX_ACTIVE), "pinned residuals");
    SCK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming), "event");
    SCK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "side stream");
    SCK(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming), "fork event");
    SCK(cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming), "join event");
    return MGLC_OK;
}

void mglc_server_destroy(mglc_server* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->done) cudaEventDestroy(s->done);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->join) cudaEventDestroy(s->join);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->arena_mem) cudaFree(s->arena_mem);
    if (s->tab_dev) cudaFree(s->tab_dev);
    if (s->counters) cudaFree(s->counters);
    if (s->resid_dev) cudaFree(s->resid_dev);
    if (s->fields_dev) cudaFree(s->fields_dev);
    if (s->tab_host) cudaFreeHost(s->tab_host);
    if (s->resid_host) cudaFreeHost(s->resid_host);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

const char* mglc_server_last_error(const mglc_server* s) { return s ? s->err.c_str() : "null server"; }

int mglc_server_submit(mglc_server* s, const mglc_request* r, long long* id) {
    if (!s || !r) return MGLC_ERR_INVALID;
    if (r->kind != MGLC_KIND_LID && r->kind != MGLC_KIND_THERMAL)
        return sfail(s, MGLC_ERR_INVALID, "request kind must be lid or thermal");
    if (r->n < 8 || r->n > 1024) return sfail(s, MGLC_ERR_INVALID, "request grid %d out of [8, 1024]", r->n);
    if (r->kind == MGLC_KIND_LID && !(r->reynolds > 0)) return sfail(s, MGLC_ERR_INVALID, "reynolds must be positive");
    if (r->kind == MGLC_KIND_THERMAL && !(r->rayleigh > 0)) return sfail(s, MGLC_ERR_INVALID, "rayleigh must be positive");
    if (footprint(s, r->kind, r->n) > s->arena.size)
        return sfail(s, MGLC_ERR_NOMEM, "a %d^3 solve does not fit the HBM budget", r->n);
    Req q;
    q.id = (long long)s->reqs.size();
    q.r = *r;
    s->reqs.push_back(q);
    if (id) *id = q.id;
    return MGLC_OK;
}

int mglc_server_run(mglc_server* s, double time_limit_s) {
    if (!s) return MGLC_ERR_INVALID;
    int rc;
    if (!s->tuned) {
        if (s->p.autotune) {
            if ((rc = autotune(s))) return rc;
        } else {
            s->tuned = true;
        }
    }
    if (!s->graph && (rc = build_graph(s))) return rc;
    // results staging: the largest solve's rho,u,v,w,T
    size_t want = 0;
    for (auto& q : s->reqs) want = std::max(want, (size_t)q.r.n * q.r.n * q.r.n * 5 * sizeof(float));
    if (s->p.keep_results && want > s->fields_bytes) {
        if (s->fields_dev) cudaFree(s->fields_dev);
        SCK(cudaMalloc((void**)&s->fields_dev, want), "result staging");
        s->fields_bytes = want;
    }
    if (s->t0 < 0) s->t0 = now_s();
    const double start = now_s();
    const int K = s->p.steps_per_iteration;
    for (;;) {
        const double t = now_s() - s->t0;
        bool pending = false;
        for (size_t q = 0; q < s->reqs.size(); q++) {
            Req& r = s->reqs[q];
            if (r.state == 0) {
                if (r.r.arrival_s <= t) {
                    r.state = 1;
                    s->waiting.push_back((int)q);
                } else {
                    pending = true;
                }
            }
        }
        if ((rc = admit(s, t))) return rc;
        if (s->active.empty()) {
            if (!pending && s->waiting.empty()) break;  // everything retired
            // idle until the next arrival
            double next = 1e30;
            for (auto& r : s->reqs)
                if (r.state == 0) next = std::min(next, r.r.arrival_s);
            const double wait = std::min(0.002, std::max(0.0, next - (now_s() - s->t0)));
            std::this_thread::sleep_for(std::chrono::duration<double>(wait));
            continue;
        }
        if (now_s() - start > time_limit_s) return sfail(s, MGLC_ERR_STATE, "time limit reached");
        const double it0 = now_s();
        {
            IterRange nvtx_range;  // graph launch .. completion (NVTX)
            SCK(cudaGraphLaunch(s->graph, s->stream), "graph launch");
            SCK(cudaEventRecord(s->done, s->stream), "event record");
            SCK(cudaEventSynchronize(s->done), "iteration");
        }
        s->stats.busy_s += now_s() - it0;
        s->stats.iterations++;
        // retire converged solves and solves at the step cap
        std::vector<int> keep;
        for (size_t a = 0; a < s->active.size(); a++) {
            Req& q = s->reqs[s->active[a]];
            q.steps += K;
            s->stats.steps_total += K;
            s->stats.cell_updates += (long long)K * q.sv.plane;
            float r;
            std::memcpy(&r, &s->resid_host[a], sizeof r);
            q.resid = r;
            const bool conv = q.steps > K && r < s->p.tol;
            if (conv || q.steps >= s->p.max_steps) {
                q.converged = conv ? 1 : 0;
                if (s->p.keep_results) {
                    const size_t nf = (q.r.kind == MGLC_KIND_THERMAL ? 5 : 4) * (size_t)q.sv.plane;
                    q.fields.resize(nf);
                    SCK(launch_serve_fields(s->p.precision, q.sv, s->fields_dev, s->stream), "fields");
                    SCK(cudaMemcpyAsync(q.fields.data(), s->fields_dev, nf * sizeof(float),
                                        cudaMemcpyDeviceToHost, s->stream), "copy fields");
                    SCK(cudaStreamSynchronize(s->stream), "fields");
                }
                q.finish_s = now_s() - s->t0;
                q.state = 3;
                s->arena.release(q.off, q.bytes);
            } else {
                keep.push_back(s->active[a]);
            }
        }
        if (keep.size() != s->active.size()) {
            s->active = keep;
            if ((rc = upload_table(s))) return rc;
        }
    }
    s->stats.wall_s = now_s() - s->t0;
    return MGLC_OK;
}

int mglc_server_results(mglc_server* s, mglc_request_result* out, int max, int* count) {
    if (!s || !count) return MGLC_ERR_INVALID;
    int n = 0;
    for (auto& q : s->reqs) {
        if (q.state != 3) continue;
        if (out && n < max) {
            mglc_request_result& o = out[n];
            o.id = q.id;
            o.kind = q.r.kind;
            o.n = q.r.n;
            o.steps = q.steps;
            o.residual = q.resid;
            o.arrival_s = q.r.arrival_s;
            o.admit_s = q.admit_s;
            o.finish_s = q.finish_s;
            o.converged = q.converged;
        }
        n++;
    }
    *count = n;
    return MGLC_OK;
}

int mglc_server_get_field(mglc_server* s, long long id, float* out) {
    if (!s || !out || id < 0 || id >= (long long)s->reqs.size()) return MGLC_ERR_INVALID;
    const Req& q = s->reqs[id];
    if (q.state != 3 || q.fields.empty())
        return sfail(s, MGLC_ERR_STATE, "request %lld has no stored fields (not retired or keep_results = 0)", id);
    std::memcpy(out, q.fields.data(), q.fields.size() * sizeof(float));
    return MGLC_OK;
}

int mglc_server_get_stats(mglc_server* s, mglc_server_stats* out) {
    if (!s || !out) return MGLC_ERR_INVALID;
    *out = s->stats;
    out->tile_threads = s->block;
    out->tile_rows = s->rows;
    out->ctas_per_sm = s->ctas_per_sm;
    return MGLC_OK;
}

}  // extern "C"
