// sf_capi.cpp — the C ABI (include/sf_capi.h): solver contexts, device
// memory, the captured step graph, host<->device state copies.
//
// Maps the reference's solver calls onto one CUDA stream per context:
//   SPHSolver<float>(params)        Include/QtSPHSolver.h:30-31   -> sf_create
//   makeReady()                     Source/Simulator.cpp:42       -> sf_make_ready
//   advanceFrame()                  Source/Simulator.cpp:49       -> sf_advance_frame / sf_step
//   getParticles()/getVelocity()    Include/QtSPHSolver.h:34-35   -> sf_get_state / sf_set_state
//   SceneManager::setupScene        Source/SceneManager.cpp:21-38 -> sf_setup_scene
//   SPHParameters::updateParams()   Source/Controller.cpp:63      -> sf_params_update
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "sf_internal.h"
#include "sf_render.h"

namespace sf {
// Recorded trajectory of sf_forward and the adjoint's buffers.
struct StepRec {
    float4* pos = nullptr;
    float4* vel = nullptr;
    float2* pr = nullptr;
    float* rho = nullptr;
    uint32_t* nbr = nullptr;
    uint32_t* cnt = nullptr;
    uint32_t* cs = nullptr;
    float4* sums = nullptr;
};
struct Trajectory {
    uint32_t nsteps = 0, ckpt = 0, n = 0, ncells_pad = 0;
    bool valid = false;
    std::vector<float4*> ck;  // per checkpoint: pos then vel (2n float4)
    std::vector<StepRec> rec; // ckpt steps of one segment
    float4* snap = nullptr;   // 2n float4: the forward's final state
    float4* stage = nullptr;  // 2n float4: the checkpoint a segment graph starts from
    double2* seg_partial = nullptr;  // ckpt x adjoint_partial_count(n) scalar partials
    // captured segment graphs (recompute + reverse sweep), by segment length
    cudaGraphExec_t seg_graph[2] = {nullptr, nullptr};
    uint32_t seg_len[2] = {0, 0};
    uint64_t graph_gen = 0;
    AdjointWork w;
    uint32_t hist_res = 0;
    unsigned long long* hist = nullptr;
    float* e2 = nullptr;
    float* target = nullptr;
    double* hpartial = nullptr;
};
}  // namespace sf

struct sf_ctx {
    uint64_t gen = 1;  // bumped whenever captured graphs become stale
    sf_params params{};
    sf::SimConst c{};
    sf::DeviceState d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    // uploads: a second stream, so that the velocity copy overlaps the sort
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_pos = nullptr, ev_vel = nullptr;
    // the GPU reads and writes pageable host memory through the host's page
    // tables (Grace: NVLink-C2C with address translation): -1 unknown, 0, 1
    int host_direct = -1;
    uint32_t* d_report = nullptr;  // sf_check_state counters
    cudaGraphExec_t step_graph = nullptr;
    bool sorted = false;  // particles uploaded and cell-sorted
    float* h_stage = nullptr;  // pinned staging for pageable caller buffers
    size_t h_stage_bytes = 0;
    sf::Trajectory* traj = nullptr;  // differentiable runs (sf_forward / sf_adjoint)
    sf::FrameState* frame = nullptr;  // device sub-step / frame state
    cudaGraphExec_t frame_graph = nullptr;
    uint64_t frame_graph_gen = 0;
    double frame_graph_time = 0.0;
    uint32_t frame_graph_max = 0;
    // render buffers (sf_render)
    int render_w = 0, render_h = 0;
    uint32_t render_n = 0;
    unsigned long long* render_keys = nullptr;
    float4* render_rgba = nullptr;
    float* render_depth = nullptr;
    uint32_t* render_owner = nullptr;
    uint32_t* render_slot = nullptr;
};

namespace {

// NVTX range over an API call (visible in Nsight timelines; a no-op without a
// tool attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define SF_RANGE(name) NvtxRange sf_nvtx_range_(name)

thread_local std::string g_error;

// Fault injection (sf_test_fail_allocation): device allocations to let
// through before one fails as out of memory; negative when disarmed.
std::atomic<int64_t> g_fail_alloc{-1};

cudaError_t dev_malloc_raw(void** p, size_t bytes) {
    int64_t k = g_fail_alloc.load();
    while (k >= 0 && !g_fail_alloc.compare_exchange_weak(k, k - 1)) {
    }
    if (k == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

template <typename T>
cudaError_t dev_malloc(T** p, size_t bytes) {
    return dev_malloc_raw(reinterpret_cast<void**>(p), bytes);
}

sf_status fail(sf_status st, const std::string& msg) {
    g_error = msg;
    return st;
}

sf_status cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();  // clear a sticky launch error where possible
    return fail(e == cudaErrorMemoryAllocation ? SF_ERR_OUT_OF_MEMORY : SF_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define SF_CUDA(call)                                      \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

#define SF_TRY(call)                    \
    do {                                \
        sf_status st_ = (call);         \
        if (st_ != SF_OK) return st_;   \
    } while (0)

constexpr uint64_t kMaxCells = 1ull << 28;

sf_status validate(const sf_params& p) {
    auto finite = [](float v) { return std::isfinite(v); };
    if (!finite(p.kernel_radius) || !(p.kernel_radius > 0.f))
        return fail(SF_ERR_INVALID_ARGUMENT, "kernel_radius must be positive and finite");
    if (!finite(p.particle_radius) || !(p.particle_radius > 0.f))
        return fail(SF_ERR_INVALID_ARGUMENT, "particle_radius must be positive and finite");
    if (!finite(p.pressure_stiffness) || p.pressure_stiffness < 0.f)
        return fail(SF_ERR_INVALID_ARGUMENT, "pressure_stiffness must be >= 0");
    if (!finite(p.viscosity) || p.viscosity < 0.f) return fail(SF_ERR_INVALID_ARGUMENT, "viscosity must be >= 0");
    if (!finite(p.boundary_restitution) || p.boundary_restitution < 0.f || p.boundary_restitution > 1.f)
        return fail(SF_ERR_INVALID_ARGUMENT, "boundary_restitution must be in [0, 1]");
    if (!finite(p.rest_density) || !(p.rest_density > 0.f))
        return fail(SF_ERR_INVALID_ARGUMENT, "rest_density must be positive");
    if (!finite(p.time_step) || !(p.time_step > 0.f)) return fail(SF_ERR_INVALID_ARGUMENT, "time_step must be > 0");
    if (!finite(p.stop_time) || p.stop_time < 0.f) return fail(SF_ERR_INVALID_ARGUMENT, "stop_time must be >= 0");
    if (p.eos != SF_EOS_LINEAR && p.eos != SF_EOS_TAIT) return fail(SF_ERR_INVALID_ARGUMENT, "unknown eos");
    if (p.num_threads < 0) return fail(SF_ERR_INVALID_ARGUMENT, "num_threads must be >= 0");
    if (p.cells_per_h < 0 || p.cells_per_h > 3)
        return fail(SF_ERR_INVALID_ARGUMENT, "cells_per_h must be 1, 2 or 3 (0 = 2)");
    if (p.adaptive_time_step != 0 && p.adaptive_time_step != 1)
        return fail(SF_ERR_INVALID_ARGUMENT, "adaptive_time_step must be 0 or 1");
    if (p.reserved[0]) return fail(SF_ERR_INVALID_ARGUMENT, "reserved fields must be zero");
    for (int a = 0; a < 3; ++a) {
        if (!finite(p.gravity[a]) || !finite(p.box_min[a]) || !finite(p.box_max[a]))
            return fail(SF_ERR_INVALID_ARGUMENT, "gravity and box must be finite");
        if (!((double)p.box_max[a] - p.box_min[a] > 2.0 * p.particle_radius))
            return fail(SF_ERR_INVALID_ARGUMENT, "box must be wider than one particle diameter on every axis");
    }
    return SF_OK;
}

sf_status ensure_stage(sf_ctx* ctx, size_t bytes) {
    if (ctx->h_stage_bytes >= bytes) return SF_OK;
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_bytes = 0;
    SF_CUDA(cudaMallocHost(&ctx->h_stage, bytes));
    ctx->h_stage_bytes = bytes;
    return SF_OK;
}

// Pageable (not page-locked, not device) host memory that the context's GPU
// can read and write in place: the device accesses pageable memory through
// the host's page tables.
bool host_direct(sf_ctx* ctx, const void* p) {
    if (ctx->host_direct < 0) {
        int a = 0, b = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, ctx->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device) != cudaSuccess) {
            cudaGetLastError();
            a = b = 0;
        }
        ctx->host_direct = (a && b) ? 1 : 0;
    }
    if (!ctx->host_direct) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeUnregistered;
}

bool is_pinned(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void free_particles(sf::DeviceState& d) {
    void* bufs[] = {d.pos, d.vel, d.pos2, d.vel2, d.pr, d.rho, d.key_slot, d.tmp, d.io, d.accel, d.nbr, d.nbr_count,
                    d.pv};
    for (void* b : bufs)
        if (b) cudaFree(b);
    d.pos = d.vel = d.pos2 = d.vel2 = d.accel = nullptr;
    d.pr = nullptr;
    d.rho = nullptr;
    d.key_slot = nullptr;
    d.tmp = nullptr;
    d.io = nullptr;
    d.nbr = nullptr;
    d.nbr_count = nullptr;
    d.pv = nullptr;
    d.cap = 0;
}

void free_grid(sf::DeviceState& d) {
    if (d.counts) cudaFree(d.counts);
    if (d.cell_start) cudaFree(d.cell_start);
    if (d.tile_sums) cudaFree(d.tile_sums);
    d.counts = d.cell_start = d.tile_sums = nullptr;
    d.ncells = d.ncells_pad = d.ntiles = 0;
}

void free_rec(sf::StepRec& r) {
    void* b[] = {r.pos, r.vel, r.pr, r.rho, r.nbr, r.cnt, r.cs, r.sums};
    for (void* p : b)
        if (p) cudaFree(p);
    r = sf::StepRec{};
}

void drop_segment_graphs(sf::Trajectory* t) {
    for (int g = 0; g < 2; ++g) {
        if (t->seg_graph[g]) cudaGraphExecDestroy(t->seg_graph[g]);
        t->seg_graph[g] = nullptr;
        t->seg_len[g] = 0;
    }
}

void free_trajectory(sf_ctx* ctx) {
    sf::Trajectory* t = ctx->traj;
    if (!t) return;
    drop_segment_graphs(t);
    if (t->stage) cudaFree(t->stage);
    if (t->seg_partial) cudaFree(t->seg_partial);
    for (float4* p : t->ck)
        if (p) cudaFree(p);
    for (auto& r : t->rec) free_rec(r);
    void* b[] = {t->snap, t->w.Xb, t->w.Vb, t->w.apb, t->w.avb, t->w.xdir, t->w.vdir, t->w.xf, t->w.vf,
                 t->w.rhob, t->w.scalars, t->hist, t->e2, t->target, t->hpartial};
    for (void* p : b)
        if (p) cudaFree(p);
    delete t;
    ctx->traj = nullptr;
}

void free_render(sf_ctx* ctx) {
    void* b[] = {ctx->render_keys, ctx->render_rgba, ctx->render_depth, ctx->render_owner, ctx->render_slot};
    for (void* p : b)
        if (p) cudaFree(p);
    ctx->render_keys = nullptr;
    ctx->render_rgba = nullptr;
    ctx->render_depth = nullptr;
    ctx->render_owner = nullptr;
    ctx->render_slot = nullptr;
    ctx->render_w = ctx->render_h = 0;
    ctx->render_n = 0;
}

void drop_graph(sf_ctx* ctx) {
    if (ctx->step_graph) cudaGraphExecDestroy(ctx->step_graph);
    ctx->step_graph = nullptr;
    ++ctx->gen;
}

// On any failure the grid is released and the context needs a new upload.
sf_status alloc_grid(sf_ctx* ctx) {
    sf::DeviceState& d = ctx->d;
    if (d.ncells == ctx->c.ncells && d.counts) return SF_OK;
    free_grid(d);
    const uint64_t pad = ((uint64_t)ctx->c.ncells + 1 + sf::kScanTile - 1) / sf::kScanTile * sf::kScanTile;
    const uint32_t ntiles = (uint32_t)(pad / sf::kScanTile);
    cudaError_t e = dev_malloc(&d.counts, pad * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&d.cell_start, pad * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&d.tile_sums, (size_t)ntiles * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(d.tile_sums, 0, (size_t)ntiles * sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.counts, 0, pad * sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.cell_start, 0, pad * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) {
        free_grid(d);
        ctx->sorted = false;
        return cuda_fail(e, "grid allocation");
    }
    d.ncells = ctx->c.ncells;
    d.ncells_pad = (uint32_t)pad;
    d.ntiles = ntiles;
    return SF_OK;
}

// On any failure the particle buffers are released and the context holds no
// particles until the next successful upload.
sf_status alloc_particles(sf_ctx* ctx, uint32_t n) {
    sf::DeviceState& d = ctx->d;
    if (n <= d.cap && d.pos) return SF_OK;
    free_trajectory(ctx);  // its buffers are sized by the capacity
    free_particles(d);
    const size_t c = n ? n : 1;
    const size_t tiles = (c + sf::kNbTile - 1) / sf::kNbTile;
    cudaError_t e = dev_malloc(&d.pos, c * sizeof(float4));
    if (e == cudaSuccess) e = dev_malloc(&d.vel, c * sizeof(float4));
    if (e == cudaSuccess) e = dev_malloc(&d.pos2, c * sizeof(float4));
    if (e == cudaSuccess) e = dev_malloc(&d.vel2, c * sizeof(float4));
    if (e == cudaSuccess) e = dev_malloc(&d.pr, c * sizeof(float2));
    if (e == cudaSuccess) e = dev_malloc(&d.rho, c * sizeof(float));
    if (e == cudaSuccess) e = dev_malloc(&d.key_slot, c * sizeof(uint2));
    if (e == cudaSuccess) e = dev_malloc(&d.tmp, c * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&d.io, c * 6 * sizeof(float));
    if (e == cudaSuccess) e = dev_malloc(&d.nbr, tiles * sf::kNbCap * sf::kNbTile * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&d.nbr_count, c * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&d.pv, c * 2 * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(d.nbr_count, 0, c * sizeof(uint32_t));
    if (e != cudaSuccess) {
        free_particles(d);
        d.n = 0;
        ctx->sorted = false;
        drop_graph(ctx);
        return cuda_fail(e, "particle buffer allocation");
    }
    d.cap = (uint32_t)c;
    return SF_OK;
}

sf_status set_device(const sf_ctx* ctx) {
    SF_CUDA(cudaSetDevice(ctx->device));
    return SF_OK;
}

sf_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return SF_OK;
}

// Upload n particles (device AoS staging already filled) and cell-sort them.
// Load a caller-order AoS state from device arrays (vel3 NULL: at rest) and
// sort it into the cell order.
sf_status sort_uploaded(sf_ctx* ctx, const float* pos3, const float* vel3) {
    sf::DeviceState& d = ctx->d;
    sf::launch_load_aos(pos3, vel3, d.n, d.pos2, d.vel2, ctx->stream);
    sf::launch_hash_count(d, d.pos2, d.n, ctx->c, d.counts, d.key_slot, ctx->stream);
    sf::enqueue_sort_tail(d, ctx->stream);
    if (ctx->frame && ctx->c.adaptive) sf::launch_init_maxima(d.vel, d.n, ctx->frame, ctx->stream);
    SF_TRY(check_launch("initial sort"));
    ctx->sorted = true;
    return SF_OK;
}

// Upload from page-locked host arrays: positions first, then the velocity
// copy on the second stream while the positions are hashed, counted and
// scattered; the gather waits for the velocities.
sf_status upload_overlapped(sf_ctx* ctx, const float* pos_xyz, const float* vel_xyz) {
    sf::DeviceState& d = ctx->d;
    if (!ctx->aux) {
        SF_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
        SF_CUDA(cudaEventCreateWithFlags(&ctx->ev_pos, cudaEventDisableTiming));
        SF_CUDA(cudaEventCreateWithFlags(&ctx->ev_vel, cudaEventDisableTiming));
    }
    const size_t bytes = (size_t)d.n * 3 * sizeof(float);
    float* io_pos = d.io;
    float* io_vel = d.io + 3 * (size_t)d.n;
    SF_CUDA(cudaMemcpyAsync(io_pos, pos_xyz, bytes, cudaMemcpyHostToDevice, ctx->stream));
    SF_CUDA(cudaEventRecord(ctx->ev_pos, ctx->stream));
    SF_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->ev_pos, 0));  // after all earlier work on io
    SF_CUDA(cudaMemcpyAsync(io_vel, vel_xyz, bytes, cudaMemcpyHostToDevice, ctx->aux));
    sf::launch_load_vel(io_vel, d.n, d.vel2, ctx->aux);
    SF_CUDA(cudaEventRecord(ctx->ev_vel, ctx->aux));
    sf::launch_load_pos(io_pos, d.n, d.pos2, ctx->stream);
    sf::launch_hash_count(d, d.pos2, d.n, ctx->c, d.counts, d.key_slot, ctx->stream);
    sf::enqueue_sort_tail(d, ctx->stream, ctx->ev_vel);
    if (ctx->frame && ctx->c.adaptive) sf::launch_init_maxima(d.vel, d.n, ctx->frame, ctx->stream);
    SF_TRY(check_launch("initial sort"));
    ctx->sorted = true;
    return SF_OK;
}

// The step as launched: with the adaptive sub-step, dt is chosen on the
// device first and the force pass reads it and raises the maxima.
void enqueue_full_step(sf_ctx* ctx) {
    if (ctx->c.adaptive) {
        sf::DeviceState dr = ctx->d;
        dr.frame = ctx->frame;
        sf::launch_choose_dt(ctx->frame, ctx->c, ctx->stream);
        sf::enqueue_step(dr, ctx->c, ctx->stream);
    } else {
        sf::enqueue_step(ctx->d, ctx->c, ctx->stream);
    }
}

sf_status capture_step(sf_ctx* ctx) {
    drop_graph(ctx);
    cudaGraph_t g = nullptr;
    SF_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_full_step(ctx);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(step)");
    e = cudaGraphInstantiate(&ctx->step_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        ctx->step_graph = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate(step)");
    }
    return SF_OK;
}

sf_status need_ctx(const sf_ctx* ctx) {
    if (!ctx) return fail(SF_ERR_INVALID_ARGUMENT, "null context");
    return SF_OK;
}

sf_status need_sorted(const sf_ctx* ctx) {
    SF_TRY(need_ctx(ctx));
    if (!ctx->sorted || ctx->d.n == 0) return fail(SF_ERR_NOT_READY, "no particles: call sf_set_state first");
    return SF_OK;
}

// Device -> host copy into a caller buffer (direct when pinned).
sf_status copy_out(sf_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!bytes) return SF_OK;
    if (is_pinned(dst)) {
        SF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
    SF_TRY(ensure_stage(ctx, bytes));
    SF_CUDA(cudaMemcpyAsync(ctx->h_stage, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    std::memcpy(dst, ctx->h_stage, bytes);
    return SF_OK;
}

sf_status copy_in(sf_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!bytes) return SF_OK;
    if (is_pinned(src)) {
        SF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
        return SF_OK;
    }
    SF_TRY(ensure_stage(ctx, bytes));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));  // staging may still feed an earlier copy
    std::memcpy(ctx->h_stage, src, bytes);
    SF_CUDA(cudaMemcpyAsync(dst, ctx->h_stage, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return SF_OK;
}

}  // namespace

namespace sf {

void build_render_const(const sf_render_params& rp, float particle_radius, uint32_t n, RenderConst* rc) {
    // glm::lookAt (right-handed) and glm::perspective, in double
    double e[3], f[3], u[3], s3[3], uu[3];
    for (int a = 0; a < 3; ++a) {
        e[a] = rp.eye[a];
        f[a] = (double)rp.focus[a] - rp.eye[a];
        u[a] = rp.up[a];
    }
    auto norm = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int a = 0; a < 3; ++a) v[a] /= l;
    };
    auto cross = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    norm(f);
    cross(f, u, s3);
    norm(s3);
    cross(s3, f, uu);
    double V[16] = {0};
    for (int a = 0; a < 3; ++a) {
        V[4 * a + 0] = s3[a];
        V[4 * a + 1] = uu[a];
        V[4 * a + 2] = -f[a];
    }
    V[12] = -(s3[0] * e[0] + s3[1] * e[1] + s3[2] * e[2]);
    V[13] = -(uu[0] * e[0] + uu[1] * e[1] + uu[2] * e[2]);
    V[14] = f[0] * e[0] + f[1] * e[1] + f[2] * e[2];
    V[15] = 1.0;
    const double kPi = 3.14159265358979323846;
    const double th = std::tan((double)rp.fovy_deg * 0.5 * kPi / 180.0);
    const double aspect = (double)rp.width / (double)rp.height;
    const double zn = rp.znear, zf = rp.zfar;
    double P[16] = {0};
    P[0] = 1.0 / (aspect * th);
    P[5] = 1.0 / th;
    P[10] = -(zf + zn) / (zf - zn);
    P[11] = -1.0;
    P[14] = -(2.0 * zf * zn) / (zf - zn);
    for (int k = 0; k < 16; ++k) {
        rc->V[k] = (float)V[k];
        rc->P[k] = (float)P[k];
    }
    // u_PointScale = height / tanf(fovy / 2) (Source/FluidRenderWidget.cpp:66)
    rc->scale = (float)rp.height / std::tan((float)((double)rp.fovy_deg * 0.5 * kPi / 180.0));
    rc->radius = rp.point_radius > 0.f ? rp.point_radius : particle_radius;
    rc->width = rp.width;
    rc->height = rp.height;
    rc->num_lights = rp.num_lights;
    std::memcpy(rc->light_position, rp.light_position, sizeof(rc->light_position));
    std::memcpy(rc->light_ambient, rp.light_ambient, sizeof(rc->light_ambient));
    std::memcpy(rc->light_diffuse, rp.light_diffuse, sizeof(rc->light_diffuse));
    std::memcpy(rc->light_specular, rp.light_specular, sizeof(rc->light_specular));
    std::memcpy(rc->mat_ambient, rp.mat_ambient, sizeof(rc->mat_ambient));
    std::memcpy(rc->mat_diffuse, rp.mat_diffuse, sizeof(rc->mat_diffuse));
    std::memcpy(rc->mat_specular, rp.mat_specular, sizeof(rc->mat_specular));
    rc->mat_shininess = rp.mat_shininess;
    rc->color_mode = rp.color_mode;
    rc->color_seed = rp.color_seed;
    // PARTICLE_COLOR_RAMP (Include/Common.h:33-42)
    const float ramp[kRampColors][3] = {{1.0f, 0.0f, 0.0f}, {1.0f, 0.5f, 0.0f}, {1.0f, 1.0f, 0.0f}, {1.0f, 0.0f, 1.0f},
                                        {0.0f, 1.0f, 0.0f}, {0.0f, 1.0f, 1.0f}, {0.0f, 0.0f, 1.0f}};
    std::memcpy(rc->ramp, ramp, sizeof(ramp));
    rc->ramp_step = (float)((double)(kRampColors - 1) / (double)(n > 1 ? n - 1 : 1));
    std::memcpy(rc->background, rp.background, sizeof(rc->background));
}

int derive_constants(const sf_params& p, SimConst* c, const char** why) {
    const double h = p.kernel_radius, r = p.particle_radius;
    const double kPi = 3.14159265358979323846;
    const double mass = (double)p.rest_density * (2.0 * r) * (2.0 * r) * (2.0 * r);
    const double h3 = h * h * h, h6 = h3 * h3, h9 = h6 * h3;
    c->h = (float)h;
    c->h2 = (float)(h * h);
    c->mass = (float)mass;
    c->cd = (float)(mass * 315.0 / (64.0 * kPi * h9));
    c->cp = (float)(mass * 45.0 / (kPi * h6) * 0.5);
    c->cv = (float)((double)p.viscosity * mass * 45.0 / (kPi * h6));
    c->k = p.pressure_stiffness;
    c->rho0 = p.rest_density;
    c->inv_rho0 = (float)(1.0 / (double)p.rest_density);
    c->dt = p.time_step;
    c->e = p.boundary_restitution;
    c->eos = p.eos;
    c->attractive = p.use_attractive_pressure ? 1 : 0;
    c->cell_base = 0;
    c->adaptive = p.adaptive_time_step ? 1 : 0;
    c->cfl_v = 0.4f;
    c->cfl_a = 0.25f;
    const int K = p.cells_per_h ? p.cells_per_h : 2;
    c->reach = K;
    double coord_max = 0.0;
    uint64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)p.box_max[a] - (double)p.box_min[a];
        c->g[a] = p.gravity[a];
        c->lo[a] = (float)((double)p.box_min[a] + r);
        c->hi[a] = (float)((double)p.box_max[a] - r);
        c->bmin[a] = p.box_min[a];
        double na = std::floor((double)K * ext / h);
        if (na < 1) na = 1;
        if (na > 65535) {
            *why = "more than 65535 cells along one axis (box / kernel_radius too large)";
            return SF_ERR_GRID_TOO_LARGE;
        }
        c->n[a] = (int)na;
        c->inv_cell[a] = (float)(na / ext);
        c->cell_w[a] = (float)(ext / na);
        cells *= (uint64_t)c->n[a];
        coord_max = std::fmax(coord_max, std::fmax(std::fabs((double)p.box_min[a]), std::fabs((double)p.box_max[a])));
    }
    // Slack of the pruning bound: a few float ulps of the largest coordinate
    // (cell assignment and the in-cell offset are each good to ~1 ulp) plus
    // 1e-5 h.
    c->prune_margin = (float)(16.0 * std::ldexp(std::fmax(coord_max, 1.0), -23) + 1e-5 * h);
    c->prune_h2 = (float)(h * h * (1.0 + 1e-4));
    if (cells > kMaxCells) {
        *why = "uniform grid would exceed 2^28 cells (box / kernel_radius too large)";
        return SF_ERR_GRID_TOO_LARGE;
    }
    c->ncells = (uint32_t)cells;
    return SF_OK;
}

}  // namespace sf

// =====================================================================
extern "C" {

SF_API const char* sf_last_error(void) { return g_error.c_str(); }

SF_API const char* sf_version(void) { return "simplefluid-gb300 0.1 (sm_103a)"; }

SF_API sf_status sf_params_default(sf_params* p) {
    if (!p) return fail(SF_ERR_INVALID_ARGUMENT, "null params");
    std::memset(p, 0, sizeof(*p));
    p->num_threads = 0;
    p->particle_radius = 0.01f;
    p->kernel_radius = 0.04f;
    p->pressure_stiffness = 50.0f;
    p->boundary_restitution = 0.1f;
    p->viscosity = 0.01f;
    p->stop_time = 5.0f;
    p->use_attractive_pressure = 0;
    p->scene = SF_SCENE_DAMBREAK_16K;
    p->rest_density = 1000.0f;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -9.8f;
    p->gravity[2] = 0.0f;
    p->time_step = 1e-4f;
    for (int a = 0; a < 3; ++a) {
        p->box_min[a] = 0.0f;
        p->box_max[a] = 1.0f;
    }
    p->eos = SF_EOS_LINEAR;
    p->cells_per_h = 2;
    return SF_OK;
}

SF_API sf_status sf_params_update(sf_params* p) {
    if (!p) return fail(SF_ERR_INVALID_ARGUMENT, "null params");
    SF_TRY(validate(*p));
    sf::SimConst c;
    const char* why = "";
    const int st = sf::derive_constants(*p, &c, &why);
    if (st) return fail(st, why);
    return SF_OK;
}

SF_API sf_status sf_scene_count(const sf_params* p, int32_t scene, uint64_t seed, uint32_t* n_out) {
    if (!p || !n_out) return fail(SF_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<float> pts;
    const char* why = "";
    const int st = sf::scene_points(*p, scene, seed, pts, &why);
    if (st) return fail(st, why);
    *n_out = (uint32_t)(pts.size() / 3);
    return SF_OK;
}

SF_API sf_status sf_setup_scene(const sf_params* p, int32_t scene, uint64_t seed, float* pos_xyz, float* vel_xyz,
                                uint32_t capacity, uint32_t* n_out) {
    if (!p || !pos_xyz) return fail(SF_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<float> pts;
    const char* why = "";
    const int st = sf::scene_points(*p, scene, seed, pts, &why);
    if (st) return fail(st, why);
    const uint32_t n = (uint32_t)(pts.size() / 3);
    if (n_out) *n_out = n;
    if (n > capacity) return fail(SF_ERR_CAPACITY, "scene has more particles than the output capacity");
    std::memcpy(pos_xyz, pts.data(), pts.size() * sizeof(float));
    if (vel_xyz) std::memset(vel_xyz, 0, pts.size() * sizeof(float));
    return SF_OK;
}

SF_API sf_status sf_select_device(int32_t device) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SF_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return fail(SF_ERR_INVALID_ARGUMENT, "device index out of range");
    SF_CUDA(cudaSetDevice(device));
    return SF_OK;
}

SF_API sf_status sf_create(const sf_params* p, sf_ctx** out) {
    if (!p || !out) return fail(SF_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    SF_TRY(validate(*p));
    sf::SimConst c;
    const char* why = "";
    int st = sf::derive_constants(*p, &c, &why);
    if (st) return fail(st, why);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SF_ERR_NO_DEVICE, "no CUDA device available");
    }
    sf_ctx* ctx = new sf_ctx();
    ctx->params = *p;
    ctx->c = c;
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return cuda_fail(e, "stream creation");
    }
    st = alloc_grid(ctx);
    if (!st) {
        e = dev_malloc(&ctx->frame, sizeof(sf::FrameState));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->frame, 0, sizeof(sf::FrameState), ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "frame state");
    }
    if (st) {
        sf_destroy(ctx);
        return st;
    }
    *out = ctx;
    return SF_OK;
}

namespace {

// Every resource a context owns (also the engine embedded in a batch).
void release_ctx(sf_ctx* ctx) {
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->aux) cudaStreamSynchronize(ctx->aux);
    free_trajectory(ctx);
    free_render(ctx);
    if (ctx->frame_graph) cudaGraphExecDestroy(ctx->frame_graph);
    ctx->frame_graph = nullptr;
    if (ctx->frame) cudaFree(ctx->frame);
    ctx->frame = nullptr;
    drop_graph(ctx);
    free_particles(ctx->d);
    free_grid(ctx->d);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    if (ctx->d_report) cudaFree(ctx->d_report);
    ctx->d_report = nullptr;
    if (ctx->ev_pos) cudaEventDestroy(ctx->ev_pos);
    if (ctx->ev_vel) cudaEventDestroy(ctx->ev_vel);
    ctx->ev_pos = ctx->ev_vel = nullptr;
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    ctx->aux = nullptr;
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = nullptr;
}

}  // namespace

SF_API sf_status sf_destroy(sf_ctx* ctx) {
    if (!ctx) return SF_OK;
    release_ctx(ctx);
    delete ctx;
    return SF_OK;
}

SF_API sf_status sf_set_params(sf_ctx* ctx, const sf_params* p) {
    SF_TRY(need_ctx(ctx));
    if (!p) return fail(SF_ERR_INVALID_ARGUMENT, "null params");
    SF_TRY(validate(*p));
    sf::SimConst c;
    const char* why = "";
    const int st = sf::derive_constants(*p, &c, &why);
    if (st) return fail(st, why);
    SF_TRY(set_device(ctx));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    const bool grid_changed = std::memcmp(c.n, ctx->c.n, sizeof(c.n)) != 0 ||
                              std::memcmp(c.bmin, ctx->c.bmin, sizeof(c.bmin)) != 0 ||
                              std::memcmp(c.inv_cell, ctx->c.inv_cell, sizeof(c.inv_cell)) != 0;
    const bool became_adaptive = c.adaptive && !ctx->c.adaptive;
    ctx->params = *p;
    ctx->c = c;
    drop_graph(ctx);
    if (became_adaptive && ctx->sorted && ctx->d.n) sf::launch_init_maxima(ctx->d.vel, ctx->d.n, ctx->frame, ctx->stream);
    if (grid_changed) {
        SF_TRY(alloc_grid(ctx));
        if (ctx->sorted && ctx->d.n) {
            // Re-bucket the current state on the new grid (positions unchanged).
            sf::DeviceState& d = ctx->d;
            SF_CUDA(cudaMemcpyAsync(d.pos2, d.pos, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            SF_CUDA(cudaMemcpyAsync(d.vel2, d.vel, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            sf::launch_hash_count(d, d.pos2, d.n, ctx->c, d.counts, d.key_slot, ctx->stream);
            sf::enqueue_sort_tail(d, ctx->stream);
            SF_TRY(check_launch("re-sort after parameter change"));
        }
    }
    return SF_OK;
}

SF_API sf_status sf_get_params(const sf_ctx* ctx, sf_params* p) {
    SF_TRY(need_ctx(ctx));
    if (!p) return fail(SF_ERR_INVALID_ARGUMENT, "null params");
    *p = ctx->params;
    return SF_OK;
}

SF_API sf_status sf_set_state(sf_ctx* ctx, const float* pos_xyz, const float* vel_xyz, uint32_t n) {
    SF_RANGE("sf_set_state");
    SF_TRY(need_ctx(ctx));
    if (n && !pos_xyz) return fail(SF_ERR_INVALID_ARGUMENT, "null positions");
    SF_TRY(set_device(ctx));
    const bool resized = n != ctx->d.n;
    SF_TRY(alloc_particles(ctx, n));
    if (resized) drop_graph(ctx);
    ctx->d.n = n;
    ctx->sorted = false;
    if (n == 0) return SF_OK;
    if (vel_xyz && is_pinned(pos_xyz) && is_pinned(vel_xyz)) {
        SF_TRY(upload_overlapped(ctx, pos_xyz, vel_xyz));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
    if (host_direct(ctx, pos_xyz) && (!vel_xyz || host_direct(ctx, vel_xyz))) {
        // pageable arrays the GPU reads in place: no staging copy
        SF_TRY(sort_uploaded(ctx, pos_xyz, vel_xyz));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
    float* io = ctx->d.io;
    const size_t bytes = (size_t)n * 3 * sizeof(float);
    SF_TRY(copy_in(ctx, io, pos_xyz, bytes));
    if (vel_xyz) SF_TRY(copy_in(ctx, io + 3 * (size_t)n, vel_xyz, bytes));
    SF_TRY(sort_uploaded(ctx, io, vel_xyz ? io + 3 * (size_t)n : nullptr));
    // The caller may reuse its buffers once this returns.
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

SF_API sf_status sf_get_state(sf_ctx* ctx, float* pos_xyz, float* vel_xyz, uint32_t n) {
    SF_RANGE("sf_get_state");
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n) return fail(SF_ERR_INVALID_ARGUMENT, "n does not match the number of particles");
    SF_TRY(set_device(ctx));
    if ((pos_xyz || vel_xyz) && (!pos_xyz || host_direct(ctx, pos_xyz)) && (!vel_xyz || host_direct(ctx, vel_xyz))) {
        // pageable arrays the GPU writes in place: no staging copy
        sf::launch_store_caller_order(ctx->d.pos, ctx->d.vel, n, ctx->d.tmp, pos_xyz, vel_xyz, ctx->stream);
        SF_TRY(check_launch("store state"));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
    float* io = ctx->d.io;
    const size_t bytes = (size_t)n * 3 * sizeof(float);
    sf::launch_store_aos(ctx->d.pos, ctx->d.vel, n, pos_xyz ? io : nullptr, vel_xyz ? io + 3 * (size_t)n : nullptr,
                         ctx->stream);
    SF_TRY(check_launch("store state"));
    if (pos_xyz) SF_TRY(copy_out(ctx, pos_xyz, io, bytes));
    if (vel_xyz) SF_TRY(copy_out(ctx, vel_xyz, io + 3 * (size_t)n, bytes));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

SF_API sf_status sf_get_num_particles(const sf_ctx* ctx, uint32_t* n_out) {
    SF_TRY(need_ctx(ctx));
    if (!n_out) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    *n_out = ctx->d.n;
    return SF_OK;
}

namespace {

// Device memory of the context's GPU (plain or managed).
sf_status need_device_array(const sf_ctx* ctx, const void* p, const char* what) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return fail(SF_ERR_INVALID_ARGUMENT, std::string(what) + " is not a CUDA pointer");
    }
    if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != ctx->device)
        return fail(SF_ERR_INVALID_ARGUMENT, std::string(what) + " is not device memory of the context's GPU");
    return SF_OK;
}

// Order `waiter` after the work queued so far on `signaller`.
sf_status stream_after(cudaStream_t waiter, cudaStream_t signaller) {
    if (!signaller || signaller == waiter) return SF_OK;
    cudaEvent_t ev;
    SF_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, signaller);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(waiter, ev, 0);
    cudaEventDestroy(ev);
    SF_CUDA(e);
    return SF_OK;
}

}  // namespace

SF_API sf_status sf_set_state_device(sf_ctx* ctx, const float* d_pos_xyz, const float* d_vel_xyz, uint32_t n,
                                     void* other) {
    SF_RANGE("sf_set_state_device");
    SF_TRY(need_ctx(ctx));
    if (n && !d_pos_xyz) return fail(SF_ERR_INVALID_ARGUMENT, "null positions");
    SF_TRY(set_device(ctx));
    if (n) SF_TRY(need_device_array(ctx, d_pos_xyz, "positions"));
    if (n && d_vel_xyz) SF_TRY(need_device_array(ctx, d_vel_xyz, "velocities"));
    const bool resized = n != ctx->d.n;
    SF_TRY(alloc_particles(ctx, n));
    if (resized) drop_graph(ctx);
    ctx->d.n = n;
    ctx->sorted = false;
    if (n == 0) return SF_OK;
    SF_TRY(stream_after(ctx->stream, (cudaStream_t)other));
    return sort_uploaded(ctx, d_pos_xyz, d_vel_xyz);
}

SF_API sf_status sf_get_state_device(sf_ctx* ctx, float* d_pos_xyz, float* d_vel_xyz, uint32_t n, void* other) {
    SF_RANGE("sf_get_state_device");
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n) return fail(SF_ERR_INVALID_ARGUMENT, "n does not match the number of particles");
    SF_TRY(set_device(ctx));
    if (n && d_pos_xyz) SF_TRY(need_device_array(ctx, d_pos_xyz, "positions"));
    if (n && d_vel_xyz) SF_TRY(need_device_array(ctx, d_vel_xyz, "velocities"));
    sf::launch_store_aos(ctx->d.pos, ctx->d.vel, n, d_pos_xyz, d_vel_xyz, ctx->stream);
    SF_TRY(check_launch("store state"));
    return stream_after((cudaStream_t)other, ctx->stream);
}

SF_API sf_status sf_device_state(sf_ctx* ctx, sf_device_view* view) {
    SF_TRY(need_sorted(ctx));
    if (!view) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    const sf::DeviceState& d = ctx->d;
    view->pos4 = reinterpret_cast<const float*>(d.pos);
    view->vel4 = reinterpret_cast<const float*>(d.vel);
    view->rho = d.rho;
    view->p_inv_rho = reinterpret_cast<const float*>(d.pr);
    view->cell_start = d.cell_start;
    view->n = d.n;
    view->ncells = d.ncells;
    view->stream = (void*)ctx->stream;
    return SF_OK;
}

SF_API sf_status sf_make_ready(sf_ctx* ctx) {
    SF_RANGE("sf_make_ready");
    SF_TRY(need_sorted(ctx));
    SF_TRY(set_device(ctx));
    if (!ctx->step_graph) SF_TRY(capture_step(ctx));
    return SF_OK;
}

SF_API sf_status sf_advance_frame(sf_ctx* ctx, float* dt_out) {
    SF_TRY(sf_step(ctx, 1));
    if (!dt_out) return SF_OK;
    if (!ctx->c.adaptive) {
        *dt_out = ctx->params.time_step;
        return SF_OK;
    }
    SF_CUDA(cudaMemcpyAsync(dt_out, &ctx->frame->dt, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

// One frame as a graph: reset the frame clock, then a conditional while node
// whose body is one sub-step followed by the frame check.
static sf_status build_frame_graph(sf_ctx* ctx, double frame_time, uint32_t max_substeps, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    SF_CUDA(cudaGraphCreate(&g, 0));
    struct GraphGuard {
        cudaGraph_t g;
        ~GraphGuard() {
            if (g) cudaGraphDestroy(g);
        }
    } guard{g};
    cudaGraphConditionalHandle h;
    SF_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    SF_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    sf::launch_frame_begin(ctx->frame, ctx->stream);
    cudaGraph_t captured = nullptr;
    SF_CUDA(cudaStreamEndCapture(ctx->stream, &captured));
    size_t nn = 0;
    SF_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    SF_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cn;
    SF_CUDA(cudaGraphAddNode(&cn, g, nodes.data(), nullptr, nn, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    SF_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    sf::DeviceState dr = ctx->d;
    dr.frame = ctx->frame;
    sf::launch_choose_dt(ctx->frame, ctx->c, ctx->stream);
    sf::enqueue_step(dr, ctx->c, ctx->stream);
    sf::launch_frame_check(ctx->frame, frame_time, max_substeps, h, ctx->stream);
    SF_CUDA(cudaStreamEndCapture(ctx->stream, &body));
    SF_CUDA(cudaGraphInstantiate(out, g, 0));
    return SF_OK;
}

SF_API sf_status sf_advance_frames(sf_ctx* ctx, uint32_t frames, double frame_time, uint32_t max_substeps,
                                   double* sim_time_out, uint32_t* substeps_out) {
    SF_RANGE("sf_advance_frames");
    SF_TRY(sf_make_ready(ctx));
    if (!(frame_time > 0.0) || max_substeps == 0) return fail(SF_ERR_INVALID_ARGUMENT, "need frame_time > 0, max_substeps > 0");
    if (!ctx->frame_graph || ctx->frame_graph_gen != ctx->gen || ctx->frame_graph_time != frame_time ||
        ctx->frame_graph_max != max_substeps) {
        if (ctx->frame_graph) cudaGraphExecDestroy(ctx->frame_graph);
        ctx->frame_graph = nullptr;
        SF_TRY(build_frame_graph(ctx, frame_time, max_substeps, &ctx->frame_graph));
        ctx->frame_graph_gen = ctx->gen;
        ctx->frame_graph_time = frame_time;
        ctx->frame_graph_max = max_substeps;
    }
    SF_CUDA(cudaMemsetAsync(&ctx->frame->substeps, 0, sizeof(uint32_t), ctx->stream));
    SF_CUDA(cudaMemsetAsync(&ctx->frame->sim_time, 0, sizeof(double), ctx->stream));
    for (uint32_t f = 0; f < frames; ++f) SF_CUDA(cudaGraphLaunch(ctx->frame_graph, ctx->stream));
    sf::FrameState fs;
    SF_CUDA(cudaMemcpyAsync(&fs, ctx->frame, sizeof(fs), cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (sim_time_out) *sim_time_out = fs.sim_time;
    if (substeps_out) *substeps_out = fs.substeps;
    return SF_OK;
}

SF_API sf_status sf_step(sf_ctx* ctx, uint32_t nsteps) {
    SF_RANGE("sf_step");
    SF_TRY(sf_make_ready(ctx));
    for (uint32_t s = 0; s < nsteps; ++s) SF_CUDA(cudaGraphLaunch(ctx->step_graph, ctx->stream));
    return SF_OK;
}

SF_API sf_status sf_synchronize(sf_ctx* ctx) {
    SF_TRY(need_ctx(ctx));
    SF_TRY(set_device(ctx));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

SF_API sf_status sf_get_stream(sf_ctx* ctx, void** stream_out) {
    SF_TRY(need_ctx(ctx));
    if (!stream_out) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    *stream_out = (void*)ctx->stream;
    return SF_OK;
}

SF_API sf_status sf_host_alloc(size_t bytes, void** ptr_out) {
    if (!ptr_out) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    *ptr_out = nullptr;
    SF_CUDA(cudaMallocHost(ptr_out, bytes ? bytes : 1));
    return SF_OK;
}

SF_API sf_status sf_host_free(void* ptr) {
    if (ptr) SF_CUDA(cudaFreeHost(ptr));
    return SF_OK;
}

SF_API sf_status sf_get_grid(const sf_ctx* ctx, uint32_t dims_out[3]) {
    SF_TRY(need_ctx(ctx));
    if (!dims_out) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    for (int a = 0; a < 3; ++a) dims_out[a] = (uint32_t)ctx->c.n[a];
    return SF_OK;
}

SF_API sf_status sf_get_sorted(sf_ctx* ctx, float* pos4, float* vel4, uint32_t* ids, uint32_t* keys, uint32_t n) {
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n) return fail(SF_ERR_INVALID_ARGUMENT, "n does not match the number of particles");
    SF_TRY(set_device(ctx));
    std::vector<float4> p(n);
    SF_TRY(copy_out(ctx, p.data(), ctx->d.pos, (size_t)n * sizeof(float4)));
    if (pos4 || ids)
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t id;
            std::memcpy(&id, &p[i].w, sizeof(id));
            if (ids) ids[i] = id;
            if (pos4) {
                pos4[4 * (size_t)i] = p[i].x;
                pos4[4 * (size_t)i + 1] = p[i].y;
                pos4[4 * (size_t)i + 2] = p[i].z;
                pos4[4 * (size_t)i + 3] = 0.f;
            }
        }
    if (vel4) SF_TRY(copy_out(ctx, vel4, ctx->d.vel, (size_t)n * sizeof(float4)));
    if (keys) {
        sf::launch_keys(ctx->d, ctx->d.pos, n, ctx->c, ctx->d.tmp, ctx->stream);
        SF_TRY(check_launch("keys"));
        SF_TRY(copy_out(ctx, keys, ctx->d.tmp, (size_t)n * sizeof(uint32_t)));
    }
    return SF_OK;
}

SF_API sf_status sf_get_cell_start(sf_ctx* ctx, uint32_t* cell_start, uint32_t count) {
    SF_TRY(need_sorted(ctx));
    if (!cell_start || count != ctx->c.ncells + 1)
        return fail(SF_ERR_INVALID_ARGUMENT, "cell_start needs ncells + 1 entries");
    SF_TRY(set_device(ctx));
    return copy_out(ctx, cell_start, ctx->d.cell_start, (size_t)count * sizeof(uint32_t));
}

SF_API sf_status sf_compute_density(sf_ctx* ctx, float* rho, float* pressure, uint32_t n) {
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n) return fail(SF_ERR_INVALID_ARGUMENT, "n does not match the number of particles");
    SF_TRY(set_device(ctx));
    sf::launch_density(ctx->d, ctx->c, ctx->stream);
    SF_TRY(check_launch("density"));
    if (rho) SF_TRY(copy_out(ctx, rho, ctx->d.rho, (size_t)n * sizeof(float)));
    if (pressure) {
        std::vector<float2> pr(n);
        SF_TRY(copy_out(ctx, pr.data(), ctx->d.pr, (size_t)n * sizeof(float2)));
        for (uint32_t i = 0; i < n; ++i) pressure[i] = pr[i].x;
    }
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

SF_API sf_status sf_compute_accel(sf_ctx* ctx, float* accel_xyz, uint32_t n) {
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n || !accel_xyz) return fail(SF_ERR_INVALID_ARGUMENT, "bad output or size");
    SF_TRY(set_device(ctx));
    if (!ctx->d.accel) SF_CUDA(dev_malloc(&ctx->d.accel, (size_t)ctx->d.cap * sizeof(float4)));
    sf::launch_density(ctx->d, ctx->c, ctx->stream);
    sf::launch_force_only(ctx->d, ctx->c, ctx->stream);
    SF_TRY(check_launch("forces"));
    std::vector<float4> a(n);
    SF_TRY(copy_out(ctx, a.data(), ctx->d.accel, (size_t)n * sizeof(float4)));
    for (uint32_t i = 0; i < n; ++i) {
        accel_xyz[3 * (size_t)i] = a[i].x;
        accel_xyz[3 * (size_t)i + 1] = a[i].y;
        accel_xyz[3 * (size_t)i + 2] = a[i].z;
    }
    return SF_OK;
}

SF_API sf_status sf_neighbour_stats(sf_ctx* ctx, uint32_t* count, uint32_t* hash, uint32_t n) {
    SF_TRY(need_sorted(ctx));
    if (n != ctx->d.n || !count || !hash) return fail(SF_ERR_INVALID_ARGUMENT, "bad output or size");
    SF_TRY(set_device(ctx));
    // The AoS staging buffer (6 floats per particle) is free between calls.
    uint32_t* dc = reinterpret_cast<uint32_t*>(ctx->d.io);
    uint32_t* dh = dc + n;
    sf::launch_neighbour_stats(ctx->d, ctx->c, dc, dh, ctx->stream);
    SF_TRY(check_launch("neighbour stats"));
    SF_TRY(copy_out(ctx, count, dc, (size_t)n * sizeof(uint32_t)));
    SF_TRY(copy_out(ctx, hash, dh, (size_t)n * sizeof(uint32_t)));
    return SF_OK;
}

SF_API sf_status sf_test_fail_allocation(int64_t after) {
    g_fail_alloc.store(after < 0 ? -1 : after);
    return SF_OK;
}

SF_API sf_status sf_check_state(sf_ctx* ctx, sf_state_report* report) {
    SF_RANGE("sf_check_state");
    SF_TRY(need_sorted(ctx));
    if (!report) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    SF_TRY(set_device(ctx));
    if (!ctx->d_report) SF_CUDA(dev_malloc(&ctx->d_report, sf::kReportWords * sizeof(uint32_t)));
    // the bucketed-index buffer is free between steps: it holds the id tally
    const bool lists = ctx->d.nbr && ctx->d.tune.list_mode != SF_LIST_NONE;
    sf::launch_check_state(ctx->d, ctx->c, lists ? ctx->d.nbr_count : nullptr, ctx->d.tmp, ctx->d_report,
                           ctx->stream);
    SF_TRY(check_launch("check state"));
    uint32_t r[sf::kReportWords];
    SF_CUDA(cudaMemcpyAsync(r, ctx->d_report, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    report->n = ctx->d.n;
    report->non_finite = r[0];
    report->outside_box = r[1];
    report->unsorted = r[2];
    report->cell_table_mismatch = r[3];
    report->bad_ids = r[4];
    report->list_overflow = r[5];
    float v2;
    std::memcpy(&v2, &r[6], sizeof(v2));
    report->max_speed = std::sqrt(v2);
    return SF_OK;
}

// ---------------------------------------------------------------- timing
namespace {

struct EventSet {
    std::vector<cudaEvent_t> ev;
    ~EventSet() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    cudaError_t create(size_t n) {
        ev.assign(n, nullptr);
        for (size_t i = 0; i < n; ++i) {
            cudaError_t e = cudaEventCreate(&ev[i]);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
};

struct Scratch {
    void* p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace

SF_API sf_status sf_step_timed(sf_ctx* ctx, uint32_t nsteps, uint64_t flush_bytes, float* total_ms, float* step_ms) {
    SF_TRY(sf_make_ready(ctx));
    if (!total_ms) return fail(SF_ERR_INVALID_ARGUMENT, "null total_ms");
    *total_ms = 0.f;
    if (!nsteps) return SF_OK;
    Scratch flush;
    if (flush_bytes) SF_CUDA(dev_malloc(&flush.p, flush_bytes));
    EventSet ev;
    SF_CUDA(ev.create(2 * (size_t)nsteps));
    for (uint32_t i = 0; i < nsteps; ++i) {
        if (flush_bytes) SF_CUDA(cudaMemsetAsync(flush.p, (int)(i & 0xff), flush_bytes, ctx->stream));
        SF_CUDA(cudaEventRecord(ev.ev[2 * i], ctx->stream));
        SF_CUDA(cudaGraphLaunch(ctx->step_graph, ctx->stream));
        SF_CUDA(cudaEventRecord(ev.ev[2 * i + 1], ctx->stream));
    }
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    double total = 0.0;
    for (uint32_t i = 0; i < nsteps; ++i) {
        float ms = 0.f;
        SF_CUDA(cudaEventElapsedTime(&ms, ev.ev[2 * i], ev.ev[2 * i + 1]));
        if (step_ms) step_ms[i] = ms;
        total += ms;
    }
    *total_ms = (float)total;
    return SF_OK;
}

SF_API sf_status sf_get_tuning(const sf_ctx* ctx, sf_tuning* t) {
    SF_TRY(need_ctx(ctx));
    if (!t) return fail(SF_ERR_INVALID_ARGUMENT, "null tuning");
    std::memset(t, 0, sizeof(*t));
    t->list_mode = ctx->d.tune.list_mode;
    t->density_block = ctx->d.tune.density_block;
    t->force_block = ctx->d.tune.force_block;
    t->prefetch = ctx->d.tune.prefetch;
    return SF_OK;
}

SF_API sf_status sf_set_tuning(sf_ctx* ctx, const sf_tuning* t) {
    SF_TRY(need_ctx(ctx));
    if (!t) return fail(SF_ERR_INVALID_ARGUMENT, "null tuning");
    if (t->list_mode < SF_LIST_NONE || t->list_mode > SF_LIST_TILE)
        return fail(SF_ERR_INVALID_ARGUMENT, "unknown list_mode");
    if ((t->density_block != 128 && t->density_block != 256) || (t->force_block != 128 && t->force_block != 256))
        return fail(SF_ERR_INVALID_ARGUMENT, "block sizes must be 128 or 256");
    if (t->prefetch != 2 && t->prefetch != 4) return fail(SF_ERR_INVALID_ARGUMENT, "prefetch must be 2 or 4");
    if (t->reserved[0] || t->reserved[1] || t->reserved[2] || t->reserved[3])
        return fail(SF_ERR_INVALID_ARGUMENT, "reserved fields must be zero");
    SF_TRY(set_device(ctx));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->d.tune.list_mode = t->list_mode;
    ctx->d.tune.density_block = t->density_block;
    ctx->d.tune.force_block = t->force_block;
    ctx->d.tune.prefetch = t->prefetch;
    drop_graph(ctx);
    return SF_OK;
}

SF_API uint32_t sf_stage_count(void) { return sf::kNumStages; }

SF_API const char* sf_stage_name(uint32_t stage) { return stage < sf::kNumStages ? sf::kStageNames[stage] : ""; }

SF_API sf_status sf_profile_steps(sf_ctx* ctx, uint32_t nsteps, uint64_t flush_bytes, float* stage_ms,
                                  uint32_t nstages) {
    SF_TRY(need_sorted(ctx));
    if (!stage_ms || nstages != sf::kNumStages) return fail(SF_ERR_INVALID_ARGUMENT, "stage_ms needs sf_stage_count()");
    SF_TRY(set_device(ctx));
    for (uint32_t s = 0; s < nstages; ++s) stage_ms[s] = 0.f;
    if (!nsteps) return SF_OK;
    Scratch flush;
    if (flush_bytes) SF_CUDA(dev_malloc(&flush.p, flush_bytes));
    const size_t per = (size_t)sf::kNumStages + 1;
    EventSet ev;
    SF_CUDA(ev.create(per * nsteps));
    for (uint32_t i = 0; i < nsteps; ++i) {
        if (flush_bytes) SF_CUDA(cudaMemsetAsync(flush.p, (int)(i & 0xff), flush_bytes, ctx->stream));
        SF_CUDA(cudaEventRecord(ev.ev[per * i], ctx->stream));
        for (uint32_t s = 0; s < sf::kNumStages; ++s) {
            sf::enqueue_stage(s, ctx->d, ctx->c, ctx->stream);
            SF_CUDA(cudaEventRecord(ev.ev[per * i + s + 1], ctx->stream));
        }
    }
    SF_TRY(check_launch("profiled step"));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> acc(sf::kNumStages, 0.0);
    for (uint32_t i = 0; i < nsteps; ++i)
        for (uint32_t s = 0; s < sf::kNumStages; ++s) {
            float ms = 0.f;
            SF_CUDA(cudaEventElapsedTime(&ms, ev.ev[per * i + s], ev.ev[per * i + s + 1]));
            acc[s] += ms;
        }
    for (uint32_t s = 0; s < sf::kNumStages; ++s) stage_ms[s] = (float)acc[s];
    return SF_OK;
}

// Allocation-free density for callers that cannot allocate device memory;
// the sort scratch is a fixed static device array (sf_noalloc.cu).
SF_API sf_status sf_density_noalloc(const sf_params* p, const float* d_pos_xyz, uint32_t n, float* d_rho,
                                    float* d_pressure, void* stream) {
    if (!p) return fail(SF_ERR_INVALID_ARGUMENT, "null params");
    if (n && !d_pos_xyz) return fail(SF_ERR_INVALID_ARGUMENT, "null positions");
    if (n && !d_rho && !d_pressure) return fail(SF_ERR_INVALID_ARGUMENT, "no output");
    SF_TRY(validate(*p));
    sf::SimConst c;
    const char* why = "";
    int st = sf::derive_constants(*p, &c, &why);
    if (st) return fail(st, why);
    st = sf::noalloc_density(*p, c, d_pos_xyz, n, d_rho, d_pressure, static_cast<cudaStream_t>(stream), &why);
    if (st) return fail(st, why);
    return SF_OK;
}

// ---------------------------------------------------------------- rendering
SF_API sf_status sf_render_params_default(sf_render_params* rp) {
    if (!rp) return fail(SF_ERR_INVALID_ARGUMENT, "null render parameters");
    std::memset(rp, 0, sizeof(*rp));
    rp->width = 1200;  // FluidRenderWidget default size (Source/FluidRenderWidget.cpp:23)
    rp->height = 1000;
    const float eye[3] = {-3.0f, 0.8f, 0.0f}, focus[3] = {0.0f, -0.2f, 0.0f}, up[3] = {0.0f, 1.0f, 0.0f};
    for (int a = 0; a < 3; ++a) {
        rp->eye[a] = eye[a];  // DEFAULT_CAMERA_POSITION (Include/Common.h:21)
        rp->focus[a] = focus[a];  // DEFAULT_CAMERA_FOCUS (Include/Common.h:22)
        rp->up[a] = up[a];
    }
    rp->fovy_deg = 55.0f;  // Source/FluidRenderWidget.cpp:66
    rp->znear = 0.1f;
    rp->zfar = 1000.0f;
    rp->num_lights = 1;  // Source/FluidRenderWidget.cpp:91-93
    const float lp[4] = {-10.0f, 10.0f, 10.0f, 1.0f};
    for (int a = 0; a < 4; ++a) {
        rp->light_position[0][a] = lp[a];
        rp->light_ambient[0][a] = 1.0f;
        rp->light_diffuse[0][a] = 1.0f;
        rp->light_specular[0][a] = 1.0f;
    }
    // CUSTOM_PARTICLE_MATERIAL (Include/Common.h:24-31)
    const float ma = 0.2f * 0.2f, md[4] = {1.0f, 0.63f, 0.3f, 1.0f};
    for (int a = 0; a < 4; ++a) {
        rp->mat_ambient[a] = ma;
        rp->mat_diffuse[a] = md[a];
        rp->mat_specular[a] = 1.0f;
    }
    rp->mat_shininess = 250.0f;
    rp->color_mode = SF_COLOR_UNIFORM;
    rp->color_seed = 20171;
    return SF_OK;
}

SF_API sf_status sf_render(sf_ctx* ctx, const sf_render_params* rp, float* rgba_out, float* depth_out,
                           uint32_t* owner_out) {
    SF_RANGE("sf_render");
    SF_TRY(need_sorted(ctx));
    if (!rp) return fail(SF_ERR_INVALID_ARGUMENT, "null render parameters");
    if (rp->width <= 0 || rp->height <= 0 || (int64_t)rp->width * rp->height > (1 << 26))
        return fail(SF_ERR_INVALID_ARGUMENT, "image size out of range");
    if (rp->num_lights < 0 || rp->num_lights > 8) return fail(SF_ERR_INVALID_ARGUMENT, "num_lights must be 0..8");
    if (rp->color_mode < SF_COLOR_UNIFORM || rp->color_mode > SF_COLOR_RAMP)
        return fail(SF_ERR_INVALID_ARGUMENT, "unknown color_mode");
    if (!(rp->fovy_deg > 0.f && rp->fovy_deg < 180.f) || !(rp->znear > 0.f) || !(rp->zfar > rp->znear))
        return fail(SF_ERR_INVALID_ARGUMENT, "bad projection");
    SF_TRY(set_device(ctx));
    const uint32_t n = ctx->d.n;
    if (ctx->render_w != rp->width || ctx->render_h != rp->height || ctx->render_n < ctx->d.cap) {
        free_render(ctx);
        const size_t np = (size_t)rp->width * rp->height;
        SF_CUDA(dev_malloc(&ctx->render_keys, np * sizeof(unsigned long long)));
        SF_CUDA(dev_malloc(&ctx->render_rgba, np * sizeof(float4)));
        SF_CUDA(dev_malloc(&ctx->render_depth, np * sizeof(float)));
        SF_CUDA(dev_malloc(&ctx->render_owner, np * sizeof(uint32_t)));
        SF_CUDA(dev_malloc(&ctx->render_slot, (size_t)ctx->d.cap * sizeof(uint32_t)));
        ctx->render_w = rp->width;
        ctx->render_h = rp->height;
        ctx->render_n = ctx->d.cap;
    }
    sf::RenderConst rc;
    sf::build_render_const(*rp, ctx->params.particle_radius, n, &rc);
    sf::launch_render(ctx->d.pos, n, rc, ctx->render_keys, ctx->render_slot, ctx->render_rgba, ctx->render_depth,
                      ctx->render_owner, ctx->stream);
    SF_TRY(check_launch("render"));
    const size_t np = (size_t)rp->width * rp->height;
    if (rgba_out) SF_TRY(copy_out(ctx, rgba_out, ctx->render_rgba, np * sizeof(float4)));
    if (depth_out) SF_TRY(copy_out(ctx, depth_out, ctx->render_depth, np * sizeof(float)));
    if (owner_out) SF_TRY(copy_out(ctx, owner_out, ctx->render_owner, np * sizeof(uint32_t)));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

// ---------------------------------------------------------------- state files
// Layout (little endian): "SFSTATE1", u32 version = 1, u32 n, f64 sim_time,
// sf_params, then n x 3 f32 positions, n x 3 f32 velocities and n u32
// particle indices, all in the solver's cell-sorted order.  Loading restores
// that order, so stepping a loaded state reproduces the saved run bit for bit.
// The n x 3 arrays can be read directly for offline use; particle i of the
// caller's order is at the row whose index entry is i.
SF_API sf_status sf_save_state(sf_ctx* ctx, const char* path, double sim_time) {
    SF_RANGE("sf_save_state");
    SF_TRY(need_sorted(ctx));
    if (!path) return fail(SF_ERR_INVALID_ARGUMENT, "null path");
    SF_TRY(set_device(ctx));
    const uint32_t n = ctx->d.n;
    uint32_t* ids_dev = ctx->d.tmp;
    sf::launch_store_sorted(ctx->d.pos, ctx->d.vel, n, ctx->d.io, ctx->d.io + 3 * (size_t)n, ids_dev, ctx->stream);
    SF_TRY(check_launch("store sorted"));
    std::vector<float> pv(6 * (size_t)n);
    std::vector<uint32_t> ids(n);
    SF_TRY(copy_out(ctx, pv.data(), ctx->d.io, pv.size() * sizeof(float)));
    SF_TRY(copy_out(ctx, ids.data(), ids_dev, ids.size() * sizeof(uint32_t)));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(SF_ERR_INVALID_ARGUMENT, std::string("cannot open for writing: ") + path);
    const char magic[8] = {'S', 'F', 'S', 'T', 'A', 'T', 'E', '1'};
    const uint32_t version = 1;
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(&version, 4, 1, f) == 1 && std::fwrite(&n, 4, 1, f) == 1 &&
              std::fwrite(&sim_time, 8, 1, f) == 1 && std::fwrite(&ctx->params, sizeof(sf_params), 1, f) == 1 &&
              std::fwrite(pv.data(), sizeof(float), pv.size(), f) == pv.size() &&
              std::fwrite(ids.data(), sizeof(uint32_t), ids.size(), f) == ids.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(SF_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
    return SF_OK;
}

SF_API sf_status sf_load_state(sf_ctx* ctx, const char* path, double* sim_time_out) {
    SF_RANGE("sf_load_state");
    SF_TRY(need_ctx(ctx));
    if (!path) return fail(SF_ERR_INVALID_ARGUMENT, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SF_ERR_INVALID_ARGUMENT, std::string("cannot open: ") + path);
    char magic[8];
    uint32_t version = 0, n = 0;
    double t = 0.0;
    sf_params p{};
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "SFSTATE1", 8) == 0 &&
              std::fread(&version, 4, 1, f) == 1 && version == 1 && std::fread(&n, 4, 1, f) == 1 &&
              std::fread(&t, 8, 1, f) == 1 && std::fread(&p, sizeof(sf_params), 1, f) == 1;
    std::vector<float> pv;
    std::vector<uint32_t> ids;
    if (ok) {
        pv.resize(6 * (size_t)n);
        ids.resize(n);
        ok = std::fread(pv.data(), sizeof(float), pv.size(), f) == pv.size() &&
             std::fread(ids.data(), sizeof(uint32_t), ids.size(), f) == ids.size();
    }
    std::fclose(f);
    if (!ok) return fail(SF_ERR_INVALID_ARGUMENT, std::string("not a valid state file: ") + path);
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t id : ids) {
        if (id >= n || seen[id]) return fail(SF_ERR_INVALID_ARGUMENT, "state file indices are not a permutation");
        seen[id] = 1;
    }
    SF_TRY(sf_set_params(ctx, &p));
    SF_TRY(set_device(ctx));
    const bool resized = n != ctx->d.n;
    SF_TRY(alloc_particles(ctx, n));
    if (resized) drop_graph(ctx);
    ctx->d.n = n;
    ctx->sorted = false;
    if (n) {
        sf::DeviceState& d = ctx->d;
        SF_TRY(copy_in(ctx, d.io, pv.data(), pv.size() * sizeof(float)));
        SF_TRY(copy_in(ctx, d.tmp, ids.data(), ids.size() * sizeof(uint32_t)));
        sf::launch_load_sorted(d.io, d.io + 3 * (size_t)n, d.tmp, n, d.pos2, d.vel2, ctx->stream);
        sf::launch_hash_count(d, d.pos2, n, ctx->c, d.counts, d.key_slot, ctx->stream);
        sf::enqueue_sort_tail(d, ctx->stream);
        if (ctx->c.adaptive) sf::launch_init_maxima(d.vel, n, ctx->frame, ctx->stream);
        SF_TRY(check_launch("load state"));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->sorted = true;
    }
    if (sim_time_out) *sim_time_out = t;
    return SF_OK;
}

// ---------------------------------------------------------------- batches
// A batch is one engine (stream, graph, particle and cell buffers) over the
// concatenation of all scenes' particles, with a per-scene constant table and
// the scenes' particle offsets in device memory.  Scene s owns cell keys
// [cell_base_s, cell_base_s + ncells_s), so one counting sort keeps every
// scene's particles contiguous (sorted positions [off_s, off_{s+1})).
}  // extern "C"

struct sf_batch {
    sf_ctx eng;
    std::vector<sf_params> params;
    std::vector<sf::SimConst> consts;
    std::vector<uint32_t> counts;  // particles per scene
    sf::SimConst* d_table = nullptr;
    uint32_t* d_off = nullptr;
};

namespace {

sf_status batch_derive(sf_batch* b, int K) {
    uint64_t base = 0;
    std::vector<sf::SimConst> consts(b->params.size());
    for (size_t s = 0; s < b->params.size(); ++s) {
        sf_params p = b->params[s];
        p.cells_per_h = K;
        SF_TRY(validate(p));
        const char* why = "";
        const int st = sf::derive_constants(p, &consts[s], &why);
        if (st) return fail(st, std::string("scene ") + std::to_string(s) + ": " + why);
        consts[s].cell_base = (uint32_t)base;
        base += consts[s].ncells;
        if (base > kMaxCells) return fail(SF_ERR_GRID_TOO_LARGE, "batch needs more than 2^28 grid cells in total");
    }
    for (auto& p : b->params) p.cells_per_h = K;
    b->consts = consts;
    b->eng.params = b->params[0];
    b->eng.c = consts[0];
    b->eng.c.cell_base = 0;
    b->eng.c.ncells = (uint32_t)base;
    return SF_OK;
}

sf_status batch_upload_table(sf_batch* b) {
    const size_t ns = b->consts.size();
    if (!b->d_table) SF_CUDA(dev_malloc(&b->d_table, ns * sizeof(sf::SimConst)));
    SF_CUDA(cudaMemcpyAsync(b->d_table, b->consts.data(), ns * sizeof(sf::SimConst), cudaMemcpyHostToDevice,
                            b->eng.stream));
    SF_CUDA(cudaStreamSynchronize(b->eng.stream));
    b->eng.d.table = b->d_table;
    b->eng.d.scene_off = b->d_off;
    b->eng.d.nscenes = (uint32_t)ns;
    return SF_OK;
}

sf_status need_batch(const sf_batch* b) {
    if (!b) return fail(SF_ERR_INVALID_ARGUMENT, "null batch");
    return SF_OK;
}

}  // namespace

extern "C" {

SF_API sf_status sf_batch_cubes(uint64_t seed, uint32_t nscenes, const sf_params* base, sf_params* params_out,
                                uint32_t* counts_out, float* pos_xyz, uint64_t capacity, uint64_t* total_out) {
    if (!base || nscenes == 0) return fail(SF_ERR_INVALID_ARGUMENT, "need base parameters and scenes");
    std::vector<sf_params> params;
    std::vector<uint32_t> counts;
    std::vector<float> pos;
    const char* why = "";
    const int st = sf::batch_cubes(seed, nscenes, *base, params, counts, pos, &why);
    if (st) return fail(st, why);
    const uint64_t total = pos.size() / 3;
    if (total_out) *total_out = total;
    if (params_out) std::memcpy(params_out, params.data(), params.size() * sizeof(sf_params));
    if (counts_out) std::memcpy(counts_out, counts.data(), counts.size() * sizeof(uint32_t));
    if (pos_xyz) {
        if (capacity < total) return fail(SF_ERR_CAPACITY, "position buffer too small");
        std::memcpy(pos_xyz, pos.data(), pos.size() * sizeof(float));
    }
    return SF_OK;
}

SF_API sf_status sf_batch_create(const sf_params* per_scene, uint32_t nscenes, sf_batch** out) {
    if (!per_scene || !out || nscenes == 0) return fail(SF_ERR_INVALID_ARGUMENT, "need at least one scene");
    *out = nullptr;
    const int K = per_scene[0].cells_per_h ? per_scene[0].cells_per_h : 2;
    for (uint32_t s = 0; s < nscenes; ++s) {
        const int Ks = per_scene[s].cells_per_h ? per_scene[s].cells_per_h : 2;
        if (Ks != K) return fail(SF_ERR_INVALID_ARGUMENT, "all scenes of a batch must share cells_per_h");
    }
    if (K > 2) return fail(SF_ERR_INVALID_ARGUMENT, "batches support cells_per_h 1 or 2");
    for (uint32_t s = 0; s < nscenes; ++s)
        if (per_scene[s].adaptive_time_step) return fail(SF_ERR_INVALID_ARGUMENT, "batches use a fixed time step");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SF_ERR_NO_DEVICE, "no CUDA device available");
    }
    sf_batch* b = new sf_batch();
    b->params.assign(per_scene, per_scene + nscenes);
    b->counts.assign(nscenes, 0);
    sf_status st = batch_derive(b, K);
    if (st) {
        delete b;
        return st;
    }
    cudaError_t e = cudaGetDevice(&b->eng.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->eng.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dev_malloc(&b->d_off, (nscenes + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_off, 0, (nscenes + 1) * sizeof(uint32_t), b->eng.stream);
    if (e != cudaSuccess) {
        sf_batch_destroy(b);
        return cuda_fail(e, "batch creation");
    }
    st = alloc_grid(&b->eng);
    if (!st) st = batch_upload_table(b);
    if (st) {
        sf_batch_destroy(b);
        return st;
    }
    *out = b;
    return SF_OK;
}

SF_API sf_status sf_batch_destroy(sf_batch* b) {
    if (!b) return SF_OK;
    release_ctx(&b->eng);
    if (b->d_table) cudaFree(b->d_table);
    if (b->d_off) cudaFree(b->d_off);
    delete b;
    return SF_OK;
}

SF_API sf_status sf_batch_num_scenes(const sf_batch* b, uint32_t* n_out) {
    SF_TRY(need_batch(b));
    if (!n_out) return fail(SF_ERR_INVALID_ARGUMENT, "null output");
    *n_out = (uint32_t)b->params.size();
    return SF_OK;
}

SF_API sf_status sf_batch_get_params(const sf_batch* b, uint32_t scene, sf_params* p) {
    SF_TRY(need_batch(b));
    if (!p || scene >= b->params.size()) return fail(SF_ERR_INVALID_ARGUMENT, "bad scene or output");
    *p = b->params[scene];
    return SF_OK;
}

SF_API sf_status sf_batch_set_state(sf_batch* b, const uint32_t* counts, const float* pos_xyz, const float* vel_xyz) {
    SF_TRY(need_batch(b));
    if (!counts) return fail(SF_ERR_INVALID_ARGUMENT, "null counts");
    const size_t ns = b->params.size();
    std::vector<uint32_t> off(ns + 1, 0);
    for (size_t s = 0; s < ns; ++s) {
        const uint64_t next = (uint64_t)off[s] + counts[s];
        if (next > 0xffffffffull) return fail(SF_ERR_CAPACITY, "more than 2^32-1 particles in a batch");
        off[s + 1] = (uint32_t)next;
    }
    SF_TRY(set_device(&b->eng));
    SF_CUDA(cudaStreamSynchronize(b->eng.stream));
    SF_CUDA(cudaMemcpy(b->d_off, off.data(), off.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    b->counts.assign(counts, counts + ns);
    return sf_set_state(&b->eng, pos_xyz, vel_xyz, off[ns]);
}

SF_API sf_status sf_batch_get_state(sf_batch* b, float* pos_xyz, float* vel_xyz, uint32_t n) {
    SF_TRY(need_batch(b));
    return sf_get_state(&b->eng, pos_xyz, vel_xyz, n);
}

SF_API sf_status sf_batch_num_particles(const sf_batch* b, uint32_t* n_out) {
    SF_TRY(need_batch(b));
    return sf_get_num_particles(&b->eng, n_out);
}

SF_API sf_status sf_batch_step(sf_batch* b, uint32_t nsteps) {
    SF_TRY(need_batch(b));
    return sf_step(&b->eng, nsteps);
}

SF_API sf_status sf_batch_check_state(sf_batch* b, sf_state_report* report) {
    SF_TRY(need_batch(b));
    return sf_check_state(&b->eng, report);
}

SF_API sf_status sf_batch_synchronize(sf_batch* b) {
    SF_TRY(need_batch(b));
    return sf_synchronize(&b->eng);
}

SF_API sf_status sf_batch_step_timed(sf_batch* b, uint32_t nsteps, uint64_t flush_bytes, float* total_ms,
                                     float* step_ms) {
    SF_TRY(need_batch(b));
    return sf_step_timed(&b->eng, nsteps, flush_bytes, total_ms, step_ms);
}

SF_API sf_status sf_batch_get_tuning(const sf_batch* b, sf_tuning* t) {
    SF_TRY(need_batch(b));
    return sf_get_tuning(&b->eng, t);
}

SF_API sf_status sf_batch_set_tuning(sf_batch* b, const sf_tuning* t) {
    SF_TRY(need_batch(b));
    if (t && t->prefetch != 2) return fail(SF_ERR_INVALID_ARGUMENT, "batches use prefetch 2");
    return sf_set_tuning(&b->eng, t);
}

SF_API sf_status sf_batch_set_cells_per_h(sf_batch* b, int32_t cells_per_h) {
    SF_TRY(need_batch(b));
    if (cells_per_h != 1 && cells_per_h != 2) return fail(SF_ERR_INVALID_ARGUMENT, "batches support cells_per_h 1 or 2");
    SF_TRY(set_device(&b->eng));
    SF_CUDA(cudaStreamSynchronize(b->eng.stream));
    SF_TRY(batch_derive(b, cells_per_h));
    drop_graph(&b->eng);
    SF_TRY(alloc_grid(&b->eng));
    SF_TRY(batch_upload_table(b));
    sf::DeviceState& d = b->eng.d;
    if (b->eng.sorted && d.n) {
        // re-bucket the current state on the new grids (positions unchanged)
        SF_CUDA(cudaMemcpyAsync(d.pos2, d.pos, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice, b->eng.stream));
        SF_CUDA(cudaMemcpyAsync(d.vel2, d.vel, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice, b->eng.stream));
        sf::launch_hash_count(d, d.pos2, d.n, b->eng.c, d.counts, d.key_slot, b->eng.stream);
        sf::enqueue_sort_tail(d, b->eng.stream);
        SF_TRY(check_launch("batch re-sort"));
    }
    return SF_OK;
}

// Autotuner: times `trial_steps` graph-replayed steps (after 2 warm-up steps)
// of every candidate configuration — grid granularity K and the kernel
// variants — each from the same snapshot of the current state, keeps the
// fastest, and restores the snapshot.  The chosen K changes the summation
// order (and so the last bits); the kernel variants do not.
SF_API sf_status sf_batch_autotune(sf_batch* b, uint32_t trial_steps, sf_tuning* chosen, int32_t* chosen_cells_per_h,
                                   float* chosen_ms_per_step) {
    SF_RANGE("sf_batch_autotune");
    SF_TRY(need_batch(b));
    SF_TRY(need_sorted(&b->eng));
    if (trial_steps == 0) return fail(SF_ERR_INVALID_ARGUMENT, "trial_steps must be > 0");
    const uint32_t n = b->eng.d.n;
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n);
    SF_TRY(sf_get_state(&b->eng, pos.data(), vel.data(), n));
    const std::vector<uint32_t> counts = b->counts;
    struct Cand {
        int K;
        sf_tuning t;
    };
    std::vector<Cand> cands;
    for (int K : {1, 2})
        for (int mode : {SF_LIST_TILE_STAGED, SF_LIST_TILE})
            for (int db : {128, 256})
                for (int fb : {128, 256}) {
                    if (mode == SF_LIST_TILE_STAGED && db != 128) continue;
                    sf_tuning t{};
                    t.list_mode = mode;
                    t.density_block = db;
                    t.force_block = fb;
                    t.prefetch = 2;
                    cands.push_back({K, t});
                }
    float best = 0.f;
    size_t best_i = 0;
    for (size_t ci = 0; ci < cands.size(); ++ci) {
        SF_TRY(sf_batch_set_cells_per_h(b, cands[ci].K));
        SF_TRY(sf_batch_set_state(b, counts.data(), pos.data(), vel.data()));
        SF_TRY(sf_set_tuning(&b->eng, &cands[ci].t));
        SF_TRY(sf_step(&b->eng, 2));
        float ms = 0.f;
        SF_TRY(sf_step_timed(&b->eng, trial_steps, 0, &ms, nullptr));
        if (ci == 0 || ms < best) {
            best = ms;
            best_i = ci;
        }
    }
    SF_TRY(sf_batch_set_cells_per_h(b, cands[best_i].K));
    SF_TRY(sf_batch_set_state(b, counts.data(), pos.data(), vel.data()));
    SF_TRY(sf_set_tuning(&b->eng, &cands[best_i].t));
    if (chosen) *chosen = cands[best_i].t;
    if (chosen_cells_per_h) *chosen_cells_per_h = cands[best_i].K;
    if (chosen_ms_per_step) *chosen_ms_per_step = best / (float)trial_steps;
    return SF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- adjoint
namespace {

// A failed trajectory allocation releases the whole trajectory, so that no
// partly allocated record set is ever used.
#define SF_ALLOC_TRAJ(ptr, bytes)                                  \
    do {                                                           \
        const cudaError_t e_ = dev_malloc(&(ptr), (bytes));        \
        if (e_ != cudaSuccess) {                                   \
            free_trajectory(ctx);                                  \
            return cuda_fail(e_, "trajectory allocation");         \
        }                                                          \
    } while (0)

sf_status ensure_work(sf_ctx* ctx) {
    sf::Trajectory* t = ctx->traj;
    const size_t n = ctx->d.cap;
    sf::AdjointWork& w = t->w;
    if (w.Xb) return SF_OK;
    SF_ALLOC_TRAJ(w.Xb, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.Vb, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.apb, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.avb, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.xdir, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.vdir, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.xf, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.vf, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.rhob, n * sizeof(float));
    SF_ALLOC_TRAJ(w.scalars, 2 * sizeof(double));
    SF_ALLOC_TRAJ(t->snap, 2 * n * sizeof(float4));
    return SF_OK;
}

sf_status ensure_records(sf_ctx* ctx, uint32_t ckpt) {
    sf::Trajectory* t = ctx->traj;
    const size_t n = ctx->d.cap;
    const size_t tiles = (n + sf::kNbTile - 1) / sf::kNbTile;
    if (t->rec.size() == ckpt && t->ncells_pad == ctx->d.ncells_pad && t->stage) return SF_OK;
    drop_segment_graphs(t);
    for (auto& r : t->rec) free_rec(r);
    if (t->stage) cudaFree(t->stage);
    if (t->seg_partial) cudaFree(t->seg_partial);
    t->stage = nullptr;
    t->seg_partial = nullptr;
    SF_ALLOC_TRAJ(t->stage, 2 * n * sizeof(float4));
    SF_ALLOC_TRAJ(t->seg_partial, (size_t)ckpt * sf::adjoint_partial_count((uint32_t)n) * sizeof(double2));
    t->rec.assign(ckpt, sf::StepRec{});
    t->ncells_pad = ctx->d.ncells_pad;
    for (auto& r : t->rec) {
        SF_ALLOC_TRAJ(r.pos, n * sizeof(float4));
        SF_ALLOC_TRAJ(r.vel, n * sizeof(float4));
        SF_ALLOC_TRAJ(r.pr, n * sizeof(float2));
        SF_ALLOC_TRAJ(r.rho, n * sizeof(float));
        SF_ALLOC_TRAJ(r.nbr, tiles * sf::kNbCap * sf::kNbTile * sizeof(uint32_t));
        SF_ALLOC_TRAJ(r.cnt, n * sizeof(uint32_t));
        SF_ALLOC_TRAJ(r.cs, (size_t)ctx->d.ncells_pad * sizeof(uint32_t));
        SF_ALLOC_TRAJ(r.sums, 2 * n * sizeof(float4));
    }
    return SF_OK;
}

// Put a sorted state (2n float4: pos then vel) back and rebuild the cell table.
sf_status restore_sorted(sf_ctx* ctx, const float4* state) {
    sf::DeviceState& d = ctx->d;
    SF_CUDA(cudaMemcpyAsync(d.pos2, state, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(d.vel2, state + d.n, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    sf::launch_hash_count(d, d.pos2, d.n, ctx->c, d.counts, d.key_slot, ctx->stream);
    sf::enqueue_sort_tail(d, ctx->stream);
    return check_launch("restore state");
}

sf_status upload_by_id(sf_ctx* ctx, float4* dst, const float* src_xyz) {
    const uint32_t n = ctx->d.n;
    std::vector<float4> h(n);
    for (uint32_t i = 0; i < n; ++i)
        h[i] = src_xyz ? make_float4(src_xyz[3 * (size_t)i], src_xyz[3 * (size_t)i + 1], src_xyz[3 * (size_t)i + 2], 0.f)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    SF_CUDA(cudaMemcpyAsync(dst, h.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

sf_status download_by_id(sf_ctx* ctx, float* dst_xyz, const float4* src) {
    if (!dst_xyz) return SF_OK;
    const uint32_t n = ctx->d.n;
    std::vector<float4> h(n);
    SF_TRY(copy_out(ctx, h.data(), src, (size_t)n * sizeof(float4)));
    for (uint32_t i = 0; i < n; ++i) {
        dst_xyz[3 * (size_t)i] = h[i].x;
        dst_xyz[3 * (size_t)i + 1] = h[i].y;
        dst_xyz[3 * (size_t)i + 2] = h[i].z;
    }
    return SF_OK;
}

// Capture one segment of `len` steps: rebuild the cell table of the
// checkpoint in t->stage, re-run the steps forward recording each step's
// inputs in its slot (the sort of step s writes the state of step s+1 straight
// into slot s+1), then the reverse sweep and the scalar accumulation.
sf_status build_segment_graph(sf_ctx* ctx, uint32_t len, cudaGraphExec_t* out) {
    sf::Trajectory* t = ctx->traj;
    sf::DeviceState& d = ctx->d;
    const uint32_t n = d.n;
    cudaStream_t st = ctx->stream;
    cudaGraph_t g = nullptr;
    SF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    sf::DeviceState r0 = d;
    r0.pos2 = t->stage;
    r0.vel2 = t->stage + n;
    r0.pos = t->rec[0].pos;
    r0.vel = t->rec[0].vel;
    r0.cell_start = t->rec[0].cs;
    sf::launch_hash_count(r0, r0.pos2, n, ctx->c, r0.counts, r0.key_slot, st);
    sf::enqueue_sort_tail(r0, st);
    for (uint32_t s = 0; s < len; ++s) {
        const sf::StepRec& r = t->rec[s];
        sf::DeviceState ds = d;
        ds.pos = r.pos;
        ds.vel = r.vel;
        ds.cell_start = r.cs;
        ds.pr = r.pr;
        ds.rho = r.rho;
        ds.nbr = r.nbr;
        ds.nbr_count = r.cnt;
        ds.sums = r.sums;
        if (ds.tune.list_mode == SF_LIST_NONE) ds.tune.list_mode = SF_LIST_TILE;
        sf::launch_density(ds, ctx->c, st);
        sf::launch_force_integrate(ds, ctx->c, st);
        sf::DeviceState dn = d;
        if (s + 1 < len) {
            dn.pos = t->rec[s + 1].pos;
            dn.vel = t->rec[s + 1].vel;
            dn.cell_start = t->rec[s + 1].cs;
        }
        sf::enqueue_sort_tail(dn, st);
    }
    const uint32_t nb = sf::adjoint_partial_count(n);
    for (int64_t s = (int64_t)len - 1; s >= 0; --s) {
        const sf::StepRec& r = t->rec[s];
        sf::AdjointStep as;
        as.n = n;
        as.pos = r.pos;
        as.vel = r.vel;
        as.pr = r.pr;
        as.rho = r.rho;
        as.nbr = r.nbr;
        as.cnt = r.cnt;
        as.cs = r.cs;
        as.sums = r.sums;
        sf::launch_adjoint_step(as, ctx->c, t->w, t->seg_partial + (size_t)s * nb, st);
    }
    sf::launch_adjoint_accumulate(t->seg_partial, len, n, t->w.scalars, st);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(adjoint segment)");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate(adjoint segment)");
    }
    return SF_OK;
}

sf_status segment_graph(sf_ctx* ctx, uint32_t len, cudaGraphExec_t* out) {
    sf::Trajectory* t = ctx->traj;
    for (int k = 0; k < 2; ++k)
        if (t->seg_graph[k] && t->seg_len[k] == len) {
            *out = t->seg_graph[k];
            return SF_OK;
        }
    int slot = t->seg_graph[0] ? 1 : 0;
    if (t->seg_graph[slot]) cudaGraphExecDestroy(t->seg_graph[slot]);
    t->seg_graph[slot] = nullptr;
    SF_TRY(build_segment_graph(ctx, len, &t->seg_graph[slot]));
    t->seg_len[slot] = len;
    *out = t->seg_graph[slot];
    return SF_OK;
}

}  // namespace

extern "C" {

SF_API sf_status sf_forward(sf_ctx* ctx, uint32_t nsteps, uint32_t ckpt_every) {
    SF_RANGE("sf_forward");
    SF_TRY(sf_make_ready(ctx));
    if (ctx->c.adaptive) return fail(SF_ERR_INVALID_ARGUMENT, "differentiation needs a fixed time step");
    if (ckpt_every == 0) return fail(SF_ERR_INVALID_ARGUMENT, "ckpt_every must be > 0");
    if (!ctx->traj) ctx->traj = new sf::Trajectory();
    sf::Trajectory* t = ctx->traj;
    sf::DeviceState& d = ctx->d;
    const uint32_t nck = (nsteps + ckpt_every - 1) / ckpt_every;
    t->valid = false;
    if (t->n != d.cap || t->ck.size() != nck) {
        for (float4* p : t->ck)
            if (p) cudaFree(p);
        t->ck.assign(nck, nullptr);
        t->n = 0;
        for (auto& p : t->ck) SF_ALLOC_TRAJ(p, 2 * (size_t)d.cap * sizeof(float4));
    }
    t->valid = false;
    for (uint32_t s = 0; s < nsteps; ++s) {
        if (s % ckpt_every == 0) {
            float4* c = t->ck[s / ckpt_every];
            SF_CUDA(cudaMemcpyAsync(c, d.pos, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
            SF_CUDA(cudaMemcpyAsync(c + d.n, d.vel, (size_t)d.n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
        }
        SF_CUDA(cudaGraphLaunch(ctx->step_graph, ctx->stream));
    }
    t->nsteps = nsteps;
    t->ckpt = ckpt_every;
    t->n = d.cap;
    t->valid = true;
    return SF_OK;
}

SF_API sf_status sf_loss_histogram(sf_ctx* ctx, const float* target, uint32_t res, double* loss_out, float* dloss_dx) {
    SF_RANGE("sf_loss_histogram");
    SF_TRY(need_sorted(ctx));
    if (!target || res == 0 || res > 1024 || !loss_out) return fail(SF_ERR_INVALID_ARGUMENT, "bad target or resolution");
    SF_TRY(set_device(ctx));
    if (!ctx->traj) ctx->traj = new sf::Trajectory();
    sf::Trajectory* t = ctx->traj;
    SF_TRY(ensure_work(ctx));
    const size_t nc = (size_t)res * res * res;
    if (t->hist_res != res) {
        if (t->hist) cudaFree(t->hist);
        if (t->e2) cudaFree(t->e2);
        if (t->target) cudaFree(t->target);
        if (t->hpartial) cudaFree(t->hpartial);
        t->hist = nullptr;
        t->e2 = t->target = nullptr;
        t->hpartial = nullptr;
        SF_ALLOC_TRAJ(t->hist, nc * sizeof(unsigned long long));
        SF_ALLOC_TRAJ(t->e2, nc * sizeof(float));
        SF_ALLOC_TRAJ(t->target, nc * sizeof(float));
        SF_ALLOC_TRAJ(t->hpartial, sf::histogram_partial_count(res) * sizeof(double));
        t->hist_res = res;
    }
    SF_TRY(copy_in(ctx, t->target, target, nc * sizeof(float)));
    float ext[3];
    for (int a = 0; a < 3; ++a) ext[a] = (float)((double)ctx->params.box_max[a] - (double)ctx->params.box_min[a]);
    sf::launch_histogram_loss(ctx->d.pos, ctx->d.n, ctx->c, ext, res, t->target, t->hist, t->e2, t->hpartial, t->w.Xb,
                              ctx->stream);
    SF_TRY(check_launch("histogram loss"));
    std::vector<double> part(sf::histogram_partial_count(res));
    SF_TRY(copy_out(ctx, part.data(), t->hpartial, part.size() * sizeof(double)));
    double L = 0.0;
    for (double v : part) L += v;
    *loss_out = L;
    return download_by_id(ctx, dloss_dx, t->w.Xb);
}

SF_API sf_status sf_adjoint(sf_ctx* ctx, const float* dloss_dx, const float* dloss_dv, float* dloss_dx0,
                            float* dloss_dv0, float* dloss_dviscosity, float* dloss_dstiffness) {
    SF_RANGE("sf_adjoint");
    SF_TRY(need_sorted(ctx));
    sf::Trajectory* t = ctx->traj;
    if (!t || !t->valid || t->n != ctx->d.cap) return fail(SF_ERR_NOT_READY, "no recorded trajectory: call sf_forward");
    SF_TRY(set_device(ctx));
    SF_TRY(ensure_work(ctx));
    SF_TRY(ensure_records(ctx, t->ckpt));
    if (t->graph_gen != ctx->gen) {
        drop_segment_graphs(t);
        t->graph_gen = ctx->gen;
    }
    sf::DeviceState& d = ctx->d;
    const uint32_t n = d.n;
    sf::AdjointWork& w = t->w;
    // keep the forward's final state to put back afterwards
    SF_CUDA(cudaMemcpyAsync(t->snap, d.pos, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(t->snap + n, d.vel, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    SF_TRY(upload_by_id(ctx, w.Xb, dloss_dx));
    SF_TRY(upload_by_id(ctx, w.Vb, dloss_dv));
    SF_CUDA(cudaMemsetAsync(w.scalars, 0, 2 * sizeof(double), ctx->stream));
    const uint32_t nck = (uint32_t)t->ck.size();
    for (int64_t seg = (int64_t)nck - 1; seg >= 0; --seg) {
        const uint32_t s0 = (uint32_t)seg * t->ckpt, len = std::min(t->nsteps, s0 + t->ckpt) - s0;
        cudaGraphExec_t g = nullptr;
        SF_TRY(segment_graph(ctx, len, &g));
        SF_CUDA(cudaMemcpyAsync(t->stage, t->ck[seg], 2 * (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                ctx->stream));
        SF_CUDA(cudaGraphLaunch(g, ctx->stream));
    }
    SF_TRY(download_by_id(ctx, dloss_dx0, w.Xb));
    SF_TRY(download_by_id(ctx, dloss_dv0, w.Vb));
    double sc[2];
    SF_TRY(copy_out(ctx, sc, w.scalars, sizeof(sc)));
    const double kPi = 3.14159265358979323846;
    const double h = ctx->params.kernel_radius, r = ctx->params.particle_radius;
    const double mass = (double)ctx->params.rest_density * (2.0 * r) * (2.0 * r) * (2.0 * r);
    const double h6 = h * h * h * h * h * h;
    if (dloss_dviscosity) *dloss_dviscosity = (float)(sc[0] * (mass * 45.0 / (kPi * h6)));
    if (dloss_dstiffness) *dloss_dstiffness = (float)sc[1];
    SF_TRY(restore_sorted(ctx, t->snap));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
}

}  // extern "C"
