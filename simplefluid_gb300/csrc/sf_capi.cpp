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
#include "sf_capi_impl.h"

namespace sf {
namespace capi {

namespace {

thread_local std::string g_error;

// Fault injection (sf_test_fail_allocation): device allocations to let
// through before one fails as out of memory; negative when disarmed.
std::atomic<int64_t> g_fail_alloc{-1};

}  // namespace

void set_fail_allocation(int64_t after) { g_fail_alloc.store(after < 0 ? -1 : after); }


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

sf_status fail(sf_status st, const std::string& msg) {
    g_error = msg;
    return st;
}

sf_status cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();  // clear a sticky launch error where possible
    return fail(e == cudaErrorMemoryAllocation ? SF_ERR_OUT_OF_MEMORY : SF_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

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
                    d.nbr_wide, d.pv};
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
    d.nbr_wide = nullptr;
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
    void* b[] = {r.pos, r.vel, r.pr, r.rho, r.nbr, r.cnt, r.cs, r.sums, r.pv};
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
    void* b[] = {t->snap, t->w.Xb, t->w.Vb, t->w.ab, t->w.xdir, t->w.vdir, t->w.xf, t->w.vf,
                 t->w.xrb, t->w.scalars, t->hist, t->e2, t->target, t->hpartial};
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
    // queued work (a step, or the sort an upload left running) may still use the old buffers
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
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
    if (e == cudaSuccess) e = dev_malloc(&d.nbr_wide, tiles * (sf::kNbTile / sf::kNbWarpTile));
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

// The second stream and its events, made on first use.
sf_status need_aux(sf_ctx* ctx) {
    if (!ctx->aux) SF_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
    for (cudaEvent_t* ev : {&ctx->ev_pos, &ctx->ev_vel, &ctx->ev_in, &ctx->ev_out})
        if (!*ev) SF_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    return SF_OK;
}

// Upload from page-locked host arrays: positions first, then the velocity
// copy on the second stream while the positions are hashed, counted and
// scattered; the gather waits for the velocities.  ev_in marks the end of
// both copies (the velocity copy starts after the position copy).
sf_status upload_overlapped(sf_ctx* ctx, const float* pos_xyz, const float* vel_xyz) {
    sf::DeviceState& d = ctx->d;
    SF_TRY(need_aux(ctx));
    const size_t bytes = (size_t)d.n * 3 * sizeof(float);
    float* io_pos = d.io;
    float* io_vel = d.io + 3 * (size_t)d.n;
    SF_CUDA(cudaMemcpyAsync(io_pos, pos_xyz, bytes, cudaMemcpyHostToDevice, ctx->stream));
    SF_CUDA(cudaEventRecord(ctx->ev_pos, ctx->stream));
    SF_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->ev_pos, 0));  // after all earlier work on io
    SF_CUDA(cudaMemcpyAsync(io_vel, vel_xyz, bytes, cudaMemcpyHostToDevice, ctx->aux));
    SF_CUDA(cudaEventRecord(ctx->ev_in, ctx->aux));
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
        dr.frame = ctx->frame;  // the density pass chooses dt, the force pass reads it
        sf::enqueue_step(dr, ctx->c, ctx->stream);
    } else {
        sf::enqueue_step(ctx->d, ctx->c, ctx->stream);
    }
}

sf_status capture_step(sf_ctx* ctx) {
    drop_graph(ctx);
    // the gather records' persisting-L2 window (reserved outside the capture)
    if (ctx->d.tune.l2_window) sf::reserve_persisting_l2((size_t)ctx->d.n * 2 * sizeof(float4));
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

// Fewer than this many particles fill few warps per SM: each force-pass thread
// then keeps four neighbours in flight instead of two (measured 5-6% faster
// steps at 16k-64k particles; two are faster at 1M).
constexpr uint32_t kSmallScene = 262144;

void apply_size_defaults(sf_ctx* ctx) {
    if (ctx->tune_explicit || ctx->d.table) return;  // batches use prefetch 2
    const int pf = ctx->d.n < kSmallScene ? 4 : 2;
    if (ctx->d.tune.prefetch != pf) {
        ctx->d.tune.prefetch = pf;
        drop_graph(ctx);
    }
}

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
    for (cudaEvent_t* ev : {&ctx->ev_pos, &ctx->ev_vel, &ctx->ev_in, &ctx->ev_out}) {
        if (*ev) cudaEventDestroy(*ev);
        *ev = nullptr;
    }
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    ctx->aux = nullptr;
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = nullptr;
}

}  // namespace capi
}  // namespace sf

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
    apply_size_defaults(ctx);
    if (n == 0) return SF_OK;
    if (vel_xyz && is_pinned(pos_xyz) && is_pinned(vel_xyz)) {
        SF_TRY(upload_overlapped(ctx, pos_xyz, vel_xyz));
        // The caller's arrays are read once both copies end; the sort goes on
        // on the stream, and the next call queues behind it.
        SF_CUDA(cudaEventSynchronize(ctx->ev_in));
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
    if (pos_xyz && vel_xyz && is_pinned(pos_xyz) && is_pinned(vel_xyz)) {
        // page-locked outputs: positions stored and copied on the stream, the
        // velocities on the second stream meanwhile; one wait for both
        SF_TRY(need_aux(ctx));
        SF_CUDA(cudaEventRecord(ctx->ev_out, ctx->stream));
        SF_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->ev_out, 0));
        sf::launch_store_aos(ctx->d.pos, ctx->d.vel, n, io, nullptr, ctx->stream);
        sf::launch_store_aos(ctx->d.pos, ctx->d.vel, n, nullptr, io + 3 * (size_t)n, ctx->aux);
        SF_TRY(check_launch("store state"));
        SF_CUDA(cudaMemcpyAsync(pos_xyz, io, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SF_CUDA(cudaMemcpyAsync(vel_xyz, io + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost, ctx->aux));
        SF_CUDA(cudaEventRecord(ctx->ev_out, ctx->aux));
        SF_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_out, 0));  // later work waits for the velocity reads
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
    sf::launch_store_aos(ctx->d.pos, ctx->d.vel, n, pos_xyz ? io : nullptr, vel_xyz ? io + 3 * (size_t)n : nullptr,
                         ctx->stream);
    SF_TRY(check_launch("store state"));
    if ((!pos_xyz || is_pinned(pos_xyz)) && (!vel_xyz || is_pinned(vel_xyz))) {
        // page-locked outputs: both copies queued, one wait
        if (pos_xyz) SF_CUDA(cudaMemcpyAsync(pos_xyz, io, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (vel_xyz)
            SF_CUDA(cudaMemcpyAsync(vel_xyz, io + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SF_CUDA(cudaStreamSynchronize(ctx->stream));
        return SF_OK;
    }
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
    apply_size_defaults(ctx);
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
    dr.frame = ctx->frame;  // the density pass chooses dt, the force pass reads it
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

}  // extern "C"
