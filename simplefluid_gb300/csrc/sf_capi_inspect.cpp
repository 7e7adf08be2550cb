// sf_capi_inspect.cpp — the C ABI's inspection, state checks, fault hook,
// timing, tuning, rendering and state-file entry points.
#include "sf_capi_impl.h"

extern "C" {

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

SF_API sf_status sf_index_checks(int32_t reset, uint64_t* failures, int32_t* compiled_in) {
#ifndef SF_DEVICE_CHECKS
#define SF_DEVICE_CHECKS 0
#endif
    if (compiled_in) *compiled_in = SF_DEVICE_CHECKS;
    const bool r = reset != 0;
    const uint64_t total = sf::index_check_failures_density(r) + sf::index_check_failures_force(r) +
                           sf::index_check_failures_adjoint(r) + sf::index_check_failures_grid(r);
    if (failures) *failures = total;
    if (SF_DEVICE_CHECKS) SF_TRY(check_launch("sf_index_checks"));
    return SF_OK;
}

SF_API sf_status sf_test_fail_allocation(int64_t after) {
    set_fail_allocation(after);
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
    t->l2_window = ctx->d.tune.l2_window;
    t->batch_cluster = ctx->d.tune.batch_cluster;
    t->batch_block = ctx->d.tune.batch_block;
    return SF_OK;
}

SF_API sf_status sf_set_tuning(sf_ctx* ctx, const sf_tuning* t) {
    SF_TRY(need_ctx(ctx));
    if (!t) return fail(SF_ERR_INVALID_ARGUMENT, "null tuning");
    if (t->list_mode < SF_LIST_NONE || t->list_mode > SF_LIST_TILE16)
        return fail(SF_ERR_INVALID_ARGUMENT, "unknown list_mode");
    if (t->l2_window != 0 && t->l2_window != 1) return fail(SF_ERR_INVALID_ARGUMENT, "l2_window must be 0 or 1");
    if (t->batch_cluster != 0 && t->batch_cluster != 2 && t->batch_cluster != 4 && t->batch_cluster != 8)
        return fail(SF_ERR_INVALID_ARGUMENT, "batch_cluster must be 0, 2, 4 or 8");
    if (t->batch_cluster && !ctx->d.table)
        return fail(SF_ERR_INVALID_ARGUMENT, "batch_cluster applies to batches only");
    if (t->batch_cluster && t->list_mode != SF_LIST_TILE)
        return fail(SF_ERR_INVALID_ARGUMENT, "the persistent batched step records SF_LIST_TILE lists");
    if (t->batch_block != 0 && t->batch_block != 256 && t->batch_block != 512 && t->batch_block != 1024)
        return fail(SF_ERR_INVALID_ARGUMENT, "batch_block must be 256, 512 or 1024");
    if ((t->density_block != 128 && t->density_block != 256) || (t->force_block != 128 && t->force_block != 256))
        return fail(SF_ERR_INVALID_ARGUMENT, "block sizes must be 128 or 256");
    if (t->prefetch != 2 && t->prefetch != 4) return fail(SF_ERR_INVALID_ARGUMENT, "prefetch must be 2 or 4");
    if (t->reserved[0]) return fail(SF_ERR_INVALID_ARGUMENT, "reserved fields must be zero");
    SF_TRY(set_device(ctx));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->d.tune.list_mode = t->list_mode;
    ctx->d.tune.density_block = t->density_block;
    ctx->d.tune.force_block = t->force_block;
    ctx->d.tune.prefetch = t->prefetch;
    ctx->d.tune.l2_window = t->l2_window;
    ctx->d.tune.batch_cluster = t->batch_cluster;
    ctx->d.tune.batch_block = t->batch_block;
    ctx->tune_explicit = true;
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

SF_API uint32_t sf_adjoint_pass_count(void) { return sf::kAdjointPasses; }

SF_API const char* sf_adjoint_pass_name(uint32_t pass) {
    return pass < sf::kAdjointPasses ? sf::kAdjointPassNames[pass] : "";
}

SF_API sf_status sf_adjoint_profile(sf_ctx* ctx, float* pass_ms, uint32_t npasses, uint32_t* steps_out) {
    SF_TRY(need_sorted(ctx));
    if (!pass_ms || npasses != sf::kAdjointPasses)
        return fail(SF_ERR_INVALID_ARGUMENT, "pass_ms needs sf_adjoint_pass_count()");
    sf::Trajectory* t = ctx->traj;
    if (!t || !t->rec_len || t->rec.size() < t->rec_len || t->n != ctx->d.cap)
        return fail(SF_ERR_NOT_READY, "no recorded segment: call sf_adjoint first");
    SF_TRY(set_device(ctx));
    for (uint32_t p = 0; p < npasses; ++p) pass_ms[p] = 0.f;
    const uint32_t len = t->rec_len, n = ctx->d.n;
    const size_t per = (size_t)sf::kAdjointPasses + 1;
    EventSet ev;
    SF_CUDA(ev.create(per * len));
    const uint32_t nb = sf::adjoint_partial_count(n);
    for (uint32_t k = 0; k < len; ++k) {
        const uint32_t s = len - 1 - k;  // the reverse sweep's order
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
        as.pv = r.pv;
        SF_CUDA(cudaEventRecord(ev.ev[per * k], ctx->stream));
        for (uint32_t p = 0; p < sf::kAdjointPasses; ++p) {
            sf::launch_adjoint_pass(p, as, ctx->c, t->w, t->seg_partial + (size_t)s * nb, ctx->stream);
            SF_CUDA(cudaEventRecord(ev.ev[per * k + p + 1], ctx->stream));
        }
    }
    SF_TRY(check_launch("profiled adjoint"));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    for (uint32_t k = 0; k < len; ++k)
        for (uint32_t p = 0; p < sf::kAdjointPasses; ++p) {
            float ms = 0.f;
            SF_CUDA(cudaEventElapsedTime(&ms, ev.ev[per * k + p], ev.ev[per * k + p + 1]));
            pass_ms[p] += ms;
        }
    if (steps_out) *steps_out = len;
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
    apply_size_defaults(ctx);
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

}  // extern "C"
