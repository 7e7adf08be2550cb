// sf_capi_adjoint.cpp — the C ABI's differentiation: checkpointed forward,
// histogram loss and the adjoint sweep.
#include "sf_capi_impl.h"

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
    SF_ALLOC_TRAJ(w.ab, 2 * n * sizeof(float4));
    SF_ALLOC_TRAJ(w.xdir, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.vdir, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.xf, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.vf, n * sizeof(float4));
    SF_ALLOC_TRAJ(w.xrb, n * sizeof(float4));
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
        SF_ALLOC_TRAJ(r.pv, 2 * n * sizeof(float4));
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
        ds.pv = r.pv;
        // the reverse passes read 32-bit lists
        if (ds.tune.list_mode != SF_LIST_TILE_STAGED) ds.tune.list_mode = SF_LIST_TILE;
        ds.tune.l2_window = 0;
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
        as.pv = r.pv;
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
    t->rec_len = std::min(t->nsteps, t->ckpt);  // the records now hold the first segment
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
