// sf_capi_batch.cpp — the C ABI's batches of independent scenes.
#include "sf_capi_impl.h"

// ---------------------------------------------------------------- batches
// A batch is one engine (stream, graph, particle and cell buffers) over the
// concatenation of all scenes' particles, with a per-scene constant table and
// the scenes' particle offsets in device memory.  Scene s owns cell keys
// [cell_base_s, cell_base_s + ncells_s), so one counting sort keeps every
// scene's particles contiguous (sorted positions [off_s, off_{s+1})).

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
        // scene cell ranges start at multiples of four cells (the persistent
        // step scans them four cells at a time); the cells between are empty
        base += (consts[s].ncells + 3) / 4 * 4;
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
    b->eng.d.scene_order = b->d_order;
    b->eng.d.scene_queue = b->d_queue;
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
    if (e == cudaSuccess) e = dev_malloc(&b->d_order, nscenes * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_malloc(&b->d_queue, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_order, 0, nscenes * sizeof(uint32_t), b->eng.stream);
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
    if (b->d_order) cudaFree(b->d_order);
    if (b->d_queue) cudaFree(b->d_queue);
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
    SF_RANGE("sf_batch_set_state");
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
    // the persistent step's queue order: largest scenes first (ties by index)
    std::vector<uint32_t> order(ns);
    for (size_t s = 0; s < ns; ++s) order[s] = (uint32_t)s;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return counts[x] > counts[y]; });
    SF_CUDA(cudaMemcpy(b->d_order, order.data(), ns * sizeof(uint32_t), cudaMemcpyHostToDevice));
    b->counts.assign(counts, counts + ns);
    return sf_set_state(&b->eng, pos_xyz, vel_xyz, off[ns]);
}

SF_API sf_status sf_batch_get_state(sf_batch* b, float* pos_xyz, float* vel_xyz, uint32_t n) {
    SF_RANGE("sf_batch_get_state");
    SF_TRY(need_batch(b));
    return sf_get_state(&b->eng, pos_xyz, vel_xyz, n);
}

SF_API sf_status sf_batch_num_particles(const sf_batch* b, uint32_t* n_out) {
    SF_TRY(need_batch(b));
    return sf_get_num_particles(&b->eng, n_out);
}

SF_API sf_status sf_batch_step(sf_batch* b, uint32_t nsteps) {
    SF_RANGE("sf_batch_step");
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
    SF_RANGE("sf_batch_step");
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
// of every candidate configuration — grid granularity K, and either the five
// launches' kernel variants or the persistent step's cluster and block size
// (its partition of the scenes over the GPU) — each from the same snapshot of
// the current state, keeps the fastest, and restores the snapshot.  The chosen K changes the summation
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
    for (int K : {1, 2}) {
        // five launches per step over all scenes
        for (int mode : {SF_LIST_TILE_STAGED, SF_LIST_TILE, SF_LIST_TILE16})
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
        // one persistent launch per step, scenes partitioned over clusters
        for (int cl : {4, 8})
            for (int bb : {256, 1024}) {
                sf_tuning t{};
                t.list_mode = SF_LIST_TILE;
                t.density_block = 256;
                t.force_block = 128;
                t.prefetch = 2;
                t.batch_cluster = cl;
                t.batch_block = bb;
                cands.push_back({K, t});
            }
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
