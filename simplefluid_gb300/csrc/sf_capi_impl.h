// sf_capi_impl.h — private to the C ABI implementation (sf_capi*.cpp):
// the context and batch objects and the helpers the API files share.
#pragma once

#include <algorithm>
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
    float4* pv = nullptr;  // 2n float4: the step's gather records
};
struct Trajectory {
    uint32_t nsteps = 0, ckpt = 0, n = 0, ncells_pad = 0;
    bool valid = false;
    std::vector<float4*> ck;  // per checkpoint: pos then vel (2n float4)
    std::vector<StepRec> rec; // ckpt steps of one segment
    uint32_t rec_len = 0;     // steps of the segment the records hold (after sf_adjoint: the first)
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
    cudaEvent_t ev_pos = nullptr, ev_vel = nullptr, ev_in = nullptr, ev_out = nullptr;
    // the GPU reads and writes pageable host memory through the host's page
    // tables (Grace: NVLink-C2C with address translation): -1 unknown, 0, 1
    int host_direct = -1;
    uint32_t* d_report = nullptr;  // sf_check_state counters
    bool tune_explicit = false;    // sf_set_tuning was called: keep its choices
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

// A batch is one engine (stream, graph, particle and cell buffers) over the
// concatenation of all scenes' particles, with a per-scene constant table and
// the scenes' particle offsets in device memory.
struct sf_batch {
    sf_ctx eng;
    std::vector<sf_params> params;
    std::vector<sf::SimConst> consts;
    std::vector<uint32_t> counts;  // particles per scene
    sf::SimConst* d_table = nullptr;
    uint32_t* d_off = nullptr;
    uint32_t* d_order = nullptr;  // scenes in decreasing particle count (the persistent step's queue order)
    uint32_t* d_queue = nullptr;  // the persistent step's queue counter
};

namespace sf {
namespace capi {

// NVTX range over an API call (visible in Nsight timelines; a no-op without a
// tool attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define SF_RANGE(name) NvtxRange sf_nvtx_range_(name)

cudaError_t dev_malloc_raw(void** p, size_t bytes);
// Arm sf_test_fail_allocation's countdown (negative: disarmed).
void set_fail_allocation(int64_t after);

template <typename T>
cudaError_t dev_malloc(T** p, size_t bytes) {
    return dev_malloc_raw(reinterpret_cast<void**>(p), bytes);
}

// errors: set the calling thread's message (sf_last_error) and return `st`
sf_status fail(sf_status st, const std::string& msg);
sf_status cuda_fail(cudaError_t e, const char* what);
sf_status check_launch(const char* what);
sf_status validate(const sf_params& p);
sf_status need_ctx(const sf_ctx* ctx);
sf_status need_sorted(const sf_ctx* ctx);
sf_status set_device(const sf_ctx* ctx);

// host memory: page-locked staging, pointer kinds, copies through staging
sf_status ensure_stage(sf_ctx* ctx, size_t bytes);
bool host_direct(sf_ctx* ctx, const void* p);
bool is_pinned(const void* p);
sf_status copy_out(sf_ctx* ctx, void* dst, const void* src, size_t bytes);
sf_status copy_in(sf_ctx* ctx, void* dst, const void* src, size_t bytes);

// device buffers; a failed allocation releases what the call had allocated
sf_status alloc_grid(sf_ctx* ctx);
sf_status alloc_particles(sf_ctx* ctx, uint32_t n);
void free_particles(sf::DeviceState& d);
void free_grid(sf::DeviceState& d);
void free_rec(sf::StepRec& r);
void drop_segment_graphs(sf::Trajectory* t);
void free_trajectory(sf_ctx* ctx);
void free_render(sf_ctx* ctx);
void release_ctx(sf_ctx* ctx);

// uploads and the captured step
sf_status sort_uploaded(sf_ctx* ctx, const float* pos3, const float* vel3);
sf_status upload_overlapped(sf_ctx* ctx, const float* pos_xyz, const float* vel_xyz);
void enqueue_full_step(sf_ctx* ctx);
sf_status capture_step(sf_ctx* ctx);
void drop_graph(sf_ctx* ctx);
// Kernel choices by particle count, unless the caller set them explicitly.
void apply_size_defaults(sf_ctx* ctx);

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

}  // namespace capi
}  // namespace sf

using namespace sf::capi;  // NOLINT: the API files use the helpers unqualified
