// sf_internal.h — shared declarations of the GB300 SPH step (not installed).
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/sf_capi.h"

namespace sf {

// Per-step constants, derived once on the host from sf_params (in double,
// rounded to float) and passed to every kernel by value.
struct SimConst {
    float h, h2;          // kernel radius and its square
    float cd;             // m * 315 / (64 pi h^9): density = cd * sum (h^2 - r^2)^3
    float cp;             // m * 45 / (pi h^6) / 2: pressure-force coefficient
    float cv;             // mu * m * 45 / (pi h^6): viscosity-force coefficient
    float k, rho0, inv_rho0;
    float dt, e;          // sub-step, boundary restitution
    float g[3];           // gravity
    float lo[3], hi[3];   // particle-centre clamp box: box_min + r, box_max - r
    float bmin[3];        // grid origin
    float inv_cell[3];    // cells per unit length, per axis
    int n[3];             // cells per axis
    int eos, attractive;
    int reach;            // cells searched on each side: K = cells per kernel radius
    uint32_t ncells;
    float mass;
    // Conservative pruning of the candidate walk (skips only cells that hold
    // no particle within h): cell widths, a slack covering the rounding of
    // cell assignment, and the squared-distance threshold h^2 (1 + 1e-4).
    float cell_w[3];
    float prune_margin;
    float prune_h2;
    uint32_t cell_base;   // first key of this scene's cells (0 outside a batch)
    // adaptive sub-step: dt = min(dt_max, cfl_v h / max|v|, cfl_a sqrt(h / max|a|))
    int adaptive;
    float cfl_v, cfl_a;
};

// Device-side frame and sub-step state (one per context).
struct FrameState {
    float dt;            // the current sub-step
    uint32_t v2max_bits; // max |v|^2 of the last sub-step (float bits, >= 0)
    uint32_t a2max_bits; // max |a|^2 of the last sub-step
    float frame_acc;     // simulated time of the current frame (float, like frameTime)
    uint32_t iter;       // sub-steps of the current frame
    uint32_t substeps;   // sub-steps since the last reset
    double sim_time;     // simulated time since the last reset: the finished frames' float times, summed
};

// Fill `c` from `p`; returns SF_OK or an error code (with message in `why`).
int derive_constants(const sf_params& p, SimConst* c, const char** why);

// Scene generator (sf_scenes.cpp): AoS float3 positions of `scene`.
int scene_points(const sf_params& p, int scene, uint64_t seed, std::vector<float>& out, const char** why);
// Batched cube workload (sf_scenes.cpp): per-scene parameters, counts and the
// concatenated AoS float3 positions.
int batch_cubes(uint64_t seed, uint32_t nscenes, const sf_params& base, std::vector<sf_params>& params,
                std::vector<uint32_t>& counts, std::vector<float>& pos, const char** why);

// Kernel choices of a context (all give bit-identical results).
struct Tuning {
    int list_mode = SF_LIST_TILE;  // SF_LIST_*: how the density pass records neighbours
    int density_block = 256;       // 128 or 256 threads
    int force_block = 128;         // 128 or 256 threads
    int prefetch = 2;              // neighbours gathered per batch in the force pass: 2 or 4
    int l2_window = 0;             // 1: persisting L2 window over the gather records
    int batch_cluster = 0;         // batches: 0 five launches per step; 2, 4, 8 one persistent launch of clusters
    int batch_block = 0;           // threads per block of the persistent step: 256, 512, 1024 (0: 256)
};

// Device buffers of one solver context (all owned by the context).
struct DeviceState {
    Tuning tune;
    uint32_t n = 0, cap = 0;
    float4* pos = nullptr;   // sorted positions, w = original index (bit pattern)
    float4* vel = nullptr;   // sorted velocities, w = 0
    float4* pos2 = nullptr;  // integrated positions before the re-sort
    float4* vel2 = nullptr;
    float2* pr = nullptr;    // (pressure, 1/density) of the last density pass
    float* rho = nullptr;    // density of the last density pass
    uint2* key_slot = nullptr;  // (cell key, arrival slot) of pos2/vel2 order
    uint32_t* tmp = nullptr;    // cell-bucketed unsorted indices
    float* io = nullptr;        // AoS staging, 6 floats per particle
    float4* accel = nullptr;    // optional acceleration output (inspection)
    uint32_t* nbr = nullptr;       // neighbour lists, tile-major (kNbCap * kNbTile per tile)
    uint32_t* nbr_count = nullptr; // neighbours of each particle (may exceed kNbCap)
    uint8_t* nbr_wide = nullptr;   // SF_LIST_TILE16: per warp tile (kNbWarpTile particles), 1 where it holds 32-bit entries
    float4* pv = nullptr;          // 2 per particle (32 bytes): (x, y, z, p), (vx, vy, vz, 1/rho)
    float4* sums = nullptr;        // optional: per particle (AP, 0), (AV, 0) of the force pass (adjoint recording)
    FrameState* frame = nullptr;   // adaptive sub-steps read dt here and raise the maxima
    // grid
    uint32_t ncells = 0, ncells_pad = 0;
    uint32_t* counts = nullptr;      // ncells_pad, zero between steps
    // per scan tile (kScanTile cells): particles counted in it, zero between steps
    uint32_t* cell_start = nullptr;  // ncells + 1
    uint32_t* tile_sums = nullptr;
    uint32_t ntiles = 0;
    // batches of independent scenes (null for a single scene): per-scene
    // constants and the first particle index of each scene (nscenes + 1)
    const SimConst* table = nullptr;
    const uint32_t* scene_off = nullptr;
    uint32_t nscenes = 0;
    // persistent batched step: scenes in decreasing particle count, and the
    // queue counter its clusters take scenes from
    const uint32_t* scene_order = nullptr;
    uint32_t* scene_queue = nullptr;
};

// Neighbour lists: up to kNbCap neighbours per particle, in tiles of kNbTile
// particles (see nbr_index in sf_device.cuh).
constexpr int kNbTile = 128;
constexpr int kNbCap = 64;
constexpr int kNbWarpTile = 32;  // tiles of SF_LIST_TILE16 lists: one warp's particles
// list emission modes of the density pass
constexpr int kEmitNone = 0, kEmitStaged = 1, kEmitTile = 2, kEmitTile16 = 3;
// SF_LIST_TILE16: entries hold the neighbour index's low 16 bits, exact when
// |j - i| <= kNear16 (j = i + (int16_t)(entry - i)).
constexpr uint32_t kNear16 = 32767;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kScanBlocksPerSM = 2;  // resident scan blocks per SM (the scan grid's size)

// Persisting L2 (sf_grid.cu).  reserve_persisting_l2(want) grows this
// process's persisting-L2 carve-out on the current device to `want` bytes
// (at most the device's maximum; a limit of the process's context, gone with
// it) and returns it (0 where the device has none); call it outside stream
// capture.  persisting_window() fills an access-policy window over
// [base, base + bytes) (cut to the device's largest window, hit ratio scaled
// to the carve-out) and returns false while no carve-out is reserved.
size_t reserve_persisting_l2(size_t want);
bool persisting_window(const void* base, size_t bytes, cudaAccessPolicyWindow* w);

// ---- kernel launchers (sf_grid.cu, sf_density.cu, sf_force.cu); all enqueue on `s`
void launch_load_aos(const float* pos3, const float* vel3, uint32_t n, float4* pos, float4* vel, cudaStream_t s);
void launch_load_pos(const float* pos3, uint32_t n, float4* pos, cudaStream_t s);
void launch_load_vel(const float* vel3, uint32_t n, float4* vel, cudaStream_t s);
void launch_load_sorted(const float* pos3, const float* vel3, const uint32_t* ids, uint32_t n, float4* pos,
                        float4* vel, cudaStream_t s);
void launch_store_sorted(const float4* pos, const float4* vel, uint32_t n, float* pos3, float* vel3, uint32_t* ids,
                         cudaStream_t s);
void launch_store_aos(const float4* pos, const float4* vel, uint32_t n, float* pos3, float* vel3, cudaStream_t s);
// Caller-order AoS output with coalesced stores (for host memory that the
// kernel writes directly); `slot` is n entries of scratch.
void launch_store_caller_order(const float4* pos, const float4* vel, uint32_t n, uint32_t* slot, float* pos3,
                               float* vel3, cudaStream_t s);
// Cell keys and histogram of an uploaded state, and its scan-tile totals.
void launch_hash_count(const DeviceState& d, const float4* pos, uint32_t n, const SimConst& c, uint32_t* counts,
                       uint2* key_slot, cudaStream_t s);
void launch_scan_cells(DeviceState& d, uint32_t n, cudaStream_t s);
void launch_scatter(const uint2* key_slot, const uint32_t* cell_start, uint32_t n, uint32_t* tmp, uint32_t* counts,
                    cudaStream_t s);
// also zeroes tile_sums (ntiles entries) for the next histogram
void launch_rank_gather(const uint2* key_slot, const uint32_t* cell_start, const uint32_t* tmp, const float4* pos_in,
                        const float4* vel_in, uint32_t n, float4* pos_out, float4* vel_out, uint32_t* tile_sums,
                        uint32_t ntiles, cudaStream_t s);
void launch_density(const DeviceState& d, const SimConst& c, cudaStream_t s);
// forces + symplectic Euler + box + next-step cell hash into pos2/vel2
void launch_force_integrate(DeviceState& d, const SimConst& c, cudaStream_t s);
// forces only: acceleration into d.accel (inspection)
void launch_force_only(DeviceState& d, const SimConst& c, cudaStream_t s);

// Index-check failures counted by the checked build's kernels, per
// translation unit (always 0 in the release build); `reset` clears them.
uint64_t index_check_failures_density(bool reset);
uint64_t index_check_failures_force(bool reset);
uint64_t index_check_failures_adjoint(bool reset);
uint64_t index_check_failures_grid(bool reset);
void launch_keys(const DeviceState& d, const float4* pos, uint32_t n, const SimConst& c, uint32_t* keys,
                 cudaStream_t s);
// State invariants for sf_check_state: `seen` is n words of scratch, `report`
// kReportWords words (see k_check_state).
constexpr uint32_t kReportWords = 8;
void launch_check_state(const DeviceState& d, const SimConst& c, const uint32_t* nbr_count, uint32_t* seen,
                        uint32_t* report, cudaStream_t s);
void launch_neighbour_stats(const DeviceState& d, const SimConst& c, uint32_t* count, uint32_t* hash,
                            cudaStream_t s);

// The sort tail shared by makeReady and every step: counts -> cell_start,
// bucket (clearing the counters), stable rank, gather pos2/vel2 -> pos/vel.
void enqueue_sort_tail(DeviceState& d, cudaStream_t s, cudaEvent_t before_gather = nullptr);
// One full sub-step on the sorted state.
void enqueue_step(DeviceState& d, const SimConst& c, cudaStream_t s);

// The sub-step as separately launchable stages (for per-stage timing).
constexpr uint32_t kNumStages = 5;
extern const char* const kStageNames[kNumStages];
void enqueue_stage(uint32_t stage, DeviceState& d, const SimConst& c, cudaStream_t s);

// ---- sub-step control (sf_frame.cu) ------------------------------------
// dt of the next sub-step from the maxima (adaptive) or the fixed step; clears the maxima.
// Maxima of the uploaded state: |v|^2 over the particles, |a|^2 = 0.
void launch_init_maxima(const float4* vel, uint32_t n, FrameState* fs, cudaStream_t s);
void launch_frame_begin(FrameState* fs, cudaStream_t s);
// frame_acc += dt, count the sub-step, continue the while node while
// (double)frame_acc < frame_time and iter < max_substeps.
void launch_frame_check(FrameState* fs, double frame_time, uint32_t max_substeps, cudaGraphConditionalHandle h,
                        cudaStream_t s);

// ---- adjoint (sf_adjoint.cu) -------------------------------------------
// One recorded forward step, in that step's sorted order.
struct AdjointStep {
    uint32_t n = 0;
    const float4* pos = nullptr;
    const float4* vel = nullptr;
    const float2* pr = nullptr;
    const float* rho = nullptr;
    const uint32_t* nbr = nullptr;
    const uint32_t* cnt = nullptr;
    const uint32_t* cs = nullptr;
    const float4* sums = nullptr;
    const float4* pv = nullptr;  // the step's 32-byte gather records (x, y, z, p), (vx, vy, vz, 1/rho)
};
// Adjoint working buffers (N particles).  Xb/Vb are indexed by particle id.
struct AdjointWork {
    float4* Xb = nullptr;
    float4* Vb = nullptr;
    float4* ab = nullptr;  // 2 per particle (32 bytes): apb = (cp tb, inv_bar), avb = (cv tb, cv_bar)
    float4* xdir = nullptr;
    float4* vdir = nullptr;
    float4* xf = nullptr;
    float4* vf = nullptr;
    float4* xrb = nullptr;  // per particle (x, y, z, rho_bar): P4's gather record
    double* scalars = nullptr;   // [sum cv_bar, sum k_bar]
};
// The adjoint step's passes: P1 integration and box (adj_integrate), P2 force
// pair terms and density adjoint (adj_forces), P4 poly6 terms (adj_density).
constexpr uint32_t kAdjointPasses = 3;
extern const char* const kAdjointPassNames[kAdjointPasses];
void launch_adjoint_pass(uint32_t pass, const AdjointStep& st, const SimConst& c, AdjointWork& w, double2* partial,
                         cudaStream_t s);
// One step's adjoint (its passes in order); its scalar block partials go to
// `partial` (adjoint_partial_count(N) entries).
void launch_adjoint_step(const AdjointStep& st, const SimConst& c, AdjointWork& w, double2* partial,
                         cudaStream_t s);
uint32_t adjoint_partial_count(uint32_t n);
// scalars += the partials of `nsteps` consecutive steps (last step first).
void launch_adjoint_accumulate(const double2* partial, uint32_t nsteps, uint32_t n, double* scalars, cudaStream_t s);
// CIC histogram loss of the sorted state; dL/dx written to Xb by particle id.
void launch_histogram_loss(const float4* pos, uint32_t n, const SimConst& c, const float box_ext[3], uint32_t res,
                           const float* target, unsigned long long* hist, float* e2, double* partial, float4* Xb,
                           cudaStream_t s);
uint32_t histogram_partial_count(uint32_t res);

// ---- persistent batched step (sf_batch.cu) --------------------------------
struct BatchStep {
    float4* pos;
    float4* vel;
    float4* pos2;
    float4* vel2;
    float2* pr;
    float* rho;
    uint2* key_slot;
    uint32_t* tmp;
    uint32_t* nbr;
    uint32_t* nbr_count;
    float4* pv;
    uint32_t* counts;
    uint32_t* cell_start;
    const SimConst* table;
    const uint32_t* scene_off;
    const uint32_t* order;
    uint32_t* queue;
    uint32_t nscenes;
    uint32_t n;
};
// Clusters of `cluster` blocks (2, 4 or 8) of `block` threads (256, 512 or
// 1024) of the persistent step that the current device keeps resident at
// once (0 if it cannot run them).
int batch_persistent_clusters(int cluster, int block, int reach);
// One sub-step of every scene: a queue reset and one launch of `nclusters`
// clusters.  Scene cell ranges must start at multiples of four cells.
void launch_batch_persistent(const BatchStep& a, int cluster, int block, int nclusters, int reach, cudaStream_t s);

// Density of caller-owned device positions using the library's fixed static
// scratch (sf_noalloc.cu); no device allocation.
int noalloc_density(const sf_params& p, const SimConst& c, const float* d_pos_xyz, uint32_t n, float* d_rho,
                    float* d_pressure, cudaStream_t stream, const char** why);

}  // namespace sf
