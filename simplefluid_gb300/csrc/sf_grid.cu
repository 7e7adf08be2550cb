// sf_grid.cu — uniform-grid neighbour search of the SPH sub-step (sm_103a):
// cell hashing, the counting sort with its cell table, particle reorder, state
// upload/download, and the stage list of one sub-step.
//
// The sort is a one-pass counting (radix-`ncells`) sort: the histogram of cell
// keys, taken by the force pass's atomics (k_hash_count for an uploaded
// state), is exclusive-scanned into the cell table, so cell start/end come out
// of the same scan that places the particles.  Stability (equal keys keep their
// previous order) is restored by ranking each particle among its cell's
// members, which makes the order deterministic and identical to a stable sort.
#include <mutex>

#include "sf_device.cuh"

namespace sf {
namespace {

// ---------------------------------------------------------------- state IO
__global__ void k_load_aos(const float* __restrict__ pos3, const float* __restrict__ vel3, uint32_t n,
                           float4* __restrict__ pos, float4* __restrict__ vel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(pos3[3 * (size_t)i], pos3[3 * (size_t)i + 1], pos3[3 * (size_t)i + 2], __uint_as_float(i));
    if (vel3)
        vel[i] = make_float4(vel3[3 * (size_t)i], vel3[3 * (size_t)i + 1], vel3[3 * (size_t)i + 2], 0.f);
    else
        vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// The two halves of k_load_aos, for uploads whose velocities arrive later.
__global__ void k_load_pos(const float* __restrict__ pos3, uint32_t n, float4* __restrict__ pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(pos3[3 * (size_t)i], pos3[3 * (size_t)i + 1], pos3[3 * (size_t)i + 2], __uint_as_float(i));
}

__global__ void k_load_vel(const float* __restrict__ vel3, uint32_t n, float4* __restrict__ vel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vel[i] = make_float4(vel3[3 * (size_t)i], vel3[3 * (size_t)i + 1], vel3[3 * (size_t)i + 2], 0.f);
}

// Sorted state with explicit particle indices (state files).
__global__ void k_load_sorted(const float* __restrict__ pos3, const float* __restrict__ vel3,
                              const uint32_t* __restrict__ ids, uint32_t n, float4* __restrict__ pos,
                              float4* __restrict__ vel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(pos3[3 * (size_t)i], pos3[3 * (size_t)i + 1], pos3[3 * (size_t)i + 2], __uint_as_float(ids[i]));
    vel[i] = make_float4(vel3[3 * (size_t)i], vel3[3 * (size_t)i + 1], vel3[3 * (size_t)i + 2], 0.f);
}

// Sorted state out (state files): AoS pos/vel in solver order plus indices.
__global__ void k_store_sorted(const float4* __restrict__ pos, const float4* __restrict__ vel, uint32_t n,
                               float* __restrict__ pos3, float* __restrict__ vel3, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i], v = vel[i];
    pos3[3 * (size_t)i] = p.x;
    pos3[3 * (size_t)i + 1] = p.y;
    pos3[3 * (size_t)i + 2] = p.z;
    vel3[3 * (size_t)i] = v.x;
    vel3[3 * (size_t)i + 1] = v.y;
    vel3[3 * (size_t)i + 2] = v.z;
    ids[i] = __float_as_uint(p.w);
}

__global__ void k_store_aos(const float4* __restrict__ pos, const float4* __restrict__ vel, uint32_t n,
                            float* __restrict__ pos3, float* __restrict__ vel3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const uint32_t id = __float_as_uint(p.w);
    if (id >= n) return;  // never for a consistent state
    if (pos3) {
        pos3[3 * (size_t)id] = p.x;
        pos3[3 * (size_t)id + 1] = p.y;
        pos3[3 * (size_t)id + 2] = p.z;
    }
    if (vel3) {
        const float4 v = vel[i];
        vel3[3 * (size_t)id] = v.x;
        vel3[3 * (size_t)id + 1] = v.y;
        vel3[3 * (size_t)id + 2] = v.z;
    }
}

// Sorted slot of every caller index.
__global__ void k_slot_of_caller(const float4* __restrict__ pos, uint32_t n, uint32_t* __restrict__ slot) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(pos[i].w);
    if (id < n) slot[id] = i;
}

// Caller-order AoS state gathered through the slot map: consecutive threads
// write consecutive particles, so the stores stay coalesced when the arrays
// are host memory that the kernel writes over the CPU-GPU link.
__global__ void k_store_caller_order(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                     const uint32_t* __restrict__ slot, uint32_t n, float* __restrict__ pos3,
                                     float* __restrict__ vel3) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t i = slot[t];
    if (i >= n) return;  // never for a consistent state
    if (pos3) {
        const float4 p = pos[i];
        pos3[3 * (size_t)t] = p.x;
        pos3[3 * (size_t)t + 1] = p.y;
        pos3[3 * (size_t)t + 2] = p.z;
    }
    if (vel3) {
        const float4 v = vel[i];
        vel3[3 * (size_t)t] = v.x;
        vel3[3 * (size_t)t + 1] = v.y;
        vel3[3 * (size_t)t + 2] = v.z;
    }
}

// ---------------------------------------------------------------- hashing
// Histogram of an uploaded (not cell-sorted) state.  Its lanes hit scattered
// scan tiles, so the tile totals come from a separate reduction instead of
// per-particle tile atomics.
template <bool kBatched>
__global__ void k_hash_count(const float4* __restrict__ pos, uint32_t n, SimConst c0, const SimConst* __restrict__ table,
                             const uint32_t* __restrict__ scene_off, uint32_t nscenes, uint32_t* __restrict__ counts,
                             uint2* __restrict__ key_slot) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, i);
    const float4 p = pos[i];
    const uint32_t key = cell_key(c, p.x, p.y, p.z);
    key_slot[i] = make_uint2(key, atomicAdd(counts + key, 1u));
}

template <bool kBatched>
__global__ void k_keys(const float4* __restrict__ pos, uint32_t n, SimConst c0, const SimConst* __restrict__ table,
                       const uint32_t* __restrict__ scene_off, uint32_t nscenes, uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, i);
    const float4 p = pos[i];
    keys[i] = cell_key(c, p.x, p.y, p.z);
}

// ---------------------------------------------------------------- scan
__device__ __forceinline__ uint32_t warp_inclusive(uint32_t x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Exclusive scan over a 1024-thread block; *total receives the block sum.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = warp_sums[lane];
        const uint32_t wi = warp_inclusive(w);
        warp_sums[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    __syncthreads();
    return r;
}

// Tile totals of the cell histogram (one block per scan tile).
__global__ void __launch_bounds__(kScanThreads) k_tile_totals(const uint4* __restrict__ counts,
                                                              uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t total;
    const uint4 q = counts[(size_t)blockIdx.x * kScanThreads + threadIdx.x];
    block_exclusive(q.x + q.y + q.z + q.w, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Exclusive scan of the cell histogram into the cell table, in one kernel.
// Block b scans the contiguous scan tiles [t0, t1) (kScanTile cells each; a
// few blocks per SM): it sums the totals of the tiles before t0 once (the
// histogram atomics accumulated them in tile_sums), then carries the running
// offset from tile to tile, loading the next tile's counts while it scans the
// current one.  Two barriers per tile; the warp totals alternate between two
// shared buffers so that a tile's writes never meet the previous tile's reads.
__global__ void __launch_bounds__(kScanThreads, kScanBlocksPerSM) k_scan(const uint4* __restrict__ counts,
                                                                         const uint32_t* __restrict__ tile_sums,
                                                                         uint32_t ntiles, uint32_t n,
                                                                         uint4* __restrict__ cell_start) {
    static_assert(kScanThreads == 1024, "one warp-sum slot per warp");
    grid_dependency_wait();
    allow_dependents();
    __shared__ uint32_t s_warp[2][32], s_before[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (ntiles + gridDim.x - 1) / gridDim.x;
    const uint32_t t0 = blockIdx.x * per, t1 = min(t0 + per, ntiles);
    if (t0 >= t1) return;  // the whole block
    uint4 q = counts[(size_t)t0 * kScanThreads + threadIdx.x];
    uint32_t before = 0;
    for (uint32_t k = threadIdx.x; k < t0; k += kScanThreads) before += tile_sums[k];
    before = __reduce_add_sync(0xffffffffu, before);
    if (lane == 0) s_before[warp] = before;
    __syncthreads();
    // warp 0 carries the offset of the current tile (the same in every lane)
    uint32_t base = warp == 0 ? __reduce_add_sync(0xffffffffu, s_before[lane]) : 0u;
    for (uint32_t t = t0; t < t1; ++t) {
        uint32_t* const ws = s_warp[(t - t0) & 1];
        uint4 qn = make_uint4(0u, 0u, 0u, 0u);
        if (t + 1 < t1) qn = counts[(size_t)(t + 1) * kScanThreads + threadIdx.x];
        const uint32_t v = q.x + q.y + q.z + q.w;
        const uint32_t inc = warp_inclusive(v);
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = ws[lane];
            const uint32_t wi = warp_inclusive(w);
            ws[lane] = wi - w + base;  // cells of the earlier warps and tiles
            base += __shfl_sync(0xffffffffu, wi, 31);
        }
        __syncthreads();
        // Entries are clamped to n: a histogram that does not sum to n (never
        // the case when each step's counts start from zero) cannot send the
        // candidate walks past the particle arrays.
        const uint32_t ex = ws[warp] + inc - v;
        cell_start[(size_t)t * kScanThreads + threadIdx.x] =
            make_uint4(min(ex, n), min(ex + q.x, n), min(ex + q.x + q.y, n), min(ex + q.x + q.y + q.z, n));
        q = qn;
    }
}

// ---------------------------------------------------------------- reorder
// Buckets indices by cell and clears the occupied cells' counters for the
// next step (only those were counted, so this leaves every counter zero).
__global__ void k_scatter(const uint2* __restrict__ key_slot, const uint32_t* __restrict__ cell_start, uint32_t n,
                          uint32_t* __restrict__ tmp, uint32_t* __restrict__ counts) {
    grid_dependency_wait();
    allow_dependents();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 ks = key_slot[i];
    const uint32_t at = cell_start[ks.x] + ks.y;
    if (at < n) tmp[at] = i;  // always, unless the histogram was inconsistent
    counts[ks.x] = 0u;
}

__global__ void k_rank_gather(const uint2* __restrict__ key_slot, const uint32_t* __restrict__ cell_start,
                              const uint32_t* __restrict__ tmp, const float4* __restrict__ pos_in,
                              const float4* __restrict__ vel_in, uint32_t n, float4* __restrict__ pos_out,
                              float4* __restrict__ vel_out, uint32_t* __restrict__ tile_sums, uint32_t ntiles) {
    grid_dependency_wait();
    allow_dependents();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // the scan-tile totals are zero again for the next histogram
    for (uint32_t t = i; t < ntiles; t += gridDim.x * blockDim.x) tile_sums[t] = 0u;
    if (i >= n) return;
    const float4 p = pos_in[i], v = vel_in[i];  // in flight while the rank is found
    const uint32_t key = key_slot[i].x;
    const uint32_t b = cell_start[key], e = cell_start[key + 1];
    uint32_t rank = 0;
    for (uint32_t t = b; t < e; ++t) rank += (tmp[t] < i) ? 1u : 0u;
    const uint32_t dst = b + rank;
    if (dst < n) {  // always, unless the histogram was inconsistent
        pos_out[dst] = p;
        vel_out[dst] = v;
    }
}

// ---------------------------------------------------------------- inspection
template <int kReach, bool kBatched>
__global__ void k_neighbour_stats(const float4* __restrict__ pos, const uint32_t* __restrict__ cs, uint32_t n,
                                  SimConst c0, const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off,
                                  uint32_t nscenes, uint32_t* __restrict__ count, uint32_t* __restrict__ hash) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, i);
    const float4 xi = pos[i];
    uint32_t cnt = 0, h = 0;
    for_candidates<kReach>(c, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
        if (j == i) return;
        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < c.h2) {
            ++cnt;
            h += mix32(__float_as_uint(xj.w));
        }
    });
    count[i] = cnt;
    hash[i] = h;
}

// Invariants of a cell-sorted state, counted into r[]: 0 non-finite
// particles, 1 particles outside the clamp box, 2 sorted neighbours whose cell
// keys decrease, 3 particles outside their cell's table range, 4 caller
// indices out of range (the rest are counted in `seen`), 5 neighbour lists
// that overflowed in the last density pass, 6 max |v|^2 (float bits).
template <bool kBatched>
__global__ void __launch_bounds__(kBlock)
    k_check_state(const float4* __restrict__ pos, const float4* __restrict__ vel, const uint32_t* __restrict__ cs,
                  const uint32_t* __restrict__ nbr_count, uint32_t n, SimConst c0,
                  const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off, uint32_t nscenes,
                  uint32_t* __restrict__ seen, uint32_t* __restrict__ r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t v2 = 0u;
    if (i < n) {
        const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, i);
        const float4 p = pos[i], v = vel[i];
        const bool finite = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) &&
                            isfinite(v.z);
        if (!finite) atomicAdd(r + 0, 1u);
        if (finite && (p.x < c.lo[0] || p.x > c.hi[0] || p.y < c.lo[1] || p.y > c.hi[1] || p.z < c.lo[2] ||
                       p.z > c.hi[2]))
            atomicAdd(r + 1, 1u);
        const uint32_t key = cell_key(c, p.x, p.y, p.z);
        if (i > 0) {
            const SimConst cq = const_of<kBatched>(c0, table, scene_off, nscenes, i - 1);
            const float4 q = pos[i - 1];
            if (cell_key(cq, q.x, q.y, q.z) > key) atomicAdd(r + 2, 1u);
        }
        if (!(cs[key] <= i && i < cs[key + 1])) atomicAdd(r + 3, 1u);
        const uint32_t id = __float_as_uint(p.w);
        if (id < n)
            atomicAdd(seen + id, 1u);
        else
            atomicAdd(r + 4, 1u);
        if (nbr_count && nbr_count[i] > (uint32_t)kNbCap) atomicAdd(r + 5, 1u);
        if (finite) v2 = __float_as_uint(fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
    }
    v2 = __reduce_max_sync(0xffffffffu, v2);
    if ((threadIdx.x & 31) == 0 && v2) atomicMax(r + 6, v2);
}

// Caller indices not seen exactly once.
__global__ void k_check_ids(const uint32_t* __restrict__ seen, uint32_t n, uint32_t* __restrict__ r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && seen[i] != 1u) atomicAdd(r + 4, 1u);
}

}  // namespace

SF_INDEX_CHECK_ACCESSOR(index_check_failures_grid)

// ---------------------------------------------------------------- persisting L2
// Persisting-L2 carve-out of the current device for this process, and the
// largest access-policy window the device takes (bytes; 0 before a
// reservation or where the device has none).
struct PersistingL2 {
    std::mutex m;
    size_t carve = 0, max_window = 0;
};
static PersistingL2* persisting_l2_of_device() {
    constexpr int kDevices = 64;
    static PersistingL2 per_device[kDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    return (dev >= 0 && dev < kDevices) ? &per_device[dev] : nullptr;
}

size_t reserve_persisting_l2(size_t want) {
    PersistingL2* p = persisting_l2_of_device();
    if (!p) return 0;
    std::lock_guard<std::mutex> lock(p->m);
    int dev = 0, maxp = 0, maxw = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess || maxp <= 0 ||
        maxw <= 0) {
        cudaGetLastError();
        return p->carve;
    }
    want = std::min(want, (size_t)maxp);
    if (want > p->carve) {
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
            cudaGetLastError();
            return p->carve;
        }
        p->carve = want;
    }
    p->max_window = (size_t)maxw;
    return p->carve;
}

bool persisting_window(const void* base, size_t bytes, cudaAccessPolicyWindow* w) {
    PersistingL2* p = persisting_l2_of_device();
    if (!p) return false;
    size_t carve, max_window;
    {
        std::lock_guard<std::mutex> lock(p->m);
        carve = p->carve;
        max_window = p->max_window;
    }
    if (!carve || !base || !bytes) return false;
    bytes = std::min(bytes, max_window);
    w->base_ptr = const_cast<void*>(base);
    w->num_bytes = bytes;
    w->hitRatio = bytes <= carve ? 1.0f : (float)((double)carve / (double)bytes);
    w->hitProp = cudaAccessPropertyPersisting;
    w->missProp = cudaAccessPropertyStreaming;
    return true;
}

// ---------------------------------------------------------------- launchers
void launch_check_state(const DeviceState& d, const SimConst& c, const uint32_t* nbr_count, uint32_t* seen,
                        uint32_t* report, cudaStream_t s) {
    cudaMemsetAsync(report, 0, kReportWords * sizeof(uint32_t), s);
    if (!d.n) return;
    cudaMemsetAsync(seen, 0, (size_t)d.n * sizeof(uint32_t), s);
    if (d.table)
        k_check_state<true><<<grid_for(d.n, kBlock), kBlock, 0, s>>>(d.pos, d.vel, d.cell_start, nbr_count, d.n, c,
                                                                     d.table, d.scene_off, d.nscenes, seen, report);
    else
        k_check_state<false><<<grid_for(d.n, kBlock), kBlock, 0, s>>>(d.pos, d.vel, d.cell_start, nbr_count, d.n, c,
                                                                      nullptr, nullptr, 0, seen, report);
    k_check_ids<<<grid_for(d.n, kBlock), kBlock, 0, s>>>(seen, d.n, report);
}
void launch_load_aos(const float* pos3, const float* vel3, uint32_t n, float4* pos, float4* vel, cudaStream_t s) {
    if (n) k_load_aos<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos3, vel3, n, pos, vel);
}

void launch_load_pos(const float* pos3, uint32_t n, float4* pos, cudaStream_t s) {
    if (n) k_load_pos<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos3, n, pos);
}

void launch_load_vel(const float* vel3, uint32_t n, float4* vel, cudaStream_t s) {
    if (n) k_load_vel<<<grid_for(n, kBlock), kBlock, 0, s>>>(vel3, n, vel);
}

void launch_load_sorted(const float* pos3, const float* vel3, const uint32_t* ids, uint32_t n, float4* pos,
                        float4* vel, cudaStream_t s) {
    if (n) k_load_sorted<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos3, vel3, ids, n, pos, vel);
}

void launch_store_sorted(const float4* pos, const float4* vel, uint32_t n, float* pos3, float* vel3, uint32_t* ids,
                         cudaStream_t s) {
    if (n) k_store_sorted<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, vel, n, pos3, vel3, ids);
}

void launch_store_aos(const float4* pos, const float4* vel, uint32_t n, float* pos3, float* vel3, cudaStream_t s) {
    if (n) k_store_aos<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, vel, n, pos3, vel3);
}

void launch_store_caller_order(const float4* pos, const float4* vel, uint32_t n, uint32_t* slot, float* pos3,
                               float* vel3, cudaStream_t s) {
    if (!n) return;
    k_slot_of_caller<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, slot);
    k_store_caller_order<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, vel, slot, n, pos3, vel3);
}

void launch_hash_count(const DeviceState& d, const float4* pos, uint32_t n, const SimConst& c, uint32_t* counts,
                       uint2* key_slot, cudaStream_t s) {
    if (!n) return;
    if (d.table)
        k_hash_count<true><<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, d.table, d.scene_off, d.nscenes, counts,
                                                                  key_slot);
    else
        k_hash_count<false><<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, nullptr, nullptr, 0, counts, key_slot);
    k_tile_totals<<<d.ntiles, kScanThreads, 0, s>>>(reinterpret_cast<const uint4*>(counts), d.tile_sums);
}

void launch_keys(const DeviceState& d, const float4* pos, uint32_t n, const SimConst& c, uint32_t* keys,
                 cudaStream_t s) {
    if (!n) return;
    if (d.table)
        k_keys<true><<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, d.table, d.scene_off, d.nscenes, keys);
    else
        k_keys<false><<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, nullptr, nullptr, 0, keys);
}

void launch_scan_cells(DeviceState& d, uint32_t /*n*/, cudaStream_t s) {
    const uint32_t blocks = std::min<uint32_t>(d.ntiles, (uint32_t)(kScanBlocksPerSM * sm_count()));
    launch_chained(k_scan, blocks, kScanThreads, s, reinterpret_cast<const uint4*>(d.counts), d.tile_sums, d.ntiles,
                   d.n, reinterpret_cast<uint4*>(d.cell_start));
}

// Buckets indices by cell and clears the counters.
void launch_scatter(const uint2* key_slot, const uint32_t* cell_start, uint32_t n, uint32_t* tmp, uint32_t* counts,
                    cudaStream_t s) {
    if (n) launch_chained(k_scatter, grid_for(n, kBlock), kBlock, s, key_slot, cell_start, n, tmp, counts);
}

// Stable rank inside each cell and the gather; also zeroes the scan-tile
// totals (ntiles entries) for the next histogram.
void launch_rank_gather(const uint2* key_slot, const uint32_t* cell_start, const uint32_t* tmp, const float4* pos_in,
                        const float4* vel_in, uint32_t n, float4* pos_out, float4* vel_out, uint32_t* tile_sums,
                        uint32_t ntiles, cudaStream_t s) {
    if (n)
        launch_chained(k_rank_gather, grid_for(n, kBlock), kBlock, s, key_slot, cell_start, tmp, pos_in, vel_in, n,
                       pos_out, vel_out, tile_sums, ntiles);
}

void launch_neighbour_stats(const DeviceState& d, const SimConst& c, uint32_t* count, uint32_t* hash,
                            cudaStream_t s) {
    if (!d.n) return;
    with_reach(c.reach, [&](auto R) {
        constexpr int K = decltype(R)::value;
        if (d.table) {
            if constexpr (K <= 2)
                k_neighbour_stats<K, true><<<grid_for(d.n, kBlock), kBlock, 0, s>>>(
                    d.pos, d.cell_start, d.n, c, d.table, d.scene_off, d.nscenes, count, hash);
        } else {
            k_neighbour_stats<K, false>
                <<<grid_for(d.n, kBlock), kBlock, 0, s>>>(d.pos, d.cell_start, d.n, c, nullptr, nullptr, 0, count, hash);
        }
    });
}

void enqueue_sort_tail(DeviceState& d, cudaStream_t s, cudaEvent_t before_gather) {
    launch_scan_cells(d, d.n, s);
    launch_scatter(d.key_slot, d.cell_start, d.n, d.tmp, d.counts, s);
    if (before_gather) cudaStreamWaitEvent(s, before_gather, 0);
    launch_rank_gather(d.key_slot, d.cell_start, d.tmp, d.pos2, d.vel2, d.n, d.pos, d.vel, d.tile_sums, d.ntiles, s);
}

const char* const kStageNames[kNumStages] = {"density", "force_integrate", "scan", "scatter", "rank_gather"};

void enqueue_stage(uint32_t stage, DeviceState& d, const SimConst& c, cudaStream_t s) {
    switch (stage) {
        case 0: launch_density(d, c, s); break;
        case 1: launch_force_integrate(d, c, s); break;
        case 2: launch_scan_cells(d, d.n, s); break;
        case 3: launch_scatter(d.key_slot, d.cell_start, d.n, d.tmp, d.counts, s); break;
        case 4:
            launch_rank_gather(d.key_slot, d.cell_start, d.tmp, d.pos2, d.vel2, d.n, d.pos, d.vel, d.tile_sums,
                               d.ntiles, s);
            break;
        default: break;
    }
}

void enqueue_step(DeviceState& d, const SimConst& c, cudaStream_t s) {
    if (d.table && d.tune.batch_cluster && d.scene_order && d.scene_queue && d.n) {
        const int block = d.tune.batch_block ? d.tune.batch_block : 256;
        const int nclusters = batch_persistent_clusters(d.tune.batch_cluster, block, c.reach);
        if (nclusters > 0) {
            const BatchStep a{d.pos,       d.vel,         d.pos2,        d.vel2,     d.pr,      d.rho,
                              d.key_slot,  d.tmp,         d.nbr,         d.nbr_count, d.pv,     d.counts,
                              d.cell_start, d.table,      d.scene_off,   d.scene_order, d.scene_queue, d.nscenes,
                              d.n};
            launch_batch_persistent(a, d.tune.batch_cluster, block, nclusters, c.reach, s);
            return;
        }
    }
    for (uint32_t st = 0; st < kNumStages; ++st) enqueue_stage(st, d, c, s);
}

}  // namespace sf
