// sf_device.cuh — device helpers shared by the kernels of the SPH sub-step.
//
// The translation units that include this header are compiled with
// -fmad=false: multiply-adds are fused only where fmaf() is written, so the
// arithmetic matches the CPU oracle operation for operation.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "sf_internal.h"

namespace sf {

constexpr int kBlock = 256;

inline unsigned grid_for(uint32_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Streaming multiprocessors of the current device (queried once per device).
inline int sm_count() {
    constexpr int kDevices = 64;
    static std::atomic<int> cached[kDevices] = {};
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kDevices && (v = cached[dev].load(std::memory_order_relaxed)) > 0) return v;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    v = std::max(v, 1);
    if (dev >= 0 && dev < kDevices) cached[dev].store(v, std::memory_order_relaxed);
    return v;
}

// Programmatic dependent launch.  The kernels of a sub-step are launched with
// launch_chained(): each may begin launching while its predecessor in the
// stream finishes.  Every such kernel calls grid_dependency_wait() before it
// touches global memory (it returns once the predecessor has completed and its
// writes are visible; a no-op without one), then allow_dependents() so that
// the next kernel's blocks are scheduled during this kernel's last wave.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// launch_chained with an access-policy window (null: none): accesses inside
// the window are cached in L2 as persisting lines, evicted after all others.
template <typename... KArgs, typename... Args>
inline void launch_chained_window(const cudaAccessPolicyWindow* window, void (*kernel)(KArgs...), unsigned grid,
                                  unsigned block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (window) {
        attr[1].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[1].val.accessPolicyWindow = *window;
        cfg.numAttrs = 2;
    }
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <typename... KArgs, typename... Args>
inline void launch_chained(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
    launch_chained_window(nullptr, kernel, grid, block, s, args...);
}

// Calls f(std::integral_constant<int, K>) for the context's reach K.
template <typename F>
inline void with_reach(int reach, F&& f) {
    switch (reach) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        default: f(std::integral_constant<int, 2>{}); break;
    }
}

__device__ __forceinline__ int cell_coord(float x, float bmin, float inv_cell, int n) {
    const float t = floorf((x - bmin) * inv_cell);
    return (t >= 0.f) ? ((t < (float)n) ? (int)t : n - 1) : 0;  // NaN -> 0
}

__device__ __forceinline__ uint32_t cell_key(const SimConst& c, float x, float y, float z) {
    const int cx = cell_coord(x, c.bmin[0], c.inv_cell[0], c.n[0]);
    const int cy = cell_coord(y, c.bmin[1], c.inv_cell[1], c.n[1]);
    const int cz = cell_coord(z, c.bmin[2], c.inv_cell[2], c.n[2]);
    return c.cell_base + ((uint32_t)cz * (uint32_t)c.n[1] + (uint32_t)cy) * (uint32_t)c.n[0] + (uint32_t)cx;
}

// Scene of particle i in a batch: the last s with scene_off[s] <= i.
__device__ __forceinline__ uint32_t scene_of(const uint32_t* __restrict__ scene_off, uint32_t nscenes, uint32_t i) {
    uint32_t lo = 0, hi = nscenes;  // invariant: scene_off[lo] <= i < scene_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(scene_off + mid) <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Constants of particle i: the launch's own, or its scene's in a batch.
template <bool kBatched>
__device__ __forceinline__ SimConst const_of(const SimConst& c0, const SimConst* __restrict__ table,
                                             const uint32_t* __restrict__ scene_off, uint32_t nscenes, uint32_t i) {
    if (!kBatched) return c0;
    return table[scene_of(scene_off, nscenes, i)];
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {  // murmur3 finaliser
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// Loads of the per-particle passes.  kNc: through the read-only path, for
// data that no thread writes during the kernel (every separately launched
// pass).  !kNc: plain (coherent) global loads, for the persistent batched step,
// which writes in one stage what its cluster reads in the next (visible
// across the cluster barrier's release/acquire, which the read-only path does
// not take part in).  The asm is volatile so that no load moves across a
// barrier.
template <bool kNc>
__device__ __forceinline__ float4 ld_f4(const float4* p) {
    if constexpr (kNc) {
        return __ldg(p);
    } else {
        float4 v;
        asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
        return v;
    }
}
template <bool kNc>
__device__ __forceinline__ float2 ld_f2(const float2* p) {
    if constexpr (kNc) {
        return __ldg(p);
    } else {
        float2 v;
        asm volatile("ld.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
        return v;
    }
}
template <bool kNc>
__device__ __forceinline__ uint32_t ld_u32(const uint32_t* p) {
    if constexpr (kNc) {
        return __ldg(p);
    } else {
        uint32_t v;
        asm volatile("ld.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
        return v;
    }
}

// Index checks of the checked build (compiled with SF_DEVICE_CHECKS=1; the
// release build compiles them out).  Every cell-table range end and every
// neighbour-list entry is checked against the particle count before it is
// used: a bad value is counted in this translation unit's counter and
// replaced by an in-range one, so the access stays inside its array and
// nothing traps.  sf_index_checks() reads and resets the counters.
#ifndef SF_DEVICE_CHECKS
#define SF_DEVICE_CHECKS 0
#endif
#if SF_DEVICE_CHECKS
static __device__ unsigned long long g_index_check_failures;  // one per translation unit
#endif
// j, a particle index, where j < n; else 0 (counted)
__device__ __forceinline__ uint32_t checked_index(uint32_t j, uint32_t n) {
#if SF_DEVICE_CHECKS
    if (j >= n) {
        atomicAdd(&g_index_check_failures, 1ull);
        return 0u;
    }
#endif
    (void)n;
    return j;
}
// v, a cell-table entry (a range end), where v <= n; else n (counted)
__device__ __forceinline__ uint32_t checked_end(uint32_t v, uint32_t n) {
#if SF_DEVICE_CHECKS
    if (v > n) {
        atomicAdd(&g_index_check_failures, 1ull);
        return n;
    }
#endif
    (void)n;
    return v;
}
// Host accessor of this translation unit's counter: fn(reset) returns it
// (0 in the release build) and clears it when `reset`.
#if SF_DEVICE_CHECKS
#define SF_INDEX_CHECK_ACCESSOR(fn)                                                               \
    uint64_t fn(bool reset) {                                                                    \
        unsigned long long v = 0;                                                                \
        cudaMemcpyFromSymbol(&v, g_index_check_failures, sizeof(v));                             \
        if (reset) {                                                                             \
            const unsigned long long z = 0;                                                      \
            cudaMemcpyToSymbol(g_index_check_failures, &z, sizeof(z));                           \
        }                                                                                        \
        return v;                                                                                \
    }
#else
#define SF_INDEX_CHECK_ACCESSOR(fn) \
    uint64_t fn(bool) { return 0; }
#endif

// Counting-sort histogram: the particle's arrival slot in its cell, and the
// cell's scan tile total (one atomic per distinct tile per warp).  Call with
// every live lane of the warp converged.
__device__ __forceinline__ uint32_t count_in_cell(uint32_t key, uint32_t* __restrict__ counts,
                                                  uint32_t* __restrict__ tile_sums) {
    const uint32_t slot = atomicAdd(counts + key, 1u);
    if (!tile_sums) return slot;  // the persistent batched step scans each scene without tile totals
    const unsigned mask = __activemask();
    const uint32_t tile = key / (uint32_t)kScanTile;
    const unsigned peers = __match_any_sync(mask, tile);
    if ((threadIdx.x & 31) == (uint32_t)(__ffs(peers) - 1)) atomicAdd(tile_sums + tile, (uint32_t)__popc(peers));
    return slot;
}

// Lower bound, minus the pruning slack, of the axis distance from a point at
// offset `off` inside its cell (width w) to the cell at offset d.
__device__ __forceinline__ float face_gap(float off, int d, float w, float margin) {
    float gap = 0.f;
    if (d > 0) gap = (float)d * w - off;
    if (d < 0) gap = off - (float)(d + 1) * w;
    return fmaxf(gap - margin, 0.f);
}

// Calls f(j, pos[j]) for the neighbour candidates of a particle at (x, y, z)
// in the canonical order: dz = -R..R, dy = -R..R, then the contiguous sorted
// range of the row's cells cx-R..cx+R (R = kReach = cells per kernel radius).
// Rows and end cells whose nearest face is provably farther than h (by a
// margin that covers the rounding of cell assignment) are skipped: they hold
// no neighbour, so skipping them changes no sum and no list.
// This form unrolls the dy rows over per-particle gap tables (fastest where
// the walk is the kernel's main loop); for_candidates_rolled below is the
// same walk in less code and fewer registers, for kernels where it is a rare
// path (the force pass's list-overflow rescan).
// for_candidate_rows calls g(b, e) with the sorted index range [b, e) of each
// candidate row in that order (ranges of rows out of reach are empty).
template <int kReach, bool kNc = true, typename G>
__device__ __forceinline__ void for_candidate_rows(const SimConst& c, const uint32_t* __restrict__ cs, uint32_t n,
                                                   float x, float y, float z, G&& g) {
    const int cx = cell_coord(x, c.bmin[0], c.inv_cell[0], c.n[0]);
    const int cy = cell_coord(y, c.bmin[1], c.inv_cell[1], c.n[1]);
    const int cz = cell_coord(z, c.bmin[2], c.inv_cell[2], c.n[2]);
    const float ox = (x - c.bmin[0]) - (float)cx * c.cell_w[0];  // positions inside the cell
    const float oy = (y - c.bmin[1]) - (float)cy * c.cell_w[1];
    const float oz = (z - c.bmin[2]) - (float)cz * c.cell_w[2];
    const uint32_t n0 = (uint32_t)c.n[0], n1 = (uint32_t)c.n[1];
    // Per row offset dy: the squared gap (infinite outside the grid).  Per row
    // end: the squared gap of the outermost cell, which is dropped when out
    // of reach.  Rounding of these sums is far inside prune_h2's slack.
    float gy2[2 * kReach + 1];
#pragma unroll
    for (int d = -kReach; d <= kReach; ++d) {
        const float g = face_gap(oy, d, c.cell_w[1], c.prune_margin);
        gy2[d + kReach] = (cy + d < 0 || cy + d >= c.n[1]) ? __int_as_float(0x7f800000) : g * g;
    }
    float glo2 = 0.f, ghi2 = 0.f;
    if (kReach > 1) {
        const float gl = face_gap(ox, -kReach, c.cell_w[0], c.prune_margin);
        const float gh = face_gap(ox, kReach, c.cell_w[0], c.prune_margin);
        glo2 = gl * gl;
        ghi2 = gh * gh;
    }
    const int xa = max(cx - kReach, 0), xb = min(cx + kReach, c.n[0] - 1);
    const int xa1 = max(cx - kReach + 1, 0), xb1 = min(cx + kReach - 1, c.n[0] - 1);
#pragma unroll 1
    for (int dz = -kReach; dz <= kReach; ++dz) {
        const int zz = cz + dz;
        if (zz < 0 || zz >= c.n[2]) continue;
        const float gz = face_gap(oz, dz, c.cell_w[2], c.prune_margin);
        const float gz2 = gz * gz;
        if (gz2 >= c.prune_h2) continue;
        // cell table of row (zz, cy); rows dy are n0 entries apart
        const uint32_t* plane = cs + c.cell_base + ((uint32_t)zz * n1 + (uint32_t)cy) * n0;
        // the plane's row ranges, loaded together (empty for rows out of reach)
        uint32_t rb[2 * kReach + 1], re[2 * kReach + 1];
#pragma unroll
        for (int dy = -kReach; dy <= kReach; ++dy) {
            const float g2 = gz2 + gy2[dy + kReach];
            const int x0 = (kReach > 1 && g2 + glo2 >= c.prune_h2) ? xa1 : xa;
            const int x1 = (kReach > 1 && g2 + ghi2 >= c.prune_h2) ? xb1 : xb;
            const uint32_t* row = plane + dy * (int)n0;
            const bool live = g2 < c.prune_h2;
            rb[dy + kReach] = live ? checked_end(ld_u32<kNc>(row + x0), n) : 0u;
            re[dy + kReach] = live ? checked_end(ld_u32<kNc>(row + x1 + 1), n) : 0u;
        }
#pragma unroll
        for (int dy = 0; dy <= 2 * kReach; ++dy) g(rb[dy], re[dy]);
    }
}

template <int kReach, bool kNc = true, typename F>
__device__ __forceinline__ void for_candidates(const SimConst& c, const uint32_t* __restrict__ cs,
                                               const float4* __restrict__ pos, uint32_t n, float x, float y, float z,
                                               F&& f) {
    for_candidate_rows<kReach, kNc>(c, cs, n, x, y, z, [&](uint32_t b, uint32_t e) {
        uint32_t j = b;
#pragma unroll 1
        for (; j + 1 < e; j += 2) {
            const float4 x0 = ld_f4<kNc>(pos + j), x1 = ld_f4<kNc>(pos + j + 1);
            f(j, x0);
            f(j + 1, x1);
        }
        if (j < e) f(j, ld_f4<kNc>(pos + j));
    });
}

// *p = v where `pred` holds, as one predicated store (no branch).  No memory
// clobber: the caller's kernel never reads what these stores write.
__device__ __forceinline__ void store_if(uint32_t* p, uint32_t v, bool pred) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.u32 [%0], %1;\n\t}" ::"l"(p),
                 "r"(v), "r"((uint32_t)pred));
}

// The low 16 bits of v at *p where `pred` holds (one predicated store; the
// store truncates the 32-bit register).
__device__ __forceinline__ void store16_if(uint16_t* p, uint32_t v, bool pred) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.u16 [%0], %1;\n\t}" ::"l"(p),
                 "r"(v), "r"((uint32_t)pred));
}

// A 16-bit list entry (zero-extended; read-only path).
__device__ __forceinline__ uint32_t ld16(const uint16_t* p) {
    uint32_t v;
    asm volatile("ld.global.nc.u16 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// The neighbour index of a 16-bit entry e of particle i: the index within
// 32767 places of i whose low 16 bits are e.
__device__ __forceinline__ uint32_t near_index(uint32_t i, uint32_t e) {
    return i + (uint32_t)(int32_t)(int16_t)(uint16_t)(e - i);
}

// The candidate walk above with both row loops rolled and the gaps computed
// per row.
template <int kReach, bool kNc = true, typename F>
__device__ __forceinline__ void for_candidates_rolled(const SimConst& c, const uint32_t* __restrict__ cs,
                                               const float4* __restrict__ pos, uint32_t n, float x, float y, float z,
                                               F&& f) {
    const int cx = cell_coord(x, c.bmin[0], c.inv_cell[0], c.n[0]);
    const int cy = cell_coord(y, c.bmin[1], c.inv_cell[1], c.n[1]);
    const int cz = cell_coord(z, c.bmin[2], c.inv_cell[2], c.n[2]);
    const float ox = (x - c.bmin[0]) - (float)cx * c.cell_w[0];  // positions inside the cell
    const float oy = (y - c.bmin[1]) - (float)cy * c.cell_w[1];
    const float oz = (z - c.bmin[2]) - (float)cz * c.cell_w[2];
#pragma unroll 1
    for (int dz = -kReach; dz <= kReach; ++dz) {
        const int zz = cz + dz;
        if (zz < 0 || zz >= c.n[2]) continue;
        const float gz = face_gap(oz, dz, c.cell_w[2], c.prune_margin);
#pragma unroll 1
        for (int dy = -kReach; dy <= kReach; ++dy) {
            const int yy = cy + dy;
            if (yy < 0 || yy >= c.n[1]) continue;
            const float gy = face_gap(oy, dy, c.cell_w[1], c.prune_margin);
            const float g2 = fmaf(gz, gz, gy * gy);
            if (g2 >= c.prune_h2) continue;
            int lo = -kReach, hi = kReach;
            if (kReach > 1) {  // drop the row's outermost cell on a side when it is out of reach
                const float gl = face_gap(ox, -kReach, c.cell_w[0], c.prune_margin);
                const float gh = face_gap(ox, kReach, c.cell_w[0], c.prune_margin);
                if (fmaf(gl, gl, g2) >= c.prune_h2) lo = 1 - kReach;
                if (fmaf(gh, gh, g2) >= c.prune_h2) hi = kReach - 1;
            }
            const int x0 = max(cx + lo, 0), x1 = min(cx + hi, c.n[0] - 1);
            const uint32_t row = c.cell_base + ((uint32_t)zz * (uint32_t)c.n[1] + (uint32_t)yy) * (uint32_t)c.n[0];
            const uint32_t b = checked_end(ld_u32<kNc>(cs + row + x0), n),
                           e = checked_end(ld_u32<kNc>(cs + row + x1 + 1), n);
#pragma unroll 1
            for (uint32_t j = b; j < e; ++j) f(j, ld_f4<kNc>(pos + j));
        }
    }
}

// One 32-byte record in one access (sm_100+ 256-bit vector load / store);
// kNc as for ld_f4.
template <bool kNc = true>
__device__ __forceinline__ void ld8(const float4* __restrict__ p, float4& a, float4& b) {
    if constexpr (kNc)
        asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                     : "l"(p));
    else
        asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                     : "l"(p));
}
__device__ __forceinline__ void st8(float4* __restrict__ p, const float4& a, const float4& b) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}

// The sub-step's dt from the previous sub-step's maxima (adaptive: CFL on
// |v| and |a|; fixed: time_step), then the maxima restart for this sub-step.
__device__ __forceinline__ void choose_dt(FrameState* __restrict__ fs, const SimConst& c) {
    float dt = c.dt;
    if (c.adaptive) {
        const float v2 = __uint_as_float(fs->v2max_bits), a2 = __uint_as_float(fs->a2max_bits);
        if (v2 > 0.f) dt = fminf(dt, (c.cfl_v * c.h) / sqrtf(v2));
        if (a2 > 0.f) dt = fminf(dt, c.cfl_a * sqrtf(c.h / sqrtf(a2)));
    }
    fs->dt = dt;
    fs->v2max_bits = 0u;
    fs->a2max_bits = 0u;
}

// Equation of state and the p >= 0 clamp (SPHParameters::bUseAttractivePressure).
__device__ __forceinline__ float pressure_of(const SimConst& c, float rho) {
    float p;
    if (c.eos == SF_EOS_TAIT) {
        const float x = rho * c.inv_rho0;
        const float x2 = x * x;
        const float x4 = x2 * x2;
        const float x7 = (x4 * x2) * x;
        p = c.k * (x7 - 1.f);
    } else {
        p = c.k * (rho - c.rho0);
    }
    if (!c.attractive) p = (p < 0.f) ? 0.f : p;
    return p;
}

// Index of particle i's k-th neighbour in the list buffer: tiles of kNbTile
// particles, k-major inside a tile, so a warp reads one 128-byte line per k.
__device__ __forceinline__ size_t nbr_index(uint32_t i, uint32_t k) {
    return ((size_t)(i / kNbTile) * kNbCap + k) * kNbTile + (i % kNbTile);
}
// SF_LIST_TILE16 lists are laid out in warp tiles of kNbWarpTile particles,
// each of which holds either 32-bit entries (nbr_w32_index, in 32-bit units)
// or 16-bit entries (nbr_w16_index, in 16-bit units: the first half of the
// tile's 32-bit region), so tiles of either width sit side by side.
__device__ __forceinline__ size_t nbr_w32_index(uint32_t i, uint32_t k) {
    return ((size_t)(i / kNbWarpTile) * kNbCap + k) * kNbWarpTile + (i % kNbWarpTile);
}
__device__ __forceinline__ size_t nbr_w16_index(uint32_t i, uint32_t k) {
    return ((size_t)(i / kNbWarpTile) * (2 * kNbCap) + k) * kNbWarpTile + (i % kNbWarpTile);
}

// Pair terms of particle i with neighbour j (|xi - xj| < h; j == i adds exact
// zeros), in the oracle's operation order.
struct PairAcc {
    float apx = 0.f, apy = 0.f, apz = 0.f, avx = 0.f, avy = 0.f, avz = 0.f;
};

// A pointer the compiler cannot see through, so loads through it are issued
// where they are written (not hoisted, not merged with earlier loads).
template <typename T>
__device__ __forceinline__ const T* opaque_ptr(const T* p) {
    const T* r;
    asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(p));
    return r;
}

__device__ __forceinline__ void pair_terms(float h, const float4& xi, const float4& vi, float pi,
                                           const float4& xj, const float2& prj, const float4& vj, PairAcc& a) {
    const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float r = sqrtf(r2);
    const float hr = h - r;
    const float w = hr * prj.y;
    a.avx = fmaf(w, vj.x - vi.x, a.avx);
    a.avy = fmaf(w, vj.y - vi.y, a.avy);
    a.avz = fmaf(w, vj.z - vi.z, a.avz);
    // The pressure term needs r > 0.  Without a branch: the quotient is taken
    // over r = 1 where r == 0 (so it stays finite), then the term's weight is
    // set to zero there, and fma(0, d, a) == a (d is finite, and an
    // accumulator that starts at +0 is never -0).
    const bool apart = r > 0.f;
    const float sp_r = ((pi + prj.x) * w) * (hr / (apart ? r : 1.f));
    const float sp = apart ? sp_r : 0.f;
    a.apx = fmaf(sp, dx, a.apx);
    a.apy = fmaf(sp, dy, a.apy);
    a.apz = fmaf(sp, dz, a.apz);
}

}  // namespace sf
