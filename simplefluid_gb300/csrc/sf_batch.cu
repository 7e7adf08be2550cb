// sf_batch.cu — the persistent batched step (sm_103a).
//
// One launch advances every scene of a batch by one sub-step.  The grid holds
// as many thread-block clusters as the GPU keeps resident; each cluster takes
// whole scenes from a queue (scenes in decreasing particle count, so the
// largest start first) and runs the five stages of the scene's sub-step
// itself, separated by the cluster's hardware barrier:
//   A density and lists    B forces, integration and the next histogram
//   C scan of the scene's cells into its cell table
//   D bucketing by cell    E stable rank and gather
// Scenes own disjoint particle ranges and cell ranges, so clusters never wait
// for one another: the only shared word is the queue counter (atomics), and a
// scene's data stay in L2 across its five stages.  Every stage performs the
// operations of the separately launched passes in the same order, so the
// results are bit-identical to the five-kernel step.
//
// Loads of data written earlier in the same launch are plain (coherent)
// global loads: each barrier.cluster arrive/wait pair is a release/acquire at
// cluster scope, which makes a stage's writes visible to the next stage's
// reads on every SM of the cluster.  No load goes through the read-only path.
#include "sf_passes.cuh"

namespace sf {
namespace {

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_blocks() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// All threads of the cluster: release this thread's writes, wait for every
// thread, acquire theirs.  (Not the .aligned form: threads may arrive from
// loops of different trip counts.)
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// The word at `p` in the shared memory of the cluster's block `rank`.
__device__ __forceinline__ uint32_t ld_shared_of(const uint32_t* p, uint32_t rank) {
    const uint32_t local = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t remote, v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(remote) : "memory");
    return v;
}
__device__ __forceinline__ uint4 ld_u32x4(const uint4* p) {
    uint4 v;
    asm volatile("ld.global.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld_u32x2(const uint2* p) {
    uint2 v;
    asm volatile("ld.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

// Inclusive warp scan.
__device__ __forceinline__ uint32_t warp_scan(uint32_t x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

template <int kReach, int kPBlock>
__global__ void __launch_bounds__(kPBlock) k_batch_persistent(BatchStep a) {
    __shared__ SimConst s_c;
    __shared__ uint32_t s_next[2];
    __shared__ uint32_t s_warp[2][kPBlock / 32];
    __shared__ uint32_t s_total;  // this block's share of the scene's cell counts (read by the later blocks)
    const uint32_t rank = cluster_rank(), nblk = cluster_blocks();
    const uint32_t tid = rank * kPBlock + threadIdx.x, nthreads = nblk * kPBlock;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t it = 0;; ++it) {
        // the next scene: block 0 takes it from the queue; the barrier also
        // ends the previous scene
        uint32_t* const slot = &s_next[it & 1];
        if (rank == 0 && threadIdx.x == 0) *slot = atomicAdd(a.queue, 1u);
        cluster_sync();
        const uint32_t q = ld_shared_of(slot, 0);
        if (q >= a.nscenes) break;
        const uint32_t s = a.order[q];
        if (threadIdx.x == 0) s_c = a.table[s];
        __syncthreads();
        const SimConst& c = s_c;
        const uint32_t off = a.scene_off[s], end = a.scene_off[s + 1];

        // A: density, equation of state, gather records, neighbour lists
        for (uint32_t i = off + tid; i < end; i += nthreads) {
            const float4 xi = ld_f4<false>(a.pos + i);
            density_one<kEmitTile, kReach, false>(i, c, xi, a.pos, a.cell_start, a.n, a.rho, a.pr, a.nbr, a.nbr_count,
                                                  a.vel, a.pv, false, nullptr, 0);
        }
        cluster_sync();

        // B: forces, integration, box, next cell key and arrival slot
        for (uint32_t i = off + tid; i < end; i += nthreads) {
            uint32_t v2 = 0u, a2 = 0u;
            force_one<1, 2, true, kReach, false, false>(i, a.pos, a.vel, a.pr, a.cell_start, a.nbr, a.nbr_count,
                                                        nullptr, a.pv, a.n, c, nullptr, nullptr, 0u, a.pos2, a.vel2,
                                                        a.counts, nullptr, a.key_slot, nullptr, nullptr, nullptr, v2,
                                                        a2);
        }
        cluster_sync();

        // C: exclusive scan of the scene's cell counts, offset by its first
        // particle, into its cell table.  The scene's cells [cb, cb + 4 Q)
        // are Q groups of four (scene cell ranges are padded to groups of
        // four); block r scans the groups [r L, (r + 1) L) after summing the
        // totals of the blocks before it.
        {
            const uint32_t Q = (c.ncells + 3) / 4, L = (Q + nblk - 1) / nblk;
            const uint32_t g0 = min(rank * L, Q), g1 = min(g0 + L, Q);
            const uint4* cnt4 = reinterpret_cast<const uint4*>(a.counts + c.cell_base);
            uint4* cs4 = reinterpret_cast<uint4*>(a.cell_start + c.cell_base);
            uint32_t part = 0;
            for (uint32_t g = g0 + threadIdx.x; g < g1; g += kPBlock) {
                const uint4 v = ld_u32x4(cnt4 + g);
                part += v.x + v.y + v.z + v.w;
            }
            part = __reduce_add_sync(0xffffffffu, part);
            if (lane == 0) s_warp[0][warp] = part;
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (int w = 0; w < kPBlock / 32; ++w) t += s_warp[0][w];
                s_total = t;
            }
            cluster_sync();
            uint32_t base = off;
            for (uint32_t r = 0; r < rank; ++r) base += ld_shared_of(&s_total, r);
            // tiles of kPBlock groups; the warp totals alternate between two
            // buffers, so one barrier per tile keeps a tile's writes from
            // meeting the previous tile's reads
            for (uint32_t t0 = g0, k = 0; t0 < g1; t0 += kPBlock, ++k) {
                uint32_t* const ws = s_warp[k & 1];
                const uint32_t g = t0 + threadIdx.x;
                const uint4 v = g < g1 ? ld_u32x4(cnt4 + g) : make_uint4(0u, 0u, 0u, 0u);
                const uint32_t sum = v.x + v.y + v.z + v.w;
                const uint32_t inc = warp_scan(sum);
                if (lane == 31) ws[warp] = inc;
                __syncthreads();
                uint32_t before = base, tile = 0;
#pragma unroll
                for (int w = 0; w < kPBlock / 32; ++w) {
                    const uint32_t x = ws[w];
                    before += w < warp ? x : 0u;
                    tile += x;
                }
                if (g < g1) {
                    // entries clamped to the scene's end, as the flat scan clamps to n
                    const uint32_t ex = before + inc - sum;
                    cs4[g] = make_uint4(min(ex, end), min(ex + v.x, end), min(ex + v.x + v.y, end),
                                        min(ex + v.x + v.y + v.z, end));
                }
                base += tile;
            }
        }
        cluster_sync();

        // D: bucket the unsorted indices by cell; clear the counters
        for (uint32_t i = off + tid; i < end; i += nthreads) {
            const uint2 ks = ld_u32x2(a.key_slot + i);
            const uint32_t at = ld_u32<false>(a.cell_start + ks.x) + ks.y;
            if (at < end) a.tmp[at] = i;  // always, unless the histogram was inconsistent
            a.counts[ks.x] = 0u;
        }
        cluster_sync();

        // E: stable rank inside each cell, gather the integrated state
        for (uint32_t i = off + tid; i < end; i += nthreads) {
            const float4 p = ld_f4<false>(a.pos2 + i), v = ld_f4<false>(a.vel2 + i);
            const uint32_t key = ld_u32x2(a.key_slot + i).x;
            const uint32_t b = ld_u32<false>(a.cell_start + key), e = ld_u32<false>(a.cell_start + key + 1);
            uint32_t r = 0;
            for (uint32_t t = b; t < e; ++t) r += (ld_u32<false>(a.tmp + t) < i) ? 1u : 0u;
            const uint32_t dst = b + r;
            if (dst < end) {  // always, unless the histogram was inconsistent
                a.pos[dst] = p;
                a.vel[dst] = v;
            }
        }
    }
    // no block leaves while another may still read its shared memory
    cluster_sync();
}

// Calls f(kernel) with the persistent kernel of this reach and block size.
template <typename F>
bool with_persistent_kernel(int reach, int block, F&& f) {
    if (block == 256) {
        reach == 1 ? f(k_batch_persistent<1, 256>) : f(k_batch_persistent<2, 256>);
    } else if (block == 512) {
        reach == 1 ? f(k_batch_persistent<1, 512>) : f(k_batch_persistent<2, 512>);
    } else if (block == 1024) {
        reach == 1 ? f(k_batch_persistent<1, 1024>) : f(k_batch_persistent<2, 1024>);
    } else {
        return false;
    }
    return true;
}

cudaLaunchConfig_t persistent_config(int cluster, int block, unsigned grid, cudaStream_t s, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

}  // namespace

int batch_persistent_clusters(int cluster, int block, int reach) {
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = persistent_config(cluster, block, (unsigned)cluster, nullptr, attr);
    int nclusters = 0;
    cudaError_t e = cudaErrorInvalidValue;
    with_persistent_kernel(reach, block,
                           [&](auto kernel) { e = cudaOccupancyMaxActiveClusters(&nclusters, kernel, &cfg); });
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nclusters;
}

void launch_batch_persistent(const BatchStep& a, int cluster, int block, int nclusters, int reach, cudaStream_t s) {
    cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), s);
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = persistent_config(cluster, block, (unsigned)(nclusters * cluster), s, attr);
    with_persistent_kernel(reach, block, [&](auto kernel) { cudaLaunchKernelEx(&cfg, kernel, a); });
}

}  // namespace sf
