// sf_force.cu — force + integration pass of the SPH sub-step (sm_103a).
//
// One thread per cell-sorted particle.  Pressure (spiky gradient, symmetrised
// (p_i + p_j) / (2 rho_j) weight), viscosity (Laplacian) and gravity from the
// neighbour list of the density pass — or from a rescan of the candidate cells
// where the list overflowed or no list was recorded — then, in the stepping
// variant, symplectic Euler, the box clamp with restitution and the next
// step's cell key and arrival slot (the counting sort's histogram).
// A neighbour on the list is one 32-byte record written by the density pass,
// (x, y, z, p) and (vx, vy, vz, 1/rho), fetched with one 256-bit load.
// kPrefetch neighbours are gathered before their terms are added, and the
// next kPrefetch list entries are loaded while they are, so the dependent
// index -> data loads of consecutive batches overlap; the terms are still
// added in list order, which keeps the sum bit-identical.  Lists of 16-bit
// entries (SF_LIST_TILE16) are decoded to indices where they are used.  The
// per-particle pass itself (force_one) is in sf_passes.cuh.
#include "sf_passes.cuh"

namespace sf {
namespace {

template <int kList, int kPrefetch, int kBlockSize, bool kIntegrate, int kReach, bool kBatched>
__global__ void __launch_bounds__(kBlockSize)
    k_force(const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ pr,
            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
            const uint8_t* __restrict__ nbr_wide, const float4* __restrict__ pv, uint32_t n, SimConst c0, const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off,
            uint32_t nscenes, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
            uint32_t* __restrict__ counts, uint32_t* __restrict__ tile_sums, uint2* __restrict__ key_slot,
            float4* __restrict__ acc_out, float4* __restrict__ sums, FrameState* __restrict__ frame) {
    grid_dependency_wait();
    allow_dependents();
    const uint32_t i = blockIdx.x * kBlockSize + threadIdx.x;
    uint32_t v2 = 0u, a2 = 0u;
    if (i < n)
        force_one<kList, kPrefetch, kIntegrate, kReach, kBatched>(i, pos, vel, pr, cs, nbr, nbr_count, nbr_wide, pv, n, c0,
                                                                  table,
                                                                     scene_off, nscenes, pos_out, vel_out, counts,
                                                                     tile_sums, key_slot, acc_out, sums, frame, v2, a2);
    if (!kBatched && kIntegrate && frame && c0.adaptive) {
        // maxima of |v'|^2 and |a|^2 over the block (non-negative floats order
        // like their bits), then one atomic each per block
        __shared__ uint32_t s_max[2][kBlockSize / 32];
        v2 = __reduce_max_sync(0xffffffffu, v2);
        a2 = __reduce_max_sync(0xffffffffu, a2);
        if ((threadIdx.x & 31) == 0) {
            s_max[0][threadIdx.x / 32] = v2;
            s_max[1][threadIdx.x / 32] = a2;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const bool have = threadIdx.x < kBlockSize / 32;
            const uint32_t mv = __reduce_max_sync(0xffffffffu, have ? s_max[0][threadIdx.x] : 0u);
            const uint32_t ma = __reduce_max_sync(0xffffffffu, have ? s_max[1][threadIdx.x] : 0u);
            if (threadIdx.x == 0) {
                atomicMax(&frame->v2max_bits, mv);
                atomicMax(&frame->a2max_bits, ma);
            }
        }
    }
}

template <int kList, int kPrefetch, int kBlockSize, bool kIntegrate>
void force_as(DeviceState& d, const SimConst& c, cudaStream_t s) {
    cudaAccessPolicyWindow w{};
    const cudaAccessPolicyWindow* win =
        (kList != 0 && d.tune.l2_window && persisting_window(d.pv, (size_t)d.n * 2 * sizeof(float4), &w)) ? &w
                                                                                                           : nullptr;
    with_reach(c.reach, [&](auto R) {
        constexpr int K = decltype(R)::value;
        float4* po = kIntegrate ? d.pos2 : nullptr;
        float4* vo = kIntegrate ? d.vel2 : nullptr;
        uint32_t* co = kIntegrate ? d.counts : nullptr;
        uint32_t* ts = kIntegrate ? d.tile_sums : nullptr;
        uint2* ks = kIntegrate ? d.key_slot : nullptr;
        float4* ac = kIntegrate ? nullptr : d.accel;
        if (d.table) {
            if constexpr (K <= 2 && kPrefetch == 2)
                launch_chained_window(win, k_force<kList, kPrefetch, kBlockSize, kIntegrate, K, true>,
                               grid_for(d.n, kBlockSize), kBlockSize, s, d.pos, d.vel, d.pr, d.cell_start, d.nbr,
                               d.nbr_count, d.nbr_wide, d.pv, d.n, c, d.table,
                               d.scene_off, d.nscenes, po, vo, co, ts, ks, ac, d.sums, (FrameState*)nullptr);
        } else {
            launch_chained_window(win, k_force<kList, kPrefetch, kBlockSize, kIntegrate, K, false>,
                           grid_for(d.n, kBlockSize), kBlockSize, s, d.pos, d.vel, d.pr, d.cell_start, d.nbr,
                           d.nbr_count, d.nbr_wide, d.pv, d.n, c,
                           (const SimConst*)nullptr, (const uint32_t*)nullptr, 0u, po, vo, co, ts, ks, ac, d.sums,
                           kIntegrate ? d.frame : nullptr);
        }
    });
}

template <bool kIntegrate>
void launch_force(DeviceState& d, const SimConst& c, cudaStream_t s) {
    if (!d.n) return;
    const bool big = d.tune.force_block == 256;
    if (!d.nbr || d.tune.list_mode == SF_LIST_NONE) {
        big ? force_as<0, 2, 256, kIntegrate>(d, c, s) : force_as<0, 2, 128, kIntegrate>(d, c, s);
    } else if (d.tune.list_mode == SF_LIST_TILE16 && d.nbr_wide) {
        if (d.tune.prefetch == 2)
            big ? force_as<2, 2, 256, kIntegrate>(d, c, s) : force_as<2, 2, 128, kIntegrate>(d, c, s);
        else
            big ? force_as<2, 4, 256, kIntegrate>(d, c, s) : force_as<2, 4, 128, kIntegrate>(d, c, s);
    } else if (d.tune.prefetch == 2) {
        big ? force_as<1, 2, 256, kIntegrate>(d, c, s) : force_as<1, 2, 128, kIntegrate>(d, c, s);
    } else {
        big ? force_as<1, 4, 256, kIntegrate>(d, c, s) : force_as<1, 4, 128, kIntegrate>(d, c, s);
    }
}

}  // namespace

SF_INDEX_CHECK_ACCESSOR(index_check_failures_force)

void launch_force_integrate(DeviceState& d, const SimConst& c, cudaStream_t s) { launch_force<true>(d, c, s); }

void launch_force_only(DeviceState& d, const SimConst& c, cudaStream_t s) { launch_force<false>(d, c, s); }

}  // namespace sf
