// sf_density.cu — density pass of the SPH sub-step (sm_103a).
//
// One thread per cell-sorted particle.  Poly6 density over the canonical
// candidates; non-neighbours add an exact zero (fma(0, 0, s) == s), so the sum
// is branch-free and bit-identical to summing neighbours only.  The pass also
// evaluates the equation of state, writes each particle's 32-byte record for
// the force pass's gathers ((x, y, z, p), (vx, vy, vz, 1/rho)), and records
// each particle's neighbours (itself included, in its canonical place) for the
// force pass:
//   kEmitNone    no list (the force pass rescans the candidate cells);
//   kEmitStaged  list staged in shared memory, written out in full lines;
//   kEmitTile    list written directly;
//   kEmitTile16  list written directly as 16-bit entries: the low half of the
//                neighbour's index, from which the force pass recovers it as
//                j = i + (int16_t)(entry - i).  That is exact while every
//                candidate lies within kNear16 sorted places of i, which each
//                particle checks before its walk from the cell table (all its
//                candidates lie between the start of its lowest candidate cell
//                and the end of its highest).  These lists are laid out in
//                warp tiles (kNbWarpTile particles); a tile in which any
//                particle fails the check stores 32-bit entries instead and
//                marks itself in nbr_wide.
// The other list modes use the tile layout of nbr_index().  nbr_count[i] is the
// full count; a count above kNbCap makes the force pass rescan that particle's
// candidates instead of reading the list.  Recording the particle itself saves
// a comparison per candidate; its pair terms in the force pass are exact
// zeros (fma(w, v_i - v_i, a) == a, and the pressure term needs r > 0).
// The per-particle pass itself (density_one) is in sf_passes.cuh.
#include "sf_passes.cuh"

namespace sf {
namespace {

template <int kMode, int kBlockSize, int kReach, bool kBatched>
__global__ void __launch_bounds__(kBlockSize)
    k_density(const float4* __restrict__ pos, const uint32_t* __restrict__ cs, uint32_t n, SimConst c0,
              const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off, uint32_t nscenes,
              float* __restrict__ rho_out, float2* __restrict__ pr_out, uint32_t* __restrict__ nbr,
              uint32_t* __restrict__ nbr_count, uint8_t* __restrict__ nbr_wide, const float4* __restrict__ vel,
              float4* __restrict__ pv, FrameState* __restrict__ frame) {
    __shared__ uint32_t s_nb[kMode == kEmitStaged ? kNbCap : 1][kMode == kEmitStaged ? kBlockSize : 1];
    grid_dependency_wait();
    allow_dependents();
    // a stepping pass with a frame state chooses this sub-step's dt
    if (frame && blockIdx.x == 0 && threadIdx.x == 0) choose_dt(frame, c0);
    const uint32_t t = threadIdx.x;
    const uint32_t i = blockIdx.x * kBlockSize + t;
    const bool live = i < n;
    const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, live ? i : 0u);
    const float4 xi = live ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // 16-bit entries: is every candidate of every particle of this warp near?
    bool wide = false;
    if constexpr (kMode == kEmitTile16) {
        const bool far = live && !candidates_near<kReach>(c, cs, n, i, xi.x, xi.y, xi.z);
        wide = __any_sync(0xffffffffu, far);
        if (live && i % kNbWarpTile == 0) nbr_wide[i / kNbWarpTile] = wide ? 1 : 0;
    }
    uint32_t cnt = 0;
    if (live)
        cnt = density_one<kMode, kReach>(i, c, xi, pos, cs, n, rho_out, pr_out, nbr, nbr_count, vel, pv, wide,
                                          kMode == kEmitStaged ? &s_nb[0][t] : nullptr, kBlockSize);
    if (kMode == kEmitStaged) {
        // Copy each warp's recorded rows out in full 128-byte lines.
        const uint32_t kmax = __reduce_max_sync(0xffffffffu, min(cnt, (uint32_t)kNbCap));
        uint32_t* tile = nbr + (size_t)blockIdx.x * kNbCap * kNbTile + t;
        for (uint32_t k = 0; k < kmax; ++k) tile[(size_t)k * kNbTile] = s_nb[k][t];
    }
}

template <int kMode, int kBlockSize>
void density_as(const DeviceState& d, const SimConst& c, cudaStream_t s) {
    // the gather records are written here and gathered by the force pass
    cudaAccessPolicyWindow w{};
    const cudaAccessPolicyWindow* win =
        (kMode != kEmitNone && d.tune.l2_window && persisting_window(d.pv, (size_t)d.n * 2 * sizeof(float4), &w))
            ? &w
            : nullptr;
    with_reach(c.reach, [&](auto R) {
        constexpr int K = decltype(R)::value;
        if (d.table) {
            if constexpr (K <= 2)
                launch_chained_window(win, k_density<kMode, kBlockSize, K, true>, grid_for(d.n, kBlockSize), kBlockSize, s,
                               d.pos, d.cell_start, d.n, c, d.table, d.scene_off, d.nscenes, d.rho, d.pr, d.nbr,
                               d.nbr_count, d.nbr_wide, d.vel, d.pv, (FrameState*)nullptr);
        } else {
            launch_chained_window(win, k_density<kMode, kBlockSize, K, false>, grid_for(d.n, kBlockSize), kBlockSize, s, d.pos,
                           d.cell_start, d.n, c, nullptr, nullptr, 0u, d.rho, d.pr, d.nbr, d.nbr_count, d.nbr_wide,
                           d.vel, d.pv, d.frame);
        }
    });
}

}  // namespace

SF_INDEX_CHECK_ACCESSOR(index_check_failures_density)

void launch_density(const DeviceState& d, const SimConst& c, cudaStream_t s) {
    if (!d.n) return;
    const bool big = d.tune.density_block == 256;
    if (!d.nbr || d.tune.list_mode == SF_LIST_NONE) {
        big ? density_as<kEmitNone, 256>(d, c, s) : density_as<kEmitNone, 128>(d, c, s);
    } else if (d.tune.list_mode == SF_LIST_TILE_STAGED) {
        density_as<kEmitStaged, kNbTile>(d, c, s);
    } else if (d.tune.list_mode == SF_LIST_TILE16 && d.nbr_wide) {
        big ? density_as<kEmitTile16, 256>(d, c, s) : density_as<kEmitTile16, 128>(d, c, s);
    } else {
        big ? density_as<kEmitTile, 256>(d, c, s) : density_as<kEmitTile, 128>(d, c, s);
    }
}

}  // namespace sf
