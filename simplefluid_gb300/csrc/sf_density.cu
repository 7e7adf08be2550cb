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
//   kEmitTile    list written directly.
// Both list modes use the tile layout of nbr_index().  nbr_count[i] is the
// full count; a count above kNbCap makes the force pass rescan that particle's
// candidates instead of reading the list.  Recording the particle itself saves
// a comparison per candidate; its pair terms in the force pass are exact
// zeros (fma(w, v_i - v_i, a) == a, and the pressure term needs r > 0).
#include "sf_device.cuh"

namespace sf {
namespace {

template <int kMode, int kBlockSize, int kReach, bool kBatched>
__global__ void __launch_bounds__(kBlockSize)
    k_density(const float4* __restrict__ pos, const uint32_t* __restrict__ cs, uint32_t n, SimConst c0,
              const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off, uint32_t nscenes,
              float* __restrict__ rho_out, float2* __restrict__ pr_out, uint32_t* __restrict__ nbr,
              uint32_t* __restrict__ nbr_count, const float4* __restrict__ vel, float4* __restrict__ pv,
              FrameState* __restrict__ frame) {
    __shared__ uint32_t s_nb[kMode == kEmitStaged ? kNbCap : 1][kMode == kEmitStaged ? kBlockSize : 1];
    grid_dependency_wait();
    allow_dependents();
    // a stepping pass with a frame state chooses this sub-step's dt
    if (frame && blockIdx.x == 0 && threadIdx.x == 0) choose_dt(frame, c0);
    const uint32_t t = threadIdx.x;
    const uint32_t i = blockIdx.x * kBlockSize + t;
    uint32_t cnt = 0;
    if (i < n) {
        const SimConst c = const_of<kBatched>(c0, table, scene_off, nscenes, i);
        const float4 xi = pos[i];
        float s = 0.f;
        uint32_t* const lst = kMode == kEmitTile ? nbr + nbr_index(i, 0) : nullptr;  // slot k at lst[k * kNbTile]
        for_candidates<kReach>(c, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const bool near = r2 < c.h2;
            const float q = near ? c.h2 - r2 : 0.f;
            s = fmaf(q * q, q, s);
            if (kMode == kEmitTile) {
                // Predicated store, no branch.  Past the cap the last slot is
                // overwritten: such a list is never read (the force pass
                // rescans particles whose count exceeds the cap).
                store_if(lst + (size_t)min(cnt, (uint32_t)kNbCap - 1) * kNbTile, j, near);
                cnt += near ? 1u : 0u;
            } else if (kMode == kEmitStaged && near) {
                if (cnt < kNbCap) s_nb[cnt][t] = j;
                ++cnt;
            }
        });
        const float rho = c.cd * s;
        const float p = pressure_of(c, rho), inv_rho = 1.f / rho;
        rho_out[i] = rho;
        pr_out[i] = make_float2(p, inv_rho);
        if (kMode != kEmitNone) {
            const float4 v = vel[i];
            st8(pv + 2 * (size_t)i, make_float4(xi.x, xi.y, xi.z, p), make_float4(v.x, v.y, v.z, inv_rho));
        }
        if (kMode != kEmitNone) nbr_count[i] = cnt;
    }
    if (kMode == kEmitStaged) {
        // Copy each warp's recorded rows out in full 128-byte lines.
        const uint32_t kmax = __reduce_max_sync(0xffffffffu, min(cnt, (uint32_t)kNbCap));
        uint32_t* tile = nbr + (size_t)blockIdx.x * kNbCap * kNbTile + t;
        for (uint32_t k = 0; k < kmax; ++k) tile[(size_t)k * kNbTile] = s_nb[k][t];
    }
}

template <int kMode, int kBlockSize>
void density_as(const DeviceState& d, const SimConst& c, cudaStream_t s) {
    with_reach(c.reach, [&](auto R) {
        constexpr int K = decltype(R)::value;
        if (d.table) {
            if constexpr (K <= 2)
                launch_chained(k_density<kMode, kBlockSize, K, true>, grid_for(d.n, kBlockSize), kBlockSize, s,
                               d.pos, d.cell_start, d.n, c, d.table, d.scene_off, d.nscenes, d.rho, d.pr, d.nbr,
                               d.nbr_count, d.vel, d.pv, (FrameState*)nullptr);
        } else {
            launch_chained(k_density<kMode, kBlockSize, K, false>, grid_for(d.n, kBlockSize), kBlockSize, s, d.pos,
                           d.cell_start, d.n, c, nullptr, nullptr, 0u, d.rho, d.pr, d.nbr, d.nbr_count, d.vel, d.pv,
                           d.frame);
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
    } else {
        big ? density_as<kEmitTile, 256>(d, c, s) : density_as<kEmitTile, 128>(d, c, s);
    }
}

}  // namespace sf
