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
// next kPrefetch list indices are loaded while they are, so the dependent
// index -> data loads of consecutive batches overlap; the terms are still
// added in list order, which keeps the sum bit-identical.
#include "sf_device.cuh"

namespace sf {
namespace {

// Forces on particle i, then (kIntegrate) its step and the next sort's
// histogram entry, or (!kIntegrate) its acceleration.  With the adaptive
// sub-step, v2 and a2 receive |v'|^2 and |a|^2 as float bits.
template <bool kUseList, int kPrefetch, bool kIntegrate, int kReach, bool kBatched>
__device__ __forceinline__ void force_one(
    uint32_t i, const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ pr,
    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
    const float4* __restrict__ pv, uint32_t n, const SimConst& c0, const SimConst* __restrict__ table,
    const uint32_t* __restrict__ scene_off, uint32_t nscenes,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint32_t* __restrict__ counts,
    uint32_t* __restrict__ tile_sums, uint2* __restrict__ key_slot, float4* __restrict__ acc_out,
    float4* __restrict__ sums, const FrameState* __restrict__ frame, uint32_t& v2, uint32_t& a2) {
    static_assert(kPrefetch >= 2, "the list tail holds up to kPrefetch - 1 neighbours");
    // A batch reads its scene's constants where they are used (the kernel
    // radius before the neighbour loop, the rest after it) instead of
    // holding them in registers across the loop.
    const uint32_t scene = kBatched ? scene_of(scene_off, nscenes, i) : 0u;
    auto consts = [&]() -> SimConst {
        if constexpr (kBatched) return *opaque_ptr(table + scene);
        else return c0;
    };
    const float h = kBatched ? opaque_ptr(table + scene)->h : c0.h;
    const float4 xi = pos[i];
    const float4 vi = vel[i];
    const float2 pri = pr[i];
    PairAcc a;
    const uint32_t cnt = kUseList ? nbr_count[i] : 0xffffffffu;
    if (cnt <= (uint32_t)kNbCap) {
        const uint32_t* lst = nbr + nbr_index(i, 0);  // slot k at lst[k * kNbTile]
        uint32_t jn[kPrefetch];
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) jn[u] = __ldg(lst + (size_t)u * kNbTile);
        uint32_t k = 0;
        for (; k + kPrefetch <= cnt; k += kPrefetch) {
            uint32_t j[kPrefetch];
            float4 xj[kPrefetch], vj[kPrefetch];
#pragma unroll
            for (int u = 0; u < kPrefetch; ++u) {
                j[u] = jn[u];
                // the next batch's indices (slots past the count hold stale values, unused)
                jn[u] = __ldg(lst + (size_t)min(k + kPrefetch + u, (uint32_t)kNbCap - 1) * kNbTile);
            }
#pragma unroll
            for (int u = 0; u < kPrefetch; ++u) ld8(pv + 2 * (size_t)checked_index(j[u], n), xj[u], vj[u]);
#pragma unroll
            for (int u = 0; u < kPrefetch; ++u)
                pair_terms(h, xi, vi, pri.x, xj[u], make_float2(xj[u].w, vj[u].w), vj[u], a);
        }
        // the last cnt - k < kPrefetch neighbours: their indices are in jn
        float4 xj[kPrefetch - 1], vj[kPrefetch - 1];
#pragma unroll
        for (int u = 0; u < kPrefetch - 1; ++u)
            if (k + u < cnt) ld8(pv + 2 * (size_t)checked_index(jn[u], n), xj[u], vj[u]);
#pragma unroll
        for (int u = 0; u < kPrefetch - 1; ++u)
            if (k + u < cnt) pair_terms(h, xi, vi, pri.x, xj[u], make_float2(xj[u].w, vj[u].w), vj[u], a);
    } else {
        const SimConst cr = consts();
        for_candidates_rolled<kReach>(cr, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
            if (j == i) return;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < cr.h2)
                pair_terms(cr.h, xi, vi, pri.x, xj, __ldg(pr + j), ldg4(vel + j), a);
        });
    }
    const SimConst c = consts();
    if (sums) {
        sums[2 * (size_t)i] = make_float4(a.apx, a.apy, a.apz, 0.f);
        sums[2 * (size_t)i + 1] = make_float4(a.avx, a.avy, a.avz, 0.f);
    }
    const float ax = fmaf(fmaf(c.cp, a.apx, c.cv * a.avx), pri.y, c.g[0]);
    const float ay = fmaf(fmaf(c.cp, a.apy, c.cv * a.avy), pri.y, c.g[1]);
    const float az = fmaf(fmaf(c.cp, a.apz, c.cv * a.avz), pri.y, c.g[2]);
    if (!kIntegrate) {
        acc_out[i] = make_float4(ax, ay, az, 0.f);
        return;
    }
    const float dt = frame ? frame->dt : c.dt;
    float v[3] = {fmaf(dt, ax, vi.x), fmaf(dt, ay, vi.y), fmaf(dt, az, vi.z)};
    float x[3] = {fmaf(dt, v[0], xi.x), fmaf(dt, v[1], xi.y), fmaf(dt, v[2], xi.z)};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        if (x[q] < c.lo[q]) {
            x[q] = c.lo[q];
            if (v[q] < 0.f) v[q] = -c.e * v[q];
        }
        if (x[q] > c.hi[q]) {
            x[q] = c.hi[q];
            if (v[q] > 0.f) v[q] = -c.e * v[q];
        }
    }
    pos_out[i] = make_float4(x[0], x[1], x[2], xi.w);
    vel_out[i] = make_float4(v[0], v[1], v[2], 0.f);
    const uint32_t key = cell_key(c, x[0], x[1], x[2]);
    key_slot[i] = make_uint2(key, count_in_cell(key, counts, tile_sums));
    if (frame && c.adaptive) {
        v2 = __float_as_uint(fmaf(v[2], v[2], fmaf(v[1], v[1], v[0] * v[0])));
        a2 = __float_as_uint(fmaf(az, az, fmaf(ay, ay, ax * ax)));
    }
}

template <bool kUseList, int kPrefetch, int kBlockSize, bool kIntegrate, int kReach, bool kBatched>
__global__ void __launch_bounds__(kBlockSize)
    k_force(const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ pr,
            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
            const float4* __restrict__ pv, uint32_t n, SimConst c0, const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off,
            uint32_t nscenes, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
            uint32_t* __restrict__ counts, uint32_t* __restrict__ tile_sums, uint2* __restrict__ key_slot,
            float4* __restrict__ acc_out, float4* __restrict__ sums, FrameState* __restrict__ frame) {
    grid_dependency_wait();
    allow_dependents();
    const uint32_t i = blockIdx.x * kBlockSize + threadIdx.x;
    uint32_t v2 = 0u, a2 = 0u;
    if (i < n)
        force_one<kUseList, kPrefetch, kIntegrate, kReach, kBatched>(i, pos, vel, pr, cs, nbr, nbr_count, pv, n, c0, table,
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

template <bool kUseList, int kPrefetch, int kBlockSize, bool kIntegrate>
void force_as(DeviceState& d, const SimConst& c, cudaStream_t s) {
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
                launch_chained(k_force<kUseList, kPrefetch, kBlockSize, kIntegrate, K, true>, grid_for(d.n, kBlockSize),
                               kBlockSize, s, d.pos, d.vel, d.pr, d.cell_start, d.nbr, d.nbr_count, d.pv, d.n, c, d.table,
                               d.scene_off, d.nscenes, po, vo, co, ts, ks, ac, d.sums, (FrameState*)nullptr);
        } else {
            launch_chained(k_force<kUseList, kPrefetch, kBlockSize, kIntegrate, K, false>, grid_for(d.n, kBlockSize),
                           kBlockSize, s, d.pos, d.vel, d.pr, d.cell_start, d.nbr, d.nbr_count, d.pv, d.n, c,
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
        big ? force_as<false, 2, 256, kIntegrate>(d, c, s) : force_as<false, 2, 128, kIntegrate>(d, c, s);
    } else if (d.tune.prefetch == 2) {
        big ? force_as<true, 2, 256, kIntegrate>(d, c, s) : force_as<true, 2, 128, kIntegrate>(d, c, s);
    } else {
        big ? force_as<true, 4, 256, kIntegrate>(d, c, s) : force_as<true, 4, 128, kIntegrate>(d, c, s);
    }
}

}  // namespace

SF_INDEX_CHECK_ACCESSOR(index_check_failures_force)

void launch_force_integrate(DeviceState& d, const SimConst& c, cudaStream_t s) { launch_force<true>(d, c, s); }

void launch_force_only(DeviceState& d, const SimConst& c, cudaStream_t s) { launch_force<false>(d, c, s); }

}  // namespace sf
