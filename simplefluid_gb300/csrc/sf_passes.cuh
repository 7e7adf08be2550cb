// sf_passes.cuh — the per-particle density and force passes of the SPH
// sub-step, shared by the separately launched kernels (sf_density.cu,
// sf_force.cu) and the persistent batched step (sf_batch.cu).
//
// kNc selects the load path: through the read-only path for kernels in which
// no thread writes what they read (the separately launched passes), plain
// coherent loads for the persistent step (see ld_f4 in sf_device.cuh).
#pragma once
#include "sf_device.cuh"

namespace sf {

// Whether every candidate of a particle at (x, y, z) lies within kNear16
// sorted places of i: the candidate cells' keys lie between those of the
// grid-clamped corner cells (cx-R, cy-R, cz-R) and (cx+R, cy+R, cz+R), so
// the candidates lie in [cs[key_lo], cs[key_hi + 1]).
template <int kReach, bool kNc = true>
__device__ __forceinline__ bool candidates_near(const SimConst& c, const uint32_t* __restrict__ cs, uint32_t n,
                                                uint32_t i, float x, float y, float z) {
    const int cx = cell_coord(x, c.bmin[0], c.inv_cell[0], c.n[0]);
    const int cy = cell_coord(y, c.bmin[1], c.inv_cell[1], c.n[1]);
    const int cz = cell_coord(z, c.bmin[2], c.inv_cell[2], c.n[2]);
    const uint32_t n0 = (uint32_t)c.n[0], n1 = (uint32_t)c.n[1];
    const uint32_t klo = c.cell_base + ((uint32_t)max(cz - kReach, 0) * n1 + (uint32_t)max(cy - kReach, 0)) * n0 +
                         (uint32_t)max(cx - kReach, 0);
    const uint32_t khi = c.cell_base +
                         ((uint32_t)min(cz + kReach, c.n[2] - 1) * n1 + (uint32_t)min(cy + kReach, c.n[1] - 1)) * n0 +
                         (uint32_t)min(cx + kReach, c.n[0] - 1);
    const uint32_t lo = checked_end(ld_u32<kNc>(cs + klo), n), hi = checked_end(ld_u32<kNc>(cs + khi + 1), n);
    return lo + kNear16 >= i && hi <= i + kNear16 + 1;
}

// The density pass of particle i at xi (see sf_density.cu): the candidate
// walk with the poly6 sum and the list emission of kMode, the equation of
// state, and the outputs rho, (p, 1/rho), the gather record and the list
// count.  `wide` selects 32-bit entries in a kEmitTile16 warp tile;
// kEmitStaged writes slot k to stage[k * stage_stride].  Returns the
// neighbour count.
template <int kMode, int kReach, bool kNc = true>
__device__ __forceinline__ uint32_t density_one(uint32_t i, const SimConst& c, const float4& xi,
                                                const float4* __restrict__ pos, const uint32_t* __restrict__ cs,
                                                uint32_t n, float* __restrict__ rho_out, float2* __restrict__ pr_out,
                                                uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count,
                                                const float4* __restrict__ vel, float4* __restrict__ pv, bool wide,
                                                uint32_t* stage, uint32_t stage_stride) {
    uint32_t cnt = 0;
    float s = 0.f;
    // The walk with the list entries stored by `emit(slot, j, near)`.
    auto walk = [&](auto emit) {
        for_candidates<kReach, kNc>(c, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const bool near = r2 < c.h2;
            const float q = near ? c.h2 - r2 : 0.f;
            s = fmaf(q * q, q, s);
            // Predicated store, no branch.  Past the cap the last slot is
            // overwritten: such a list is never read (the force pass
            // rescans particles whose count exceeds the cap).
            emit(min(cnt, (uint32_t)kNbCap - 1), j, near);
            cnt += near ? 1u : 0u;
        });
    };
    if constexpr (kMode == kEmitTile) {
        uint32_t* const lst = nbr + nbr_index(i, 0);  // slot k at lst[k * kNbTile]
        walk([&](uint32_t k, uint32_t j, bool near) { store_if(lst + (size_t)k * kNbTile, j, near); });
    } else if constexpr (kMode == kEmitTile16) {
        if (wide) {
            uint32_t* const w32 = nbr + nbr_w32_index(i, 0);
            walk([&](uint32_t k, uint32_t j, bool near) { store_if(w32 + (size_t)k * kNbWarpTile, j, near); });
        } else {
            uint16_t* const w16 = reinterpret_cast<uint16_t*>(nbr) + nbr_w16_index(i, 0);
            walk([&](uint32_t k, uint32_t j, bool near) { store16_if(w16 + (size_t)k * kNbWarpTile, j, near); });
        }
    } else if constexpr (kMode == kEmitStaged) {
        walk([&](uint32_t, uint32_t j, bool near) {
            if (near && cnt < kNbCap) stage[(size_t)cnt * stage_stride] = j;
        });
    } else {
        walk([](uint32_t, uint32_t, bool) {});
    }
    const float rho = c.cd * s;
    const float p = pressure_of(c, rho), inv_rho = 1.f / rho;
    rho_out[i] = rho;
    pr_out[i] = make_float2(p, inv_rho);
    if (kMode != kEmitNone) {
        const float4 v = ld_f4<kNc>(vel + i);
        st8(pv + 2 * (size_t)i, make_float4(xi.x, xi.y, xi.z, p), make_float4(v.x, v.y, v.z, inv_rho));
        nbr_count[i] = cnt;
    }
    return cnt;
}

// Pair terms of particle i over its neighbour list, in list order.  Slot k
// of the list is the raw entry load(k); decode(entry) is the neighbour's
// index.  Batches of kPrefetch neighbours are gathered before their terms are
// added, while the next batch's entries are loaded; entries are decoded where
// they are used, so their loads stay in flight.
template <int kPrefetch, bool kNc, typename Load, typename Decode>
__device__ __forceinline__ void gather_list(uint32_t cnt, Load load, Decode decode, const float4* __restrict__ pv,
                                            uint32_t n, float h, const float4& xi, const float4& vi, float pi,
                                            PairAcc& a) {
    static_assert(kPrefetch >= 2, "the list tail holds up to kPrefetch - 1 neighbours");
    uint32_t en[kPrefetch];
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) en[u] = load((uint32_t)u);
    uint32_t k = 0;
    for (; k + kPrefetch <= cnt; k += kPrefetch) {
        uint32_t j[kPrefetch];
        float4 xj[kPrefetch], vj[kPrefetch];
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
            j[u] = decode(en[u]);
            // the next batch's entries (slots past the count hold stale values, unused)
            en[u] = load(min(k + kPrefetch + u, (uint32_t)kNbCap - 1));
        }
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) ld8<kNc>(pv + 2 * (size_t)checked_index(j[u], n), xj[u], vj[u]);
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) pair_terms(h, xi, vi, pi, xj[u], make_float2(xj[u].w, vj[u].w), vj[u], a);
    }
    // the last cnt - k < kPrefetch neighbours: their entries are in en
    float4 xj[kPrefetch - 1], vj[kPrefetch - 1];
#pragma unroll
    for (int u = 0; u < kPrefetch - 1; ++u)
        if (k + u < cnt) ld8<kNc>(pv + 2 * (size_t)checked_index(decode(en[u]), n), xj[u], vj[u]);
#pragma unroll
    for (int u = 0; u < kPrefetch - 1; ++u)
        if (k + u < cnt) pair_terms(h, xi, vi, pi, xj[u], make_float2(xj[u].w, vj[u].w), vj[u], a);
}

// Forces on particle i, then (kIntegrate) its step and the next sort's
// histogram entry, or (!kIntegrate) its acceleration.  With the adaptive
// sub-step, v2 and a2 receive |v'|^2 and |a|^2 as float bits.
// kList: 0 no list (rescan), 1 32-bit entries, 2 16-bit entries (32-bit in
// warp tiles marked in nbr_wide).  tile_sums may be null (no scan-tile
// totals).
template <int kList, int kPrefetch, bool kIntegrate, int kReach, bool kBatched, bool kNc = true>
__device__ __forceinline__ void force_one(
    uint32_t i, const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ pr,
    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
    const uint8_t* __restrict__ nbr_wide, const float4* __restrict__ pv, uint32_t n, const SimConst& c0,
    const SimConst* __restrict__ table, const uint32_t* __restrict__ scene_off, uint32_t nscenes,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint32_t* __restrict__ counts,
    uint32_t* __restrict__ tile_sums, uint2* __restrict__ key_slot, float4* __restrict__ acc_out,
    float4* __restrict__ sums, const FrameState* __restrict__ frame, uint32_t& v2, uint32_t& a2) {
    // A batch reads its scene's constants where they are used (the kernel
    // radius before the neighbour loop, the rest after it) instead of
    // holding them in registers across the loop.
    const uint32_t scene = kBatched ? scene_of(scene_off, nscenes, i) : 0u;
    auto consts = [&]() -> SimConst {
        if constexpr (kBatched) return *opaque_ptr(table + scene);
        else return c0;
    };
    const float h = kBatched ? opaque_ptr(table + scene)->h : c0.h;
    const float4 xi = ld_f4<kNc>(pos + i);
    const float4 vi = ld_f4<kNc>(vel + i);
    const float2 pri = ld_f2<kNc>(pr + i);
    PairAcc a;
    const uint32_t cnt = kList ? ld_u32<kNc>(nbr_count + i) : 0xffffffffu;
    if (cnt <= (uint32_t)kNbCap) {
        auto same = [](uint32_t e) { return e; };
        if constexpr (kList == 2) {
            // warp tiles of 16-bit entries, or of 32-bit entries where marked
            if (!nbr_wide[i / kNbWarpTile]) {
                const uint16_t* w16 = reinterpret_cast<const uint16_t*>(nbr) + nbr_w16_index(i, 0);
                gather_list<kPrefetch, kNc>(
                    cnt, [&](uint32_t k) { return ld16(w16 + (size_t)k * kNbWarpTile); },
                    [&](uint32_t e) { return near_index(i, e); }, pv, n, h, xi, vi, pri.x, a);
            } else {
                const uint32_t* w32 = nbr + nbr_w32_index(i, 0);
                gather_list<kPrefetch, kNc>(
                    cnt, [&](uint32_t k) { return ld_u32<kNc>(w32 + (size_t)k * kNbWarpTile); }, same, pv, n, h, xi,
                    vi, pri.x, a);
            }
        } else {
            const uint32_t* lst = nbr + nbr_index(i, 0);  // slot k at lst[k * kNbTile]
            gather_list<kPrefetch, kNc>(
                cnt, [&](uint32_t k) { return ld_u32<kNc>(lst + (size_t)k * kNbTile); }, same, pv, n, h, xi, vi,
                pri.x, a);
        }
    } else {
        const SimConst cr = consts();
        for_candidates_rolled<kReach, kNc>(cr, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
            if (j == i) return;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < cr.h2)
                pair_terms(cr.h, xi, vi, pri.x, xj, ld_f2<kNc>(pr + j), ld_f4<kNc>(vel + j), a);
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

}  // namespace sf
