// sf_adjoint.cu — hand-written adjoint of the SPH sub-step and of the CIC
// histogram loss (sm_103a).
//
// The neighbour structure of each step is held fixed (piecewise constant):
// the backward pass re-runs each segment forward from a checkpoint, recording
// per step the sorted state, density/pressure, the neighbour lists and the
// force sums (AP, AV), then walks the steps in reverse.  One step's adjoint is
// three gather passes over the recorded neighbours, so every accumulation is
// per particle, deterministic and free of atomics on particle data:
//   P1  integration (symplectic Euler, box clamp with restitution) and the
//       acceleration's own inputs: a = (cp AP + cv AV) inv + g;
//   P2  force pair terms in both orientations of every pair (spiky pressure,
//       symmetrised weights, viscosity), then rho_bar from 1/rho and the EOS;
//   P4  poly6 density terms onto positions; adjoints written back by particle.
// Adjoint vectors between steps live in caller-index space (index = original
// particle id), so the per-step re-sort needs no explicit adjoint permutation.
// Scalar gradients (viscosity, stiffness) are reduced per block in double,
// then summed in block order by one block: bit-reproducible.
//
// The CPU oracle (oracle/sph_oracle.cpp, adjoint_step) performs the same
// operations in the same order.
#include "sf_device.cuh"

namespace sf {
namespace {

constexpr int kAdjBlock = 128;

// Calls f(j, pos[j]) for the neighbours j != i (|xi - xj| < h) of sorted
// particle i, in canonical order: from the recorded list, or by walking the
// candidate cells when the list overflowed.
template <int kReach, typename F>
__device__ __forceinline__ void for_neighbours(const SimConst& c, uint32_t i, const float4& xi,
                                               const float4* __restrict__ pos, uint32_t n,
                                               const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr,
                                               const uint32_t* __restrict__ cnt, F&& f) {
    const uint32_t m = __ldg(cnt + i);
    if (m <= (uint32_t)kNbCap) {
        const uint32_t* lst = nbr + nbr_index(i, 0);  // slot k at lst[k * kNbTile]
        uint32_t jn = __ldg(lst);
        for (uint32_t k = 0; k < m; ++k) {
            const uint32_t j = checked_index(jn, n);
            // the next index is in flight while this neighbour is processed
            // (slots past the count hold stale values, never used)
            jn = __ldg(lst + (size_t)min(k + 1, (uint32_t)kNbCap - 1) * kNbTile);
            if (j != i) f(j, ldg4(pos + j));  // the list records the particle itself
        }
    } else {
        for_candidates<kReach>(c, cs, pos, n, xi.x, xi.y, xi.z, [&](uint32_t j, const float4& xj) {
            if (j == i) return;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < c.h2) f(j, xj);
        });
    }
}

__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return fmaf(az, bz, fmaf(ay, by, ax * bx));
}

// P1: per sorted particle.  Outputs the 32-byte record abrec = apb (cp tb,
// inv_bar), avb (cv tb, cv_bar), and xdir/vdir = the integration's direct
// adjoints.
__global__ void __launch_bounds__(kAdjBlock)
    k_adj_integrate(const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ pr,
                    const float4* __restrict__ sums, uint32_t n, SimConst c, const float4* __restrict__ Xb,
                    const float4* __restrict__ Vb, float4* __restrict__ abrec, float4* __restrict__ xdir,
                    float4* __restrict__ vdir) {
    const uint32_t i = blockIdx.x * kAdjBlock + threadIdx.x;
    if (i >= n) return;
    const float4 x4 = pos[i], v4 = vel[i];
    const uint32_t id = __float_as_uint(x4.w);
    const float inv = pr[i].y;
    const float4 AP = sums[2 * (size_t)i], AV = sums[2 * (size_t)i + 1];
    const float4 xb4 = Xb[id], vb4 = Vb[id];
    const float xs[3] = {x4.x, x4.y, x4.z}, vs[3] = {v4.x, v4.y, v4.z};
    const float aps[3] = {AP.x, AP.y, AP.z}, avs[3] = {AV.x, AV.y, AV.z};
    const float xbs[3] = {xb4.x, xb4.y, xb4.z}, vbs[3] = {vb4.x, vb4.y, vb4.z};
    float t[3], tb[3], ab[3], xd[3], vd[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        t[a] = fmaf(c.cp, aps[a], c.cv * avs[a]);
        const float acc = fmaf(t[a], inv, c.g[a]);
        const float vpre = fmaf(c.dt, acc, vs[a]);
        const float xpre = fmaf(c.dt, vpre, xs[a]);
        const bool lo = xpre < c.lo[a], hi = xpre > c.hi[a];
        const bool pass = !lo && !hi;
        const float sv = ((lo && vpre < 0.f) || (hi && vpre > 0.f)) ? -c.e : 1.f;
        const float xbpre = pass ? xbs[a] : 0.f;
        const float vbpre = fmaf(sv, vbs[a], c.dt * xbpre);
        xd[a] = xbpre;
        vd[a] = vbpre;
        ab[a] = c.dt * vbpre;
        tb[a] = ab[a] * inv;
    }
    const float invb = dot3f(ab[0], ab[1], ab[2], t[0], t[1], t[2]);
    const float cvb = dot3f(tb[0], tb[1], tb[2], avs[0], avs[1], avs[2]);
    st8(abrec + 2 * (size_t)i, make_float4(c.cp * tb[0], c.cp * tb[1], c.cp * tb[2], invb),
        make_float4(c.cv * tb[0], c.cv * tb[1], c.cv * tb[2], cvb));
    xdir[i] = make_float4(xd[0], xd[1], xd[2], 0.f);
    vdir[i] = make_float4(vd[0], vd[1], vd[2], 0.f);
}

// dp/drho and dp/dk of the equation of state (0 where the clamp is active).
__device__ __forceinline__ void eos_derivs(const SimConst& c, float rho, float& dpdrho, float& dpdk) {
    float ppre, dr, dk;
    if (c.eos == SF_EOS_TAIT) {
        const float x = rho * c.inv_rho0;
        const float x2 = x * x;
        const float x4 = x2 * x2;
        const float x6 = x4 * x2;
        const float x7 = x6 * x;
        ppre = c.k * (x7 - 1.f);
        dr = (7.f * c.k) * (x6 * c.inv_rho0);
        dk = x7 - 1.f;
    } else {
        ppre = c.k * (rho - c.rho0);
        dr = c.k;
        dk = rho - c.rho0;
    }
    const bool act = c.attractive || ppre > 0.f;
    dpdrho = act ? dr : 0.f;
    dpdk = act ? dk : 0.f;
}

// P2: force pair terms of every pair in both orientations, then the density
// adjoint of the particle.  Outputs xrb = (x, y, z, rho_bar), P4's gather
// record, xf = (force x_bar, k_bar) and vf.
// A neighbour is two 32-byte records, each one 256-bit load: the step's
// (x, y, z, p | vx, vy, vz, 1/rho) and P1's (apb | avb).
template <int kReach>
__global__ void __launch_bounds__(kAdjBlock)
    k_adj_forces(const float4* __restrict__ pos, const float4* __restrict__ pv, const float2* __restrict__ pr,
                 const float* __restrict__ rho, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr,
                 const uint32_t* __restrict__ cnt, uint32_t n, SimConst c, const float4* __restrict__ ab,
                 float4* __restrict__ xrb, float4* __restrict__ xf, float4* __restrict__ vf) {
    const uint32_t k = blockIdx.x * kAdjBlock + threadIdx.x;
    if (k >= n) return;
    float4 xk, vk, apbk, avbk;
    ld8(pv + 2 * (size_t)k, xk, vk);
    ld8(ab + 2 * (size_t)k, apbk, avbk);
    const float2 prk = pr[k];
    const float pk = prk.x, invk = prk.y;
    float pb = 0.f, invacc = 0.f;
    float xb0 = 0.f, xb1 = 0.f, xb2 = 0.f, vb0 = 0.f, vb1 = 0.f, vb2 = 0.f;
    auto pair = [&](const float4& xj, const float4& vj, const float4& apbj, const float4& avbj) {
        const float d0 = xk.x - xj.x, d1 = xk.y - xj.y, d2 = xk.z - xj.z;
        const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
        const float r = sqrtf(r2);
        const float hr = c.h - r;
        const float pj = xj.w, invj = vj.w;
        const float dv0 = vj.x - vk.x, dv1 = vj.y - vk.y, dv2 = vj.z - vk.z;
        const float ps = pk + pj;
        // orientation A: k is i, j the neighbour
        const float wkj = hr * invj;
        vb0 = fmaf(-wkj, avbk.x, vb0);
        vb1 = fmaf(-wkj, avbk.y, vb1);
        vb2 = fmaf(-wkj, avbk.z, vb2);
        float wb = dot3f(avbk.x, avbk.y, avbk.z, dv0, dv1, dv2);
        float rb = 0.f;
        // orientation B: j is i, k the neighbour
        const float wjk = hr * invk;
        vb0 = fmaf(wjk, avbj.x, vb0);
        vb1 = fmaf(wjk, avbj.y, vb1);
        vb2 = fmaf(wjk, avbj.z, vb2);
        float wb2 = -dot3f(avbj.x, avbj.y, avbj.z, dv0, dv1, dv2);
        float rb2 = 0.f;
        if (r > 0.f) {
            const float q = hr / r;
            const float S = (ps * wkj) * q;
            const float Sb = dot3f(apbk.x, apbk.y, apbk.z, d0, d1, d2);
            xb0 = fmaf(S, apbk.x, xb0);
            xb1 = fmaf(S, apbk.y, xb1);
            xb2 = fmaf(S, apbk.z, xb2);
            pb = fmaf(Sb, wkj * q, pb);
            wb = fmaf(Sb, ps * q, wb);
            const float qb = Sb * (ps * wkj);
            rb = -((qb * c.h) / r2);
            const float S2 = (ps * wjk) * q;
            const float Sb2 = -dot3f(apbj.x, apbj.y, apbj.z, d0, d1, d2);
            xb0 = fmaf(-S2, apbj.x, xb0);
            xb1 = fmaf(-S2, apbj.y, xb1);
            xb2 = fmaf(-S2, apbj.z, xb2);
            pb = fmaf(Sb2, wjk * q, pb);
            wb2 = fmaf(Sb2, ps * q, wb2);
            const float qb2 = Sb2 * (ps * wjk);
            rb2 = -((qb2 * c.h) / r2);
        }
        rb = fmaf(-wb, invj, rb);
        invacc = fmaf(wb2, hr, invacc);
        rb2 = fmaf(-wb2, invk, rb2);
        if (r > 0.f) {
            const float g = (rb + rb2) / r;
            xb0 = fmaf(g, d0, xb0);
            xb1 = fmaf(g, d1, xb1);
            xb2 = fmaf(g, d2, xb2);
        }
    };
    const uint32_t m = __ldg(cnt + k);
    if (m <= (uint32_t)kNbCap) {
        // The next neighbour's records and the index after it are in flight
        // while a neighbour is processed.  The list holds the particle itself
        // (skipped); slots past the count hold stale values, never used.
        const uint32_t* lst = nbr + nbr_index(k, 0);  // slot s at lst[s * kNbTile]
        uint32_t jc = checked_index(__ldg(lst), n), jn = __ldg(lst + kNbTile);
        float4 nx, nv, na, nb;
        if (m) {
            ld8(pv + 2 * (size_t)jc, nx, nv);
            ld8(ab + 2 * (size_t)jc, na, nb);
        }
        for (uint32_t s = 0; s < m; ++s) {
            const uint32_t j = jc;
            const float4 xj = nx, vj = nv, apbj = na, avbj = nb;
            if (s + 1 < m) {
                jc = checked_index(jn, n);
                jn = __ldg(lst + (size_t)min(s + 2, (uint32_t)kNbCap - 1) * kNbTile);
                ld8(pv + 2 * (size_t)jc, nx, nv);
                ld8(ab + 2 * (size_t)jc, na, nb);
            }
            if (j != k) pair(xj, vj, apbj, avbj);
        }
    } else {
        for_candidates<kReach>(c, cs, pos, n, xk.x, xk.y, xk.z, [&](uint32_t j, const float4& xp) {
            if (j == k) return;
            const float dx = xk.x - xp.x, dy = xk.y - xp.y, dz = xk.z - xp.z;
            if (!(fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < c.h2)) return;
            float4 xj, vj, apbj, avbj;
            ld8(pv + 2 * (size_t)j, xj, vj);
            ld8(ab + 2 * (size_t)j, apbj, avbj);
            pair(xj, vj, apbj, avbj);
        });
    }
    const float ib = apbk.w + invacc;
    float dpdrho, dpdk;
    eos_derivs(c, rho[k], dpdrho, dpdk);
    xrb[k] = make_float4(xk.x, xk.y, xk.z, fmaf(pb, dpdrho, -((ib * invk) * invk)));
    xf[k] = make_float4(xb0, xb1, xb2, pb * dpdk);
    vf[k] = make_float4(vb0, vb1, vb2, 0.f);
}

// P4: poly6 density terms onto positions; the step's input adjoints are
// written back by particle id.
// Also reduces the step's scalar adjoints (cv_bar in avb.w of the ab record, k_bar in xf.w) per
// block, in thread order, into partial[blockIdx.x].
template <int kReach>
__global__ void __launch_bounds__(kAdjBlock)
    k_adj_density(const float4* __restrict__ pos, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ nbr,
                  const uint32_t* __restrict__ cnt, uint32_t n, SimConst c, float m6cd, const float4* __restrict__ xrb,
                  const float4* __restrict__ xdir, const float4* __restrict__ vdir, const float4* __restrict__ xf,
                  const float4* __restrict__ vf, const float4* __restrict__ ab, float4* __restrict__ Xb,
                  float4* __restrict__ Vb, double2* __restrict__ partial) {
    __shared__ double s0[kAdjBlock], s1[kAdjBlock];
    const uint32_t k = blockIdx.x * kAdjBlock + threadIdx.x;
    s0[threadIdx.x] = k < n ? (double)ab[2 * (size_t)k + 1].w : 0.0;
    s1[threadIdx.x] = k < n ? (double)xf[k].w : 0.0;
    __syncthreads();
    for (int o = kAdjBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(s0[0], s1[0]);
    if (k >= n) return;
    const float4 xk = pos[k];
    const float rbk = xrb[k].w;
    float x0 = 0.f, x1 = 0.f, x2 = 0.f;
    for_neighbours<kReach>(c, k, xk, pos, n, cs, nbr, cnt, [&](uint32_t j, const float4&) {
        const float4 xj = ldg4(xrb + j);  // position and rho_bar in one load
        const float d0 = xk.x - xj.x, d1 = xk.y - xj.y, d2 = xk.z - xj.z;
        const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
        const float q = c.h2 - r2;
        const float sc = (rbk + xj.w) * (q * q);
        x0 = fmaf(sc, d0, x0);
        x1 = fmaf(sc, d1, x1);
        x2 = fmaf(sc, d2, x2);
    });
    const uint32_t id = __float_as_uint(xk.w);
    const float4 xd = xdir[k], xfk = xf[k], vd = vdir[k], vfk = vf[k];
    Xb[id] = make_float4(fmaf(m6cd, x0, xd.x + xfk.x), fmaf(m6cd, x1, xd.y + xfk.y), fmaf(m6cd, x2, xd.z + xfk.z), 0.f);
    Vb[id] = make_float4(vd.x + vfk.x, vd.y + vfk.y, vd.z + vfk.z, 0.f);
}

// Adds the block partials of `nsteps` steps to acc[0..1].  Eight steps at a
// time, one warp per step: lane l sums blocks l, l + 32, ... in order and a
// fixed shuffle tree combines the lanes; thread 0 then adds the step sums
// last step first (the order the adjoint visits them).  Deterministic.
constexpr int kAccThreads = 256;

__global__ void __launch_bounds__(kAccThreads)
    k_accumulate_scalars(const double2* __restrict__ partial, uint32_t nsteps, uint32_t nblocks,
                         double* __restrict__ acc) {
    constexpr int kWarps = kAccThreads / 32;
    __shared__ double s0[kWarps], s1[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double a = 0.0, b = 0.0;
    if (threadIdx.x == 0) {
        a = acc[0];
        b = acc[1];
    }
    for (int64_t hi = (int64_t)nsteps; hi > 0; hi -= kWarps) {
        const int64_t st = hi - 1 - warp;  // the same in every lane of the warp
        double x = 0.0, y = 0.0;
        if (st >= 0) {
            for (uint32_t t = lane; t < nblocks; t += 32) {
                const double2 v = partial[(size_t)st * nblocks + t];
                x += v.x;
                y += v.y;
            }
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_down_sync(0xffffffffu, x, o);
                y += __shfl_down_sync(0xffffffffu, y, o);
            }
        }
        if (lane == 0) {
            s0[warp] = x;
            s1[warp] = y;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 0; w < kWarps && hi - 1 - w >= 0; ++w) {  // steps hi-1, hi-2, ...
                a += s0[w];
                b += s1[w];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        acc[0] = a;
        acc[1] = b;
    }
}

constexpr int kRedBlock = 256;

// ------------------------------------------------------------------ loss
// CIC (cloud-in-cell) histogram on res^3 cell-centred bins over the box,
// normalised by the particle count.  Deposits are 2^-32 fixed point in 64-bit
// integer atomics, so the histogram does not depend on the order of arrival.
__device__ __forceinline__ void cic(const SimConst& c, const float ext_inv[3], float x, float y, float z, int i0[3],
                                    float w0[3], float w1[3]) {
    const float p3[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float u = (p3[a] - c.bmin[a]) * ext_inv[a] - 0.5f;
        const float fl = floorf(u);
        const float f = u - fl;
        i0[a] = (int)fl;
        w0[a] = 1.f - f;
        w1[a] = f;
    }
}

struct HistDims {
    float inv[3];  // res / extent per axis
    int res;
};

__global__ void k_hist_deposit(const float4* __restrict__ pos, uint32_t n, SimConst c, HistDims hd,
                               unsigned long long* __restrict__ hist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos[i];
    int i0[3];
    float w0[3], w1[3];
    cic(c, hd.inv, x.x, x.y, x.z, i0, w0, w1);
    const int R = hd.res;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ix = i0[0] + (q & 1), iy = i0[1] + ((q >> 1) & 1), iz = i0[2] + ((q >> 2) & 1);
        if (ix < 0 || iy < 0 || iz < 0 || ix >= R || iy >= R || iz >= R) continue;
        const float w = ((q & 1) ? w1[0] : w0[0]) * ((q & 2) ? w1[1] : w0[1]) * ((q & 4) ? w1[2] : w0[2]);
        if (!(w > 0.f)) continue;
        atomicAdd(hist + ((size_t)iz * R + iy) * R + ix, (unsigned long long)llrint((double)w * 4294967296.0));
    }
}

// e[c] = 2 (H_c - T_c) / n and per-block partial sums of (H_c - T_c)^2.
__global__ void __launch_bounds__(kRedBlock)
    k_hist_error(const unsigned long long* __restrict__ hist, const float* __restrict__ target, uint32_t ncells,
                 uint32_t n, float* __restrict__ e2, double* __restrict__ partial) {
    __shared__ double s[kRedBlock];
    const uint32_t cidx = blockIdx.x * kRedBlock + threadIdx.x;
    double sq = 0.0;
    if (cidx < ncells) {
        const double H = (double)hist[cidx] * (1.0 / 4294967296.0) / (double)n;
        const double e = H - (double)target[cidx];
        e2[cidx] = (float)(2.0 * e / (double)n);
        sq = e * e;
    }
    s[threadIdx.x] = sq;
    __syncthreads();
    for (int o = kRedBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// dL/dx of each particle, written by particle id.
__global__ void k_hist_grad(const float4* __restrict__ pos, uint32_t n, SimConst c, HistDims hd,
                            const float* __restrict__ e2, float4* __restrict__ Xb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos[i];
    int i0[3];
    float w0[3], w1[3];
    cic(c, hd.inv, x.x, x.y, x.z, i0, w0, w1);
    const int R = hd.res;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ix = i0[0] + (q & 1), iy = i0[1] + ((q >> 1) & 1), iz = i0[2] + ((q >> 2) & 1);
        if (ix < 0 || iy < 0 || iz < 0 || ix >= R || iy >= R || iz >= R) continue;
        const float e = e2[((size_t)iz * R + iy) * R + ix];
        const float wx = (q & 1) ? w1[0] : w0[0], wy = (q & 2) ? w1[1] : w0[1], wz = (q & 4) ? w1[2] : w0[2];
        const float sx = (q & 1) ? hd.inv[0] : -hd.inv[0], sy = (q & 2) ? hd.inv[1] : -hd.inv[1],
                    sz = (q & 4) ? hd.inv[2] : -hd.inv[2];
        g0 += e * (sx * (wy * wz));
        g1 += e * (sy * (wx * wz));
        g2 += e * (sz * (wx * wy));
    }
    Xb[__float_as_uint(x.w)] = make_float4(g0, g1, g2, 0.f);
}

}  // namespace

SF_INDEX_CHECK_ACCESSOR(index_check_failures_adjoint)

// ------------------------------------------------------------------ launchers
const char* const kAdjointPassNames[kAdjointPasses] = {"adj_integrate", "adj_forces", "adj_density"};

void launch_adjoint_pass(uint32_t pass, const AdjointStep& st, const SimConst& c, AdjointWork& w, double2* partial,
                         cudaStream_t s) {
    const uint32_t n = st.n;
    if (!n) return;
    const unsigned g = grid_for(n, kAdjBlock);
    if (pass == 0) {
        k_adj_integrate<<<g, kAdjBlock, 0, s>>>(st.pos, st.vel, st.pr, st.sums, n, c, w.Xb, w.Vb, w.ab, w.xdir,
                                                w.vdir);
        return;
    }
    const float m6cd = (float)(-6.0 * (double)c.cd);
    with_reach(c.reach, [&](auto R) {
        constexpr int K = decltype(R)::value;
        if (pass == 1)
            k_adj_forces<K><<<g, kAdjBlock, 0, s>>>(st.pos, st.pv, st.pr, st.rho, st.cs, st.nbr, st.cnt, n, c, w.ab,
                                                    w.xrb, w.xf, w.vf);
        else if (pass == 2)
            k_adj_density<K><<<g, kAdjBlock, 0, s>>>(st.pos, st.cs, st.nbr, st.cnt, n, c, m6cd, w.xrb, w.xdir, w.vdir,
                                                     w.xf, w.vf, w.ab, w.Xb, w.Vb, partial);
    });
}

void launch_adjoint_step(const AdjointStep& st, const SimConst& c, AdjointWork& w, double2* partial,
                         cudaStream_t s) {
    for (uint32_t p = 0; p < kAdjointPasses; ++p) launch_adjoint_pass(p, st, c, w, partial, s);
}

uint32_t adjoint_partial_count(uint32_t n) { return grid_for(n, kAdjBlock); }

void launch_adjoint_accumulate(const double2* partial, uint32_t nsteps, uint32_t n, double* scalars, cudaStream_t s) {
    k_accumulate_scalars<<<1, kAccThreads, 0, s>>>(partial, nsteps, adjoint_partial_count(n), scalars);
}

void launch_histogram_loss(const float4* pos, uint32_t n, const SimConst& c, const float box_ext[3], uint32_t res,
                           const float* target, unsigned long long* hist, float* e2, double* partial, float4* Xb,
                           cudaStream_t s) {
    HistDims hd;
    hd.res = (int)res;
    for (int a = 0; a < 3; ++a) hd.inv[a] = (float)((double)res / (double)box_ext[a]);
    const uint32_t ncells = res * res * res;
    cudaMemsetAsync(hist, 0, (size_t)ncells * sizeof(unsigned long long), s);
    if (n) k_hist_deposit<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, hd, hist);
    k_hist_error<<<grid_for(ncells, kRedBlock), kRedBlock, 0, s>>>(hist, target, ncells, n ? n : 1, e2, partial);
    if (n && Xb) k_hist_grad<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, c, hd, e2, Xb);
}

uint32_t histogram_partial_count(uint32_t res) { return grid_for(res * res * res, kRedBlock); }

}  // namespace sf
