// sph_oracle.cpp — CPU restatement of the SimpleFluid SPH step.  TEST
// INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU-baseline
// leg of the benchmark call it as the checker.  The product never links it.
//
// What it restates, and from where:
//  * Scene generators: Source/SceneManager.cpp:21-173 of the reference, line by
//    line (lattice origin, spacing 2r, int-truncated counts, i->j->k loop
//    order, the sphere test of :83, the second dambreak block counting down
//    from bMax at :165, zero velocity).  Pinned against the reference's own
//    SceneManager.cpp compiled under oracle/_ref (see build_ref.sh).
//  * Frame semantics: Source/Simulator.cpp:44-56 (advanceFrame returns the
//    sub-step dt, the caller accumulates frames).
//  * The solver itself (SPHSolver<float>::advanceFrame, called at
//    Source/Simulator.cpp:49) lives in the author's external "Banana" library,
//    which is not vendored, pinned or present.  Its arithmetic is restated from
//    the published method it names: Mueller, Charypar & Gross, "Particle-Based
//    Fluid Simulation for Interactive Applications", SCA 2003 — poly6 density,
//    p = k(rho - rho0) (or Tait), spiky-gradient pressure force with the
//    symmetrised (p_i + p_j)/(2 rho_j) weight, viscosity-Laplacian force,
//    gravity, symplectic Euler and a restitution box.  Parity with Banana's own
//    numbers is therefore UNPINNED; the restatement is cross-checked by kernel
//    normalisation, rest density of a lattice, pairwise momentum conservation
//    and an FP32/FP64 band (tests/test_oracle.py).
//
// Canonical semantics shared with the CUDA path (both sides implement them
// independently; every choice is fixed here):
//  * uniform grid over [box_min, box_max] with K = cells_per_h (0 -> 2) and
//    n_a = max(1, floor(K * ext_a / h)) cells per axis (cell edge >= h/K);
//    cell coord = floor((x - box_min) * inv_cell) clamped to [0, n_a - 1]
//    (NaN -> 0); key = (cz*ny + cy)*nx + cx.
//  * stable sort of the current particle order by key (counting sort).
//  * neighbours of sorted particle i are visited in the order dz = -K..K,
//    dy = -K..K, then the contiguous sorted range of cells cx-K..cx+K
//    (clamped to the grid).  A faster implementation may skip cells that
//    provably hold no particle within h; that changes no sum.
//  * explicit fused multiply-adds where written (std::fma), no other
//    contraction (built with -ffp-contract=off), IEEE sqrt and division.
//  * derived constants computed in double, then rounded to the working type.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sf_capi.h"

namespace {

template <typename Real>
struct Derived {
    Real h, h2, mass, cd, cp, cv, k, rho0, inv_rho0, dt, e, r;
    Real g[3], lo[3], hi[3], bmin[3], inv_cell[3];
    int n[3];
    int eos, attractive, reach, adaptive;
    uint64_t ncells;
};

template <typename Real>
int derive(const sf_params* p, Derived<Real>* d) {
    if (!p) return SF_ERR_INVALID_ARGUMENT;
    const double h = p->kernel_radius, r = p->particle_radius;
    if (!(h > 0) || !(r > 0) || !(p->rest_density > 0)) return SF_ERR_INVALID_ARGUMENT;
    const double pi = 3.14159265358979323846;
    const double mass = (double)p->rest_density * (2.0 * r) * (2.0 * r) * (2.0 * r);
    const double h3 = h * h * h, h6 = h3 * h3, h9 = h6 * h3;
    d->h = (Real)h;
    d->h2 = (Real)(h * h);
    d->mass = (Real)mass;
    d->cd = (Real)(mass * 315.0 / (64.0 * pi * h9));
    d->cp = (Real)(mass * 45.0 / (pi * h6) * 0.5);
    d->cv = (Real)((double)p->viscosity * mass * 45.0 / (pi * h6));
    d->k = (Real)p->pressure_stiffness;
    d->rho0 = (Real)p->rest_density;
    d->inv_rho0 = (Real)(1.0 / (double)p->rest_density);
    d->dt = (Real)p->time_step;
    d->e = (Real)p->boundary_restitution;
    d->r = (Real)r;
    d->eos = p->eos;
    d->attractive = p->use_attractive_pressure;
    d->adaptive = p->adaptive_time_step;
    const int K = p->cells_per_h ? p->cells_per_h : 2;
    if (K < 1 || K > 3) return SF_ERR_INVALID_ARGUMENT;
    d->reach = K;
    d->ncells = 1;
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)p->box_max[a] - (double)p->box_min[a];
        if (!(ext > 2.0 * r)) return SF_ERR_INVALID_ARGUMENT;
        d->g[a] = (Real)p->gravity[a];
        d->lo[a] = (Real)((double)p->box_min[a] + r);
        d->hi[a] = (Real)((double)p->box_max[a] - r);
        d->bmin[a] = (Real)p->box_min[a];
        double na = std::floor((double)K * ext / h);
        if (na < 1) na = 1;
        if (na > 65535) return SF_ERR_GRID_TOO_LARGE;
        d->n[a] = (int)na;
        d->inv_cell[a] = (Real)(na / ext);
        d->ncells *= (uint64_t)d->n[a];
    }
    if (d->ncells > (1ull << 28)) return SF_ERR_GRID_TOO_LARGE;
    return SF_OK;
}

template <typename Real>
inline int cell_coord(Real x, Real bmin, Real inv_cell, int n) {
    Real t = std::floor((x - bmin) * inv_cell);
    if (t >= (Real)0) return (t < (Real)n) ? (int)t : n - 1;
    return 0;  // negative or NaN
}

template <typename Real>
inline uint32_t cell_key(const Derived<Real>& d, const Real* x) {
    const int cx = cell_coord(x[0], d.bmin[0], d.inv_cell[0], d.n[0]);
    const int cy = cell_coord(x[1], d.bmin[1], d.inv_cell[1], d.n[1]);
    const int cz = cell_coord(x[2], d.bmin[2], d.inv_cell[2], d.n[2]);
    return (uint32_t)(((uint64_t)cz * d.n[1] + cy) * d.n[0] + cx);
}

inline uint32_t mix32(uint32_t x) {  // murmur3 finaliser
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

void set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

// Keys of the current order; stable counting sort of pos/vel/ids by key;
// cell_start[ncells + 1].
template <typename Real>
void sort_and_grid(const Derived<Real>& d, uint32_t n, Real* pos, Real* vel, uint32_t* ids,
                   std::vector<uint32_t>& keys, std::vector<uint32_t>& cell_start) {
    keys.resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) keys[i] = cell_key(d, pos + 3 * i);
    cell_start.assign(d.ncells + 1, 0);
    for (uint32_t i = 0; i < n; ++i) cell_start[keys[i] + 1]++;
    for (uint64_t c = 0; c < d.ncells; ++c) cell_start[c + 1] += cell_start[c];
    std::vector<uint32_t> fill(cell_start.begin(), cell_start.end() - 1);
    std::vector<uint32_t> dst(n);
    for (uint32_t i = 0; i < n; ++i) dst[i] = fill[keys[i]]++;  // stable: ascending i
    std::vector<Real> tp(3 * (size_t)n), tv(3 * (size_t)n);
    std::vector<uint32_t> ti(n), tk(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint32_t o = dst[i];
        for (int a = 0; a < 3; ++a) {
            tp[3 * (size_t)o + a] = pos[3 * i + a];
            tv[3 * (size_t)o + a] = vel[3 * i + a];
        }
        ti[o] = ids[i];
        tk[o] = keys[i];
    }
    std::memcpy(pos, tp.data(), sizeof(Real) * 3 * (size_t)n);
    std::memcpy(vel, tv.data(), sizeof(Real) * 3 * (size_t)n);
    std::memcpy(ids, ti.data(), sizeof(uint32_t) * n);
    keys.swap(tk);
}

// Cell table of an already sorted state.
template <typename Real>
int grid_of_sorted(const Derived<Real>& d, uint32_t n, const Real* pos, std::vector<uint32_t>& cell_start) {
    cell_start.assign(d.ncells + 1, 0);
    uint32_t prev = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t k = cell_key(d, pos + 3 * (size_t)i);
        if (k < prev) return SF_ERR_INVALID_ARGUMENT;  // not sorted
        prev = k;
        cell_start[k + 1]++;
    }
    for (uint64_t c = 0; c < d.ncells; ++c) cell_start[c + 1] += cell_start[c];
    return SF_OK;
}

// Visit neighbour candidates of sorted particle i in canonical order.
template <typename Real, typename F>
inline void for_candidates(const Derived<Real>& d, const std::vector<uint32_t>& cs, const Real* xi, F&& f) {
    const int cx = cell_coord(xi[0], d.bmin[0], d.inv_cell[0], d.n[0]);
    const int cy = cell_coord(xi[1], d.bmin[1], d.inv_cell[1], d.n[1]);
    const int cz = cell_coord(xi[2], d.bmin[2], d.inv_cell[2], d.n[2]);
    const int R = d.reach;
    const int x0 = std::max(cx - R, 0), x1 = std::min(cx + R, d.n[0] - 1);
    for (int z = cz - R; z <= cz + R; ++z) {
        if (z < 0 || z >= d.n[2]) continue;
        for (int y = cy - R; y <= cy + R; ++y) {
            if (y < 0 || y >= d.n[1]) continue;
            const uint64_t row = ((uint64_t)z * d.n[1] + y) * d.n[0];
            const uint32_t b = cs[row + x0], e = cs[row + x1 + 1];
            for (uint32_t j = b; j < e; ++j) f(j);
        }
    }
}

template <typename Real>
inline Real r2_of(const Real* xi, const Real* xj, Real* dx) {
    dx[0] = xi[0] - xj[0];
    dx[1] = xi[1] - xj[1];
    dx[2] = xi[2] - xj[2];
    return std::fma(dx[2], dx[2], std::fma(dx[1], dx[1], dx[0] * dx[0]));
}

template <typename Real>
void density_pass(const Derived<Real>& d, uint32_t n, const Real* pos, const std::vector<uint32_t>& cs,
                  Real* rho, Real* prs, Real* inv_rho) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const Real* xi = pos + 3 * i;
        Real s = 0;
        for_candidates(d, cs, xi, [&](uint32_t j) {
            Real dx[3];
            const Real r2 = r2_of(xi, pos + 3 * (size_t)j, dx);
            if (r2 < d.h2) {
                const Real q = d.h2 - r2;
                s = std::fma(q * q, q, s);
            }
        });
        const Real rh = d.cd * s;
        Real p;
        if (d.eos == SF_EOS_TAIT) {
            const Real x = rh * d.inv_rho0;
            const Real x2 = x * x;
            const Real x4 = x2 * x2;
            const Real x7 = (x4 * x2) * x;
            p = d.k * (x7 - (Real)1);
        } else {
            p = d.k * (rh - d.rho0);
        }
        if (!d.attractive) p = (p < (Real)0) ? (Real)0 : p;
        if (rho) rho[i] = rh;
        prs[i] = p;
        inv_rho[i] = (Real)1 / rh;
    }
}

template <typename Real>
void accel_pass(const Derived<Real>& d, uint32_t n, const Real* pos, const Real* vel, const Real* prs,
                const Real* inv_rho, const std::vector<uint32_t>& cs, Real* acc, Real* ap_out = nullptr,
                Real* av_out = nullptr) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const Real* xi = pos + 3 * i;
        const Real* vi = vel + 3 * i;
        const Real pi_ = prs[i];
        Real ap[3] = {0, 0, 0}, av[3] = {0, 0, 0};
        for_candidates(d, cs, xi, [&](uint32_t j) {
            if ((int64_t)j == i) return;
            Real dx[3];
            const Real r2 = r2_of(xi, pos + 3 * (size_t)j, dx);
            if (r2 < d.h2) {
                const Real r = std::sqrt(r2);
                const Real hr = d.h - r;
                const Real w = hr * inv_rho[j];
                const Real* vj = vel + 3 * (size_t)j;
                av[0] = std::fma(w, vj[0] - vi[0], av[0]);
                av[1] = std::fma(w, vj[1] - vi[1], av[1]);
                av[2] = std::fma(w, vj[2] - vi[2], av[2]);
                if (r > (Real)0) {
                    const Real sp = ((pi_ + prs[j]) * w) * (hr / r);
                    ap[0] = std::fma(sp, dx[0], ap[0]);
                    ap[1] = std::fma(sp, dx[1], ap[1]);
                    ap[2] = std::fma(sp, dx[2], ap[2]);
                }
            }
        });
        for (int a = 0; a < 3; ++a) {
            const Real t = std::fma(d.cp, ap[a], d.cv * av[a]);
            acc[3 * i + a] = std::fma(t, inv_rho[i], d.g[a]);
            if (ap_out) ap_out[3 * i + a] = ap[a];
            if (av_out) av_out[3 * i + a] = av[a];
        }
    }
}

template <typename Real>
void integrate_pass(const Derived<Real>& d, uint32_t n, Real* pos, Real* vel, const Real* acc, Real dt) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        for (int a = 0; a < 3; ++a) {
            Real v = std::fma(dt, acc[3 * i + a], vel[3 * i + a]);
            Real x = std::fma(dt, v, pos[3 * i + a]);
            if (x < d.lo[a]) {
                x = d.lo[a];
                if (v < (Real)0) v = -d.e * v;
            }
            if (x > d.hi[a]) {
                x = d.hi[a];
                if (v > (Real)0) v = -d.e * v;
            }
            pos[3 * i + a] = x;
            vel[3 * i + a] = v;
        }
    }
}

// One sub-step after another, with the sub-step rule of the context: fixed
// dt, or the adaptive dt = min(dt_max, 0.4 h / max|v|, 0.25 sqrt(h / max|a|))
// from the maxima of the previous sub-step (|v| after integration; for the
// first sub-step max|v| of the initial state and no acceleration term).
template <typename Real>
struct SubStepper {
    const Derived<Real>& d;
    uint32_t n;
    Real v2max = 0, a2max = 0, last_dt = 0;
    std::vector<uint32_t> keys, cs;
    std::vector<Real> prs, inv, acc;
    SubStepper(const Derived<Real>& dd, uint32_t nn, const Real* vel) : d(dd), n(nn), prs(nn), inv(nn), acc(3 * (size_t)nn) {
        for (uint32_t i = 0; i < n; ++i) v2max = std::max(v2max, sq3(vel + 3 * (size_t)i));
    }
    static Real sq3(const Real* v) { return std::fma(v[2], v[2], std::fma(v[1], v[1], v[0] * v[0])); }
    Real choose_dt() const {
        Real dt = d.dt;
        if (d.adaptive) {
            const Real cfl_v = (Real)0.4f, cfl_a = (Real)0.25f;
            if (v2max > (Real)0) dt = std::min(dt, (cfl_v * d.h) / std::sqrt(v2max));
            if (a2max > (Real)0) dt = std::min(dt, cfl_a * std::sqrt(d.h / std::sqrt(a2max)));
        }
        return dt;
    }
    void step(Real* pos, Real* vel, uint32_t* ids) {
        const Real dt = choose_dt();
        sort_and_grid(d, n, pos, vel, ids, keys, cs);
        density_pass(d, n, pos, cs, (Real*)nullptr, prs.data(), inv.data());
        accel_pass(d, n, pos, vel, prs.data(), inv.data(), cs, acc.data());
        integrate_pass(d, n, pos, vel, acc.data(), dt);
        if (d.adaptive) {
            Real vm = 0, am = 0;
            for (uint32_t i = 0; i < n; ++i) {
                vm = std::max(vm, sq3(vel + 3 * (size_t)i));
                am = std::max(am, sq3(&acc[3 * (size_t)i]));
            }
            v2max = vm;
            a2max = am;
        }
        last_dt = dt;
    }
};

template <typename Real>
int step_impl(const sf_params* p, uint32_t n, Real* pos, Real* vel, uint32_t* ids, uint32_t nsteps,
              int threads) {
    Derived<Real> d;
    int st = derive(p, &d);
    if (st) return st;
    if (n == 0) return SF_OK;
    if (!pos || !vel || !ids) return SF_ERR_INVALID_ARGUMENT;
    set_threads(threads);
    SubStepper<Real> stepper(d, n, vel);
    for (uint32_t s = 0; s < nsteps; ++s) stepper.step(pos, vel, ids);
    return SF_OK;
}


// ------------------------------------------------------------- adjoint --
// Hand-written adjoint of one sub-step with the neighbour structure of that
// step held fixed (piecewise-constant), and of the CIC histogram loss.  The
// CUDA adjoint performs the same operations in the same order.
//
// Forward step per particle (sorted order of the step), for reference:
//   rho = cd sum_j (h^2 - r^2)^3, p = EOS(rho) (clamped), inv = 1/rho
//   AP = sum_j (p_i + p_j) w_ij (hr/r) d_ij,  AV = sum_j w_ij (v_j - v_i),
//   w_ij = hr inv_j, hr = h - r, d_ij = x_i - x_j
//   a = (cp AP + cv AV) inv + g;  v' = v + dt a;  x' = x + dt v';  box clamp.
template <typename Real>
struct StepRecord {
    std::vector<Real> pos, vel, rho, prs, inv, ap, av;
    std::vector<uint32_t> ids, cs;
};

template <typename Real>
inline Real dot3(const Real* a, const Real* b) {
    return std::fma(a[2], b[2], std::fma(a[1], b[1], a[0] * b[0]));
}

// dp/drho and dp/dk of the equation of state, 0 where the clamp is active.
template <typename Real>
inline void eos_derivs(const Derived<Real>& d, Real rho, Real* dpdrho, Real* dpdk) {
    Real ppre, dr, dk;
    if (d.eos == SF_EOS_TAIT) {
        const Real x = rho * d.inv_rho0;
        const Real x2 = x * x;
        const Real x4 = x2 * x2;
        const Real x6 = x4 * x2;
        const Real x7 = x6 * x;
        ppre = d.k * (x7 - (Real)1);
        dr = ((Real)7 * d.k) * (x6 * d.inv_rho0);
        dk = x7 - (Real)1;
    } else {
        ppre = d.k * (rho - d.rho0);
        dr = d.k;
        dk = rho - d.rho0;
    }
    const bool act = d.attractive || ppre > (Real)0;
    *dpdrho = act ? dr : (Real)0;
    *dpdk = act ? dk : (Real)0;
}

template <typename Real>
void adjoint_step(const Derived<Real>& d, uint32_t n, const StepRecord<Real>& R, Real* Xb, Real* Vb, double* mub,
                  double* kb) {
    std::vector<Real> apb(3 * (size_t)n), avb(3 * (size_t)n), invb(n), xdir(3 * (size_t)n), vdir(3 * (size_t)n);
    std::vector<Real> cvb(n), rhob(n), xf(3 * (size_t)n), vf(3 * (size_t)n), kbp(n);
    // P1: integration and the acceleration's own inputs
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint32_t id = R.ids[i];
        const Real inv = R.inv[i];
        Real tb[3], t[3], ab3[3];
        for (int a = 0; a < 3; ++a) {
            const Real x = R.pos[3 * i + a], v = R.vel[3 * i + a];
            t[a] = std::fma(d.cp, R.ap[3 * i + a], d.cv * R.av[3 * i + a]);
            const Real acc = std::fma(t[a], inv, d.g[a]);
            const Real vpre = std::fma(d.dt, acc, v);
            const Real xpre = std::fma(d.dt, vpre, x);
            const bool lo = xpre < d.lo[a], hi = xpre > d.hi[a];
            const bool pass = !lo && !hi;
            const Real sv = ((lo && vpre < (Real)0) || (hi && vpre > (Real)0)) ? -d.e : (Real)1;
            const Real xbpre = pass ? Xb[3 * (size_t)id + a] : (Real)0;
            const Real vbpre = std::fma(sv, Vb[3 * (size_t)id + a], d.dt * xbpre);
            xdir[3 * i + a] = xbpre;
            vdir[3 * i + a] = vbpre;
            ab3[a] = d.dt * vbpre;
            tb[a] = ab3[a] * inv;
            apb[3 * i + a] = d.cp * tb[a];
            avb[3 * i + a] = d.cv * tb[a];
        }
        invb[i] = dot3(ab3, t);
        const Real av3[3] = {R.av[3 * i], R.av[3 * i + 1], R.av[3 * i + 2]};
        cvb[i] = dot3(tb, av3);
    }
    // P2: pair terms of the forces, both orientations of each pair; then the
    // density adjoint of each particle (inverse and equation of state)
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        const Real* xk = &R.pos[3 * k];
        const Real* vk = &R.vel[3 * k];
        const Real pk = R.prs[k], invk = R.inv[k];
        const Real* apbk = &apb[3 * k];
        const Real* avbk = &avb[3 * k];
        Real pb = 0, invacc = 0, xb[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
        for_candidates(d, R.cs, xk, [&](uint32_t j) {
            if ((int64_t)j == k) return;
            Real dd[3];
            const Real r2 = r2_of(xk, &R.pos[3 * (size_t)j], dd);
            if (!(r2 < d.h2)) return;
            const Real r = std::sqrt(r2);
            const Real hr = d.h - r;
            const Real pj = R.prs[j], invj = R.inv[j];
            const Real* vj = &R.vel[3 * (size_t)j];
            const Real* apbj = &apb[3 * (size_t)j];
            const Real* avbj = &avb[3 * (size_t)j];
            const Real dv[3] = {vj[0] - vk[0], vj[1] - vk[1], vj[2] - vk[2]};
            const Real ps = pk + pj;
            // orientation A: k is i, j is the neighbour
            const Real wkj = hr * invj;
            for (int a = 0; a < 3; ++a) vb[a] = std::fma(-wkj, avbk[a], vb[a]);
            Real wb = dot3(avbk, dv);
            Real rb = 0;
            // orientation B: j is i, k is the neighbour
            const Real wjk = hr * invk;
            for (int a = 0; a < 3; ++a) vb[a] = std::fma(wjk, avbj[a], vb[a]);
            Real wb2 = -dot3(avbj, dv);
            Real rb2 = 0;
            if (r > (Real)0) {
                const Real q = hr / r;
                const Real S = (ps * wkj) * q;
                const Real Sb = dot3(apbk, dd);
                for (int a = 0; a < 3; ++a) xb[a] = std::fma(S, apbk[a], xb[a]);
                pb = std::fma(Sb, wkj * q, pb);
                wb = std::fma(Sb, ps * q, wb);
                const Real qb = Sb * (ps * wkj);
                rb = -((qb * d.h) / r2);
                const Real S2 = (ps * wjk) * q;
                const Real Sb2 = -dot3(apbj, dd);
                for (int a = 0; a < 3; ++a) xb[a] = std::fma(-S2, apbj[a], xb[a]);
                pb = std::fma(Sb2, wjk * q, pb);
                wb2 = std::fma(Sb2, ps * q, wb2);
                const Real qb2 = Sb2 * (ps * wjk);
                rb2 = -((qb2 * d.h) / r2);
            }
            rb = std::fma(-wb, invj, rb);
            invacc = std::fma(wb2, hr, invacc);
            rb2 = std::fma(-wb2, invk, rb2);
            if (r > (Real)0) {
                const Real g = (rb + rb2) / r;
                for (int a = 0; a < 3; ++a) xb[a] = std::fma(g, dd[a], xb[a]);
            }
        });
        const Real ib = invb[k] + invacc;
        Real dpdrho, dpdk;
        eos_derivs(d, R.rho[k], &dpdrho, &dpdk);
        rhob[k] = std::fma(pb, dpdrho, -((ib * invk) * invk));
        kbp[k] = pb * dpdk;
        for (int a = 0; a < 3; ++a) {
            xf[3 * k + a] = xb[a];
            vf[3 * k + a] = vb[a];
        }
    }
    // P4: density adjoint onto positions; write the step's input adjoints
    const Real m6cd = (Real)(-6.0 * (double)d.cd);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        const Real* xk = &R.pos[3 * k];
        const Real rbk = rhob[k];
        Real xd[3] = {0, 0, 0};
        for_candidates(d, R.cs, xk, [&](uint32_t j) {
            if ((int64_t)j == k) return;
            Real dd[3];
            const Real r2 = r2_of(xk, &R.pos[3 * (size_t)j], dd);
            if (!(r2 < d.h2)) return;
            const Real q = d.h2 - r2;
            const Real sc = (rbk + rhob[j]) * (q * q);
            for (int a = 0; a < 3; ++a) xd[a] = std::fma(sc, dd[a], xd[a]);
        });
        const uint32_t id = R.ids[k];
        for (int a = 0; a < 3; ++a) {
            const Real xt = xdir[3 * k + a] + xf[3 * k + a];
            Xb[3 * (size_t)id + a] = std::fma(m6cd, xd[a], xt);
            Vb[3 * (size_t)id + a] = vdir[3 * k + a] + vf[3 * k + a];
        }
    }
    double cvs = 0, ks = 0;
    for (uint32_t i = 0; i < n; ++i) {
        cvs += (double)cvb[i];
        ks += (double)kbp[i];
    }
    *mub += cvs;
    *kb += ks;
}

// CIC histogram on res^3 cells over the box (cell-centred), normalised by n.
template <typename Real>
void hist_weights(const Derived<Real>& d, const Real* bext, uint32_t res, const Real* x, int i0[3], Real w0[3],
                  Real w1[3], Real dw[3]) {
    for (int a = 0; a < 3; ++a) {
        const Real inv = (Real)res / bext[a];
        const Real u = (x[a] - d.bmin[a]) * inv - (Real)0.5;
        const Real fl = std::floor(u);
        const Real f = u - fl;
        i0[a] = (int)fl;
        w0[a] = (Real)1 - f;
        w1[a] = f;
        dw[a] = inv;
    }
}

template <typename Real>
Real histogram_loss(const Derived<Real>& d, const Real* bext, uint32_t n, const Real* pos, const Real* target,
                    uint32_t res, Real* dldx, std::vector<double>* hist_out) {
    const size_t nc = (size_t)res * res * res;
    std::vector<double> H(nc, 0.0);
    for (uint32_t p = 0; p < n; ++p) {
        int i0[3];
        Real w0[3], w1[3], dw[3];
        hist_weights(d, bext, res, pos + 3 * (size_t)p, i0, w0, w1, dw);
        for (int c = 0; c < 8; ++c) {
            const int ix = i0[0] + (c & 1), iy = i0[1] + ((c >> 1) & 1), iz = i0[2] + ((c >> 2) & 1);
            if (ix < 0 || iy < 0 || iz < 0 || ix >= (int)res || iy >= (int)res || iz >= (int)res) continue;
            const Real w = ((c & 1) ? w1[0] : w0[0]) * ((c & 2) ? w1[1] : w0[1]) * ((c & 4) ? w1[2] : w0[2]);
            H[((size_t)iz * res + iy) * res + ix] += (double)w;
        }
    }
    double L = 0;
    for (size_t c = 0; c < nc; ++c) {
        H[c] /= (double)n;
        const double e = H[c] - (double)target[c];
        L += e * e;
    }
    if (dldx) {
        for (uint32_t p = 0; p < n; ++p) {
            int i0[3];
            Real w0[3], w1[3], dw[3];
            hist_weights(d, bext, res, pos + 3 * (size_t)p, i0, w0, w1, dw);
            Real g[3] = {0, 0, 0};
            for (int c = 0; c < 8; ++c) {
                const int ix = i0[0] + (c & 1), iy = i0[1] + ((c >> 1) & 1), iz = i0[2] + ((c >> 2) & 1);
                if (ix < 0 || iy < 0 || iz < 0 || ix >= (int)res || iy >= (int)res || iz >= (int)res) continue;
                const size_t cc = ((size_t)iz * res + iy) * res + ix;
                const Real e2 = (Real)(2.0 * (H[cc] - (double)target[cc]) / (double)n);
                const Real wx = (c & 1) ? w1[0] : w0[0], wy = (c & 2) ? w1[1] : w0[1], wz = (c & 4) ? w1[2] : w0[2];
                const Real sx = (c & 1) ? dw[0] : -dw[0], sy = (c & 2) ? dw[1] : -dw[1], sz = (c & 4) ? dw[2] : -dw[2];
                g[0] += e2 * (sx * (wy * wz));
                g[1] += e2 * (sy * (wx * wz));
                g[2] += e2 * (sz * (wx * wy));
            }
            for (int a = 0; a < 3; ++a) dldx[3 * (size_t)p + a] = g[a];
        }
    }
    if (hist_out) *hist_out = H;
    return (Real)L;
}

// Forward nsteps from (pos0, vel0), CIC loss at the end (or, with `seed_x`,
// the given adjoint of the final state instead), and the adjoint back to the
// initial state, recomputing segments of `ckpt` steps from checkpoints.
template <typename Real>
int grad_impl(const sf_params* p, uint32_t n, const Real* pos0, const Real* vel0, uint32_t nsteps, uint32_t ckpt,
              const Real* target, uint32_t res, Real* loss_out, Real* gx0, Real* gv0, Real* gmu, Real* gk,
              Real* pos_final, int threads, const Real* seed_x = nullptr, const Real* seed_v = nullptr) {
    Derived<Real> d;
    int st = derive(p, &d);
    if (st) return st;
    if (!pos0 || !vel0 || n == 0 || ckpt == 0) return SF_ERR_INVALID_ARGUMENT;
    if (!seed_x && (!target || res == 0)) return SF_ERR_INVALID_ARGUMENT;
    set_threads(threads);
    Real bext[3];
    for (int a = 0; a < 3; ++a) bext[a] = (Real)((double)p->box_max[a] - (double)p->box_min[a]);
    const size_t n3 = 3 * (size_t)n;
    std::vector<Real> pos(pos0, pos0 + n3), vel(vel0, vel0 + n3);
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    struct Ckpt {
        std::vector<Real> pos, vel;
        std::vector<uint32_t> ids;
    };
    std::vector<Ckpt> cks;
    std::vector<uint32_t> keys, cs;
    std::vector<Real> prs(n), inv(n), acc(n3);
    for (uint32_t s = 0; s < nsteps; ++s) {
        if (s % ckpt == 0) cks.push_back({pos, vel, ids});
        sort_and_grid(d, n, pos.data(), vel.data(), ids.data(), keys, cs);
        density_pass(d, n, pos.data(), cs, (Real*)nullptr, prs.data(), inv.data());
        accel_pass(d, n, pos.data(), vel.data(), prs.data(), inv.data(), cs, acc.data());
        integrate_pass(d, n, pos.data(), vel.data(), acc.data(), d.dt);
    }
    // loss at the final state (array order = the last step's sorted order)
    std::vector<Real> Xb(n3, (Real)0), Vb(n3, (Real)0);
    if (seed_x) {
        std::memcpy(Xb.data(), seed_x, n3 * sizeof(Real));
        if (seed_v) std::memcpy(Vb.data(), seed_v, n3 * sizeof(Real));
    } else {
        std::vector<Real> dldx(n3);
        const Real L = histogram_loss(d, bext, n, pos.data(), target, res, dldx.data(), nullptr);
        if (loss_out) *loss_out = L;
        for (uint32_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) Xb[3 * (size_t)ids[i] + a] = dldx[3 * (size_t)i + a];
    }
    if (pos_final)
        for (uint32_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) pos_final[3 * (size_t)ids[i] + a] = pos[3 * (size_t)i + a];
    double mub = 0, kb = 0;
    for (int64_t seg = (int64_t)cks.size() - 1; seg >= 0; --seg) {
        const uint32_t s0 = (uint32_t)seg * ckpt, s1 = std::min(nsteps, s0 + ckpt);
        std::vector<StepRecord<Real>> recs(s1 - s0);
        std::vector<Real> ps = cks[seg].pos, vs = cks[seg].vel;
        std::vector<uint32_t> is = cks[seg].ids;
        for (uint32_t s = s0; s < s1; ++s) {
            StepRecord<Real>& R = recs[s - s0];
            sort_and_grid(d, n, ps.data(), vs.data(), is.data(), keys, R.cs);
            R.pos = ps;
            R.vel = vs;
            R.ids = is;
            R.rho.resize(n);
            R.prs.resize(n);
            R.inv.resize(n);
            R.ap.resize(n3);
            R.av.resize(n3);
            density_pass(d, n, ps.data(), R.cs, R.rho.data(), R.prs.data(), R.inv.data());
            accel_pass(d, n, ps.data(), vs.data(), R.prs.data(), R.inv.data(), R.cs, acc.data(), R.ap.data(),
                       R.av.data());
            integrate_pass(d, n, ps.data(), vs.data(), acc.data(), d.dt);
        }
        for (int64_t s = (int64_t)s1 - 1; s >= (int64_t)s0; --s) adjoint_step(d, n, recs[s - s0], Xb.data(), Vb.data(), &mub, &kb);
    }
    if (gx0) std::memcpy(gx0, Xb.data(), n3 * sizeof(Real));
    if (gv0) std::memcpy(gv0, Vb.data(), n3 * sizeof(Real));
    // cv = mu * m * 45 / (pi h^6)
    const double pi = 3.14159265358979323846;
    const double hh = (double)p->kernel_radius, rr = (double)p->particle_radius;
    const double mass = (double)p->rest_density * (2.0 * rr) * (2.0 * rr) * (2.0 * rr);
    const double h6 = hh * hh * hh * hh * hh * hh;
    if (gmu) *gmu = (Real)(mub * (mass * 45.0 / (pi * h6)));
    if (gk) *gk = (Real)kb;
    return SF_OK;
}


// ------------------------------------------------------------- rendering --
// Restatement of the reference's point-sprite shaders (Shaders/particle.vs.glsl:24-35,
// Shaders/particle.fs.glsl:46-83) as two passes: nearest centre depth per
// pixel (ties to the lower particle index), then Blinn-Phong shading of the
// winner.  Matrices follow glm::lookAt / glm::perspective.
struct RCo {
    float V[16], P[16], scale, radius;
    int W, H;
};

RCo render_const(const sf_render_params* rp, float particle_radius) {
    RCo rc;
    double e[3], f[3], u[3], s3[3], uu[3];
    for (int a = 0; a < 3; ++a) {
        e[a] = rp->eye[a];
        f[a] = (double)rp->focus[a] - rp->eye[a];
        u[a] = rp->up[a];
    }
    auto norm = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int a = 0; a < 3; ++a) v[a] /= l;
    };
    norm(f);
    s3[0] = f[1] * u[2] - f[2] * u[1];
    s3[1] = f[2] * u[0] - f[0] * u[2];
    s3[2] = f[0] * u[1] - f[1] * u[0];
    norm(s3);
    uu[0] = s3[1] * f[2] - s3[2] * f[1];
    uu[1] = s3[2] * f[0] - s3[0] * f[2];
    uu[2] = s3[0] * f[1] - s3[1] * f[0];
    double V[16] = {0}, P[16] = {0};
    for (int a = 0; a < 3; ++a) {
        V[4 * a] = s3[a];
        V[4 * a + 1] = uu[a];
        V[4 * a + 2] = -f[a];
    }
    V[12] = -(s3[0] * e[0] + s3[1] * e[1] + s3[2] * e[2]);
    V[13] = -(uu[0] * e[0] + uu[1] * e[1] + uu[2] * e[2]);
    V[14] = f[0] * e[0] + f[1] * e[1] + f[2] * e[2];
    V[15] = 1.0;
    const double pi = 3.14159265358979323846;
    const double th = std::tan((double)rp->fovy_deg * 0.5 * pi / 180.0);
    const double aspect = (double)rp->width / (double)rp->height;
    P[0] = 1.0 / (aspect * th);
    P[5] = 1.0 / th;
    P[10] = -((double)rp->zfar + rp->znear) / ((double)rp->zfar - rp->znear);
    P[11] = -1.0;
    P[14] = -(2.0 * rp->zfar * (double)rp->znear) / ((double)rp->zfar - rp->znear);
    for (int k = 0; k < 16; ++k) {
        rc.V[k] = (float)V[k];
        rc.P[k] = (float)P[k];
    }
    rc.scale = (float)rp->height / std::tan((float)((double)rp->fovy_deg * 0.5 * pi / 180.0));
    rc.radius = rp->point_radius > 0.f ? rp->point_radius : particle_radius;
    rc.W = rp->width;
    rc.H = rp->height;
    return rc;
}

struct SplatO {
    float e[3], x0, y0, size, depth;
};

// The vertex stage (Shaders/particle.vs.glsl:24-35): eye-space centre e,
// point size and clip position c of one particle.  The view matrix's bottom
// row is (0, 0, 0, 1), so the eye coordinate's w is exactly 1 and the
// projection's last column is added as is.
void vertex_o(const RCo& rc, const float* p, float* e, float& size, float* c) {
    for (int r = 0; r < 3; ++r) e[r] = ((rc.V[r] * p[0] + rc.V[4 + r] * p[1]) + rc.V[8 + r] * p[2]) + rc.V[12 + r];
    const float dist = std::sqrt((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]);
    size = rc.radius * (rc.scale / dist);
    for (int r = 0; r < 4; ++r) c[r] = ((rc.P[r] * e[0] + rc.P[4 + r] * e[1]) + rc.P[8 + r] * e[2]) + rc.P[12 + r];
}

bool splat_o(const RCo& rc, const float* p, SplatO& s) {
    float c[4];
    vertex_o(rc, p, s.e, s.size, c);
    if (!(c[3] > 0.f)) return false;
    if (c[0] < -c[3] || c[0] > c[3] || c[1] < -c[3] || c[1] > c[3] || c[2] < -c[3] || c[2] > c[3]) return false;
    const float nx = c[0] / c[3], ny = c[1] / c[3], nz = c[2] / c[3];
    const float wx = (nx * 0.5f + 0.5f) * (float)rc.W;
    const float wy = (ny * 0.5f + 0.5f) * (float)rc.H;
    s.depth = nz * 0.5f + 0.5f;
    s.x0 = wx - s.size * 0.5f;
    s.y0 = ((float)rc.H - wy) - s.size * 0.5f;
    return true;
}

// gl_PointCoord (u, v) to the sprite normal's x and y and their squared
// length (Shaders/particle.fs.glsl:67-68).
float coord_normal_o(float u, float v, float& nx, float& ny) {
    nx = u * 2.0f + -1.0f;
    ny = v * -2.0f + 1.0f;
    return nx * nx + ny * ny;
}

// Pixel (px, row) of a splat: its point coordinate, then the normal.
float disc_o(const SplatO& s, int px, int row, float& nx, float& ny) {
    const float u = (((float)px + 0.5f) - s.x0) / s.size;
    const float v = (((float)row + 0.5f) - s.y0) / s.size;
    return coord_normal_o(u, v, nx, ny);
}

void normalize_o(float* v) {
    const float len = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    for (int a = 0; a < 3; ++a) v[a] = v[a] / len;
}

// The fragment stage from the normal on (Shaders/particle.fs.glsl:46-59 and
// 70-83) for a fragment that was not discarded: Blinn-Phong per light,
// summed in light order; surf is the surface colour (the particle's colour,
// or the material's diffuse colour).
void shade_o(const sf_render_params* rp, float radius, const float* e, float nx, float ny, float mag,
             const float* surf, float* out) {
    const float nrm[3] = {nx, ny, std::sqrt(1.0f - mag)};
    float view[3] = {e[0], e[1], e[2]};
    normalize_o(view);
    const float frag[3] = {e[0] + nrm[0] * radius, e[1] + nrm[1] * radius, e[2] + nrm[2] * radius};
    float shade[3] = {0, 0, 0};
    for (int l = 0; l < rp->num_lights; ++l) {
        float ld[3] = {rp->light_position[l][0] - frag[0], rp->light_position[l][1] - frag[1],
                       rp->light_position[l][2] - frag[2]};
        normalize_o(ld);
        float hd[3] = {ld[0] - view[0], ld[1] - view[1], ld[2] - view[2]};
        normalize_o(hd);
        const float diff = std::max((nrm[0] * ld[0] + nrm[1] * ld[1]) + nrm[2] * ld[2], 0.f);
        const float spec =
            std::pow(std::max((hd[0] * nrm[0] + hd[1] * nrm[1]) + hd[2] * nrm[2], 0.f), rp->mat_shininess);
        for (int a = 0; a < 3; ++a) {
            const float amb = rp->light_ambient[l][a] * rp->mat_ambient[a];
            const float dif = (rp->light_diffuse[l][a] * diff) * surf[a];
            const float spc = (rp->light_specular[l][a] * spec) * rp->mat_specular[a];
            shade[a] += (amb + dif) + spc;
        }
    }
    out[0] = shade[0];
    out[1] = shade[1];
    out[2] = shade[2];
    out[3] = 1.0f;
}

void color_o(const sf_render_params* rp, uint32_t id, uint32_t n, float* col) {
    if (rp->color_mode == SF_COLOR_RANDOM) {
        uint64_t z = rp->color_seed ^ ((uint64_t)id * 0x9E3779B97F4A7C15ull);
        for (int a = 0; a < 3; ++a) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t q = z;
            q = (q ^ (q >> 30)) * 0xBF58476D1CE4E5B9ull;
            q = (q ^ (q >> 27)) * 0x94D049BB133111EBull;
            q ^= q >> 31;
            col[a] = (float)(q >> 40) * (1.0f / 16777216.0f);
        }
    } else {
        static const float ramp[7][3] = {{1.0f, 0.0f, 0.0f}, {1.0f, 0.5f, 0.0f}, {1.0f, 1.0f, 0.0f}, {1.0f, 0.0f, 1.0f},
                                         {0.0f, 1.0f, 0.0f}, {0.0f, 1.0f, 1.0f}, {0.0f, 0.0f, 1.0f}};
        const float step = (float)(6.0 / (double)(n > 1 ? n - 1 : 1));
        const float t = (float)id * step;
        int k = (int)std::floor(t);
        k = k < 0 ? 0 : (k > 5 ? 5 : k);
        const float f = t - (float)k;
        for (int a = 0; a < 3; ++a) col[a] = std::fma(f, ramp[k + 1][a] - ramp[k][a], ramp[k][a]);
    }
}

// ---------------------------------------------------------------- scenes --
// Restatement of Source/SceneManager.cpp.  Vec3 arithmetic is per component
// in float, as glm does it.
struct V3 {
    float x, y, z;
};

void push(std::vector<float>& out, float x, float y, float z) {
    out.push_back(x);
    out.push_back(y);
    out.push_back(z);
}

// CubeDrop: Source/SceneManager.cpp:41-64
void scene_cube_drop(float r, std::vector<float>& out) {
    const V3 bmin{-0.5f, -0.5f, -0.5f}, bmax{0.5f, 0.5f, 0.5f};
    const float s = 2.0f * r;
    const int gx = (int)((bmax.x - bmin.x) / s), gy = (int)((bmax.y - bmin.y) / s), gz = (int)((bmax.z - bmin.z) / s);
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) push(out, bmin.x + s * (float)i, bmin.y + s * (float)j, bmin.z + s * (float)k);
}

// SphereDrop: Source/SceneManager.cpp:67-91
void scene_sphere_drop(float r, std::vector<float>& out) {
    const V3 c{0.0f, 0.0f, 0.0f};
    const float radius = 0.5f;
    const V3 bmin{c.x - radius, c.y - radius, c.z - radius};
    const float s = 2.0f * r;
    const int g = 1 * (int)(2.0f * radius / s);
    for (int i = 0; i < g; ++i)
        for (int j = 0; j < g; ++j)
            for (int k = 0; k < g; ++k) {
                const float px = bmin.x + s * (float)i, py = bmin.y + s * (float)j, pz = bmin.z + s * (float)k;
                const float dx = px - c.x, dy = py - c.y, dz = pz - c.z;
                const float len = std::sqrt((dx * dx + dy * dy) + dz * dz);
                if (len > radius) continue;
                push(out, px, py, pz);
            }
}

// Dambreak: Source/SceneManager.cpp:94-119
void scene_dambreak(float r, std::vector<float>& out) {
    V3 bmin{-1.0f, -1.0f, -1.0f};
    const V3 bmax{0.4f, 0.4f, -0.5f};
    bmin = V3{bmin.x + r, bmin.y + r, bmin.z + r};
    const float s = 2.0f * r;
    const int gx = (int)((bmax.x - bmin.x) / s), gy = (int)((bmax.y - bmin.y) / s), gz = (int)((bmax.z - bmin.z) / s);
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) push(out, bmin.x + s * (float)i, bmin.y + s * (float)j, bmin.z + s * (float)k);
}

// DoubleDambreak: Source/SceneManager.cpp:122-173
void scene_double_dambreak(float r, std::vector<float>& out) {
    const float s = 2.0f * r;
    scene_dambreak(r, out);  // first block (:131-148) is the Dambreak block
    V3 bmin{-0.4f, -1.0f, 0.5f};
    bmin = V3{bmin.x + 0.0f, bmin.y + r, bmin.z + 0.0f};
    const V3 bmax{1.0f - r, 0.4f - 0.0f, 1.0f - r};
    const int gx = (int)((bmax.x - bmin.x) / s), gy = (int)((bmax.y - bmin.y) / s), gz = (int)((bmax.z - bmin.z) / s);
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) push(out, bmax.x - s * (float)i, bmax.y - s * (float)j, bmax.z - s * (float)k);
}

// Uniform double in [0,1) from the top 53 bits of a 64-bit Mersenne twister.
struct Jitter {
    std::mt19937_64 eng;
    double amp;  // 0.1 * spacing
    Jitter(uint64_t seed, double spacing) : eng(seed), amp(0.1 * spacing) {}
    float next() {
        const double u = (double)(eng() >> 11) * (1.0 / 9007199254740992.0);
        return (float)((2.0 * u - 1.0) * amp);
    }
};

// Benchmark lattice block: counts (a, b, c); origin corner `o`; per-axis
// direction sign (+1 from box_min + r, -1 from box_max - r).
void lattice_block(const sf_params* p, int ca, int cb, int cc, const int sgn[3], Jitter* jit, std::vector<float>& out) {
    const float r = p->particle_radius, s = 2.0f * r;
    float o[3];
    for (int a = 0; a < 3; ++a) o[a] = sgn[a] > 0 ? p->box_min[a] + r : p->box_max[a] - r;
    for (int i = 0; i < ca; ++i)
        for (int j = 0; j < cb; ++j)
            for (int k = 0; k < cc; ++k) {
                const int idx[3] = {i, j, k};
                float q[3];
                for (int a = 0; a < 3; ++a) q[a] = sgn[a] > 0 ? o[a] + s * (float)idx[a] : o[a] - s * (float)idx[a];
                if (jit)
                    for (int a = 0; a < 3; ++a) q[a] = q[a] + jit->next();
                push(out, q[0], q[1], q[2]);
            }
}

void scene_sphere_pool(const sf_params* p, uint64_t seed, std::vector<float>& out) {
    const float r = p->particle_radius, s = 2.0f * r;
    Jitter jit(seed, s);
    const int nx = (int)(((double)p->box_max[0] - p->box_min[0]) / s);
    const int nz = (int)(((double)p->box_max[2] - p->box_min[2]) / s);
    const int ny = (int)(0.3 / (double)s);
    const int up[3] = {1, 1, 1};
    lattice_block(p, nx, ny, nz, up, &jit, out);
    const float R = 0.15f;
    const float c[3] = {0.5f * (p->box_min[0] + p->box_max[0]), p->box_min[1] + 0.6f,
                        0.5f * (p->box_min[2] + p->box_max[2])};
    const int m = (int)(2.0f * R / s);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            for (int k = 0; k < m; ++k) {
                const float q[3] = {(c[0] - R) + s * ((float)i + 0.5f), (c[1] - R) + s * ((float)j + 0.5f),
                                    (c[2] - R) + s * ((float)k + 0.5f)};
                const float dx = q[0] - c[0], dy = q[1] - c[1], dz = q[2] - c[2];
                if ((dx * dx + dy * dy) + dz * dz > R * R) continue;
                const float a = jit.next(), b = jit.next(), e = jit.next();
                push(out, q[0] + a, q[1] + b, q[2] + e);
            }
}

int make_scene(const sf_params* p, int scene, uint64_t seed, std::vector<float>& out) {
    if (!p || !(p->particle_radius > 0)) return SF_ERR_INVALID_ARGUMENT;
    const float r = p->particle_radius;
    out.clear();
    switch (scene) {
        case SF_SCENE_CUBE_DROP: scene_cube_drop(r, out); break;
        case SF_SCENE_SPHERE_DROP: scene_sphere_drop(r, out); break;
        case SF_SCENE_DAMBREAK: scene_dambreak(r, out); break;
        case SF_SCENE_DOUBLE_DAMBREAK: scene_double_dambreak(r, out); break;
        case SF_SCENE_DAMBREAK_16K: {
            const int up[3] = {1, 1, 1};
            lattice_block(p, 20, 40, 20, up, nullptr, out);
            break;
        }
        case SF_SCENE_DAMBREAK_64K: {
            const int up[3] = {1, 1, 1};
            lattice_block(p, 32, 64, 32, up, nullptr, out);
            break;
        }
        case SF_SCENE_DOUBLE_DAMBREAK_1M: {
            Jitter jit(seed, 2.0 * r);
            const int a[3] = {1, 1, 1}, b[3] = {-1, 1, -1};
            lattice_block(p, 64, 128, 64, a, &jit, out);
            lattice_block(p, 64, 128, 64, b, &jit, out);
            break;
        }
        case SF_SCENE_SPHERE_POOL: scene_sphere_pool(p, seed, out); break;
        default: return SF_ERR_INVALID_ARGUMENT;
    }
    if (out.size() / 3 > 0xffffffffull) return SF_ERR_CAPACITY;
    return SF_OK;
}

}  // namespace

// ------------------------------------------------------------- C exports --
extern "C" {

// Derived constants, for tests: h, h2, mass, cd, cp, cv, lo[3], hi[3], inv_cell[3], n[3]
int sfo_derive(const sf_params* p, double* out16) {
    Derived<float> d;
    int st = derive(p, &d);
    if (st) return st;
    const double v[16] = {d.h,      d.h2,     d.mass,   d.cd,     d.cp,     d.cv,     d.lo[0],  d.lo[1],
                          d.lo[2],  d.hi[0],  d.hi[1],  d.hi[2],  (double)d.n[0], (double)d.n[1], (double)d.n[2],
                          (double)d.ncells};
    std::memcpy(out16, v, sizeof(v));
    return SF_OK;
}

int sfo_scene(const sf_params* p, int scene, uint64_t seed, float* pos3, uint32_t cap, uint32_t* n_out) {
    std::vector<float> out;
    int st = make_scene(p, scene, seed, out);
    if (st) return st;
    const uint32_t n = (uint32_t)(out.size() / 3);
    if (n_out) *n_out = n;
    if (pos3) {
        if (cap < n) return SF_ERR_CAPACITY;
        std::memcpy(pos3, out.data(), out.size() * sizeof(float));
    }
    return SF_OK;
}

#define SFO_DEFINE(SUFFIX, Real)                                                                            \
    int sfo_sort_##SUFFIX(const sf_params* p, uint32_t n, Real* pos, Real* vel, uint32_t* ids,              \
                          uint32_t* keys_out, uint32_t* cell_start_out) {                                    \
        Derived<Real> d;                                                                                    \
        int st = derive(p, &d);                                                                             \
        if (st) return st;                                                                                  \
        std::vector<uint32_t> keys, cs;                                                                     \
        sort_and_grid(d, n, pos, vel, ids, keys, cs);                                                       \
        if (keys_out) std::memcpy(keys_out, keys.data(), sizeof(uint32_t) * n);                             \
        if (cell_start_out) std::memcpy(cell_start_out, cs.data(), sizeof(uint32_t) * cs.size());           \
        return SF_OK;                                                                                       \
    }                                                                                                       \
    int sfo_density_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos, Real* rho, Real* prs,         \
                             Real* inv_rho) {                                                               \
        Derived<Real> d;                                                                                    \
        int st = derive(p, &d);                                                                             \
        if (st) return st;                                                                                  \
        std::vector<uint32_t> cs;                                                                           \
        if ((st = grid_of_sorted(d, n, pos, cs))) return st;                                                \
        density_pass(d, n, pos, cs, rho, prs, inv_rho);                                                     \
        return SF_OK;                                                                                       \
    }                                                                                                       \
    int sfo_accel_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos, const Real* vel, const Real* prs, \
                           const Real* inv_rho, Real* acc) {                                                \
        Derived<Real> d;                                                                                    \
        int st = derive(p, &d);                                                                             \
        if (st) return st;                                                                                  \
        std::vector<uint32_t> cs;                                                                           \
        if ((st = grid_of_sorted(d, n, pos, cs))) return st;                                                \
        accel_pass(d, n, pos, vel, prs, inv_rho, cs, acc);                                                  \
        return SF_OK;                                                                                       \
    }                                                                                                       \
    int sfo_integrate_##SUFFIX(const sf_params* p, uint32_t n, Real* pos, Real* vel, const Real* acc) {     \
        Derived<Real> d;                                                                                    \
        int st = derive(p, &d);                                                                             \
        if (st) return st;                                                                                  \
        integrate_pass(d, n, pos, vel, acc, d.dt);                                                          \
        return SF_OK;                                                                                       \
    }                                                                                                       \
    int sfo_neighbour_stats_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos, const uint32_t* ids,   \
                                     uint32_t* count, uint32_t* hash) {                                     \
        Derived<Real> d;                                                                                    \
        int st = derive(p, &d);                                                                             \
        if (st) return st;                                                                                  \
        std::vector<uint32_t> cs;                                                                           \
        if ((st = grid_of_sorted(d, n, pos, cs))) return st;                                                \
        _Pragma("omp parallel for schedule(dynamic, 256)") for (int64_t i = 0; i < (int64_t)n; ++i) {        \
            uint32_t c = 0, hsh = 0;                                                                        \
            for_candidates(d, cs, pos + 3 * i, [&](uint32_t j) {                                            \
                if ((int64_t)j == i) return;                                                                \
                Real dx[3];                                                                                 \
                if (r2_of(pos + 3 * i, pos + 3 * (size_t)j, dx) < d.h2) {                                   \
                    ++c;                                                                                    \
                    hsh += mix32(ids[j]);                                                                   \
                }                                                                                           \
            });                                                                                             \
            count[i] = c;                                                                                   \
            hash[i] = hsh;                                                                                  \
        }                                                                                                   \
        return SF_OK;                                                                                       \
    }                                                                                                       \
    int sfo_step_##SUFFIX(const sf_params* p, uint32_t n, Real* pos, Real* vel, uint32_t* ids, uint32_t nsteps, \
                          int threads) {                                                                    \
        return step_impl<Real>(p, n, pos, vel, ids, nsteps, threads);                                       \
    }

SFO_DEFINE(f32, float)
SFO_DEFINE(f64, double)

#define SFO_GRAD(SUFFIX, Real)                                                                                   \
    int sfo_grad_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos0, const Real* vel0, uint32_t nsteps,    \
                          uint32_t ckpt, const Real* target, uint32_t res, Real* loss, Real* gx0, Real* gv0,      \
                          Real* gmu, Real* gk, Real* pos_final, int threads) {                                   \
        return grad_impl<Real>(p, n, pos0, vel0, nsteps, ckpt, target, res, loss, gx0, gv0, gmu, gk, pos_final,  \
                               threads);                                                                         \
    }                                                                                                            \
    int sfo_loss_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos, const Real* target, uint32_t res,      \
                          Real* loss, Real* dldx, double* hist) {                                                \
        Derived<Real> d;                                                                                         \
        int st = derive(p, &d);                                                                                  \
        if (st) return st;                                                                                       \
        Real bext[3];                                                                                            \
        for (int a = 0; a < 3; ++a) bext[a] = (Real)((double)p->box_max[a] - (double)p->box_min[a]);             \
        std::vector<double> H;                                                                                   \
        *loss = histogram_loss(d, bext, n, pos, target, res, dldx, hist ? &H : nullptr);                         \
        if (hist) std::memcpy(hist, H.data(), H.size() * sizeof(double));                                        \
        return SF_OK;                                                                                            \
    }

SFO_GRAD(f32, float)
SFO_GRAD(f64, double)

// Adjoint from a given final-state adjoint (seed_x, seed_v: n*3 in the
// caller's particle order) — the same inputs sf_adjoint takes.
#define SFO_ADJ(SUFFIX, Real)                                                                                     \
    int sfo_adjoint_##SUFFIX(const sf_params* p, uint32_t n, const Real* pos0, const Real* vel0, uint32_t nsteps,  \
                             uint32_t ckpt, const Real* seed_x, const Real* seed_v, Real* gx0, Real* gv0, Real* gmu, \
                             Real* gk, Real* pos_final, int threads) {                                             \
        if (!seed_x) return SF_ERR_INVALID_ARGUMENT;                                                               \
        return grad_impl<Real>(p, n, pos0, vel0, nsteps, ckpt, nullptr, 0, nullptr, gx0, gv0, gmu, gk, pos_final,  \
                               threads, seed_x, seed_v);                                                           \
    }
SFO_ADJ(f32, float)
SFO_ADJ(f64, double)

// Render n particles given in the caller's order (index = particle id).
int sfo_render(const sf_params* p, const sf_render_params* rp, uint32_t n, const float* pos3, float* rgba,
               float* depth, uint32_t* owner) {
    if (!p || !rp || !pos3 || rp->width <= 0 || rp->height <= 0) return SF_ERR_INVALID_ARGUMENT;
    const RCo rc = render_const(rp, p->particle_radius);
    const size_t np = (size_t)rc.W * rc.H;
    std::vector<uint64_t> keys(np, ~0ull);
    for (uint32_t i = 0; i < n; ++i) {
        SplatO s;
        if (!splat_o(rc, pos3 + 3 * (size_t)i, s) || !(s.size > 0.f)) continue;
        const int x_lo = std::max((int)std::ceil(s.x0 - 0.5f), 0);
        const int x_hi = std::min((int)std::ceil(s.x0 + s.size - 0.5f) - 1, rc.W - 1);
        const int y_lo = std::max((int)std::ceil(s.y0 - 0.5f), 0);
        const int y_hi = std::min((int)std::ceil(s.y0 + s.size - 0.5f) - 1, rc.H - 1);
        uint32_t db;
        std::memcpy(&db, &s.depth, 4);
        const uint64_t key = ((uint64_t)db << 32) | i;
        for (int row = y_lo; row <= y_hi; ++row)
            for (int px = x_lo; px <= x_hi; ++px) {
                float nx, ny;
                if (disc_o(s, px, row, nx, ny) > 1.0f) continue;
                uint64_t& k = keys[(size_t)row * rc.W + px];
                if (key < k) k = key;
            }
    }
    for (size_t pix = 0; pix < np; ++pix) {
        const uint64_t key = keys[pix];
        float out[4] = {rp->background[0], rp->background[1], rp->background[2], rp->background[3]};
        float dep = 1.0f;
        uint32_t own = 0xffffffffu;
        if (key != ~0ull) {
            const uint32_t id = (uint32_t)(key & 0xffffffffull);
            SplatO s;
            splat_o(rc, pos3 + 3 * (size_t)id, s);
            const int px = (int)(pix % (size_t)rc.W), row = (int)(pix / (size_t)rc.W);
            float nx, ny;
            const float mag = disc_o(s, px, row, nx, ny);
            float surf[3] = {rp->mat_diffuse[0], rp->mat_diffuse[1], rp->mat_diffuse[2]};
            if (rp->color_mode != SF_COLOR_UNIFORM) color_o(rp, id, n, surf);
            shade_o(rp, rc.radius, s.e, nx, ny, mag, surf, out);
            dep = s.depth;
            own = id;
        }
        if (rgba)
            for (int a = 0; a < 4; ++a) rgba[4 * pix + a] = out[a];
        if (depth) depth[pix] = dep;
        if (owner) owner[pix] = own;
    }
    return SF_OK;
}

// The render's camera: the view and projection matrices (column-major), the
// point scale (Source/FluidRenderWidget.cpp:66) and the point radius.
int sfo_render_camera(const sf_params* p, const sf_render_params* rp, float* V16, float* P16, float* scale,
                      float* radius) {
    if (!p || !rp || rp->width <= 0 || rp->height <= 0) return SF_ERR_INVALID_ARGUMENT;
    const RCo rc = render_const(rp, p->particle_radius);
    for (int k = 0; k < 16; ++k) {
        if (V16) V16[k] = rc.V[k];
        if (P16) P16[k] = rc.P[k];
    }
    if (scale) *scale = rc.scale;
    if (radius) *radius = rc.radius;
    return SF_OK;
}

// The vertex stage for n particles: eye-space centres (n x 3), point sizes
// and clip positions (n x 4).
int sfo_particle_vertex(const sf_params* p, const sf_render_params* rp, uint32_t n, const float* pos3, float* eye3,
                        float* size, float* clip4) {
    if (!p || !rp || !pos3 || rp->width <= 0 || rp->height <= 0) return SF_ERR_INVALID_ARGUMENT;
    const RCo rc = render_const(rp, p->particle_radius);
    for (uint32_t i = 0; i < n; ++i) vertex_o(rc, pos3 + 3 * (size_t)i, eye3 + 3 * (size_t)i, size[i], clip4 + 4 * (size_t)i);
    return SF_OK;
}

// The fragment stage for n fragments: sprite centre in eye space (n x 3),
// point coordinate (n x 2) and surface colour (n x 3; NULL = the material's
// diffuse colour).  discarded[k] = 1 where the coordinate falls outside the
// disc (rgba then untouched), else 0 with rgba (n x 4) written.
int sfo_particle_fragment(const sf_params* p, const sf_render_params* rp, uint32_t n, const float* eye3,
                          const float* uv2, const float* color3, float* rgba4, uint8_t* discarded) {
    if (!p || !rp || !eye3 || !uv2 || !rgba4 || !discarded) return SF_ERR_INVALID_ARGUMENT;
    const float radius = rp->point_radius > 0.f ? rp->point_radius : p->particle_radius;
    for (uint32_t k = 0; k < n; ++k) {
        float nx, ny;
        const float mag = coord_normal_o(uv2[2 * (size_t)k], uv2[2 * (size_t)k + 1], nx, ny);
        discarded[k] = mag > 1.0f ? 1 : 0;
        if (discarded[k]) continue;
        const float* surf = color3 ? color3 + 3 * (size_t)k : rp->mat_diffuse;
        shade_o(rp, radius, eye3 + 3 * (size_t)k, nx, ny, mag, surf, rgba4 + 4 * (size_t)k);
    }
    return SF_OK;
}

// The frame loop of Source/Simulator.cpp:46-51: per frame, sub-steps until
// their dt summed in float reach frame_time (or max_substeps were taken).
int sfo_frames_f32(const sf_params* p, uint32_t n, float* pos, float* vel, uint32_t* ids, uint32_t frames,
                   double frame_time, uint32_t max_substeps, int threads, double* sim_time, uint32_t* substeps,
                   float* dts, uint32_t dts_cap) {
    Derived<float> d;
    int st = derive(p, &d);
    if (st) return st;
    if (!pos || !vel || !ids || n == 0 || max_substeps == 0) return SF_ERR_INVALID_ARGUMENT;
    set_threads(threads);
    SubStepper<float> stp(d, n, vel);
    double t = 0.0;
    uint32_t total = 0;
    for (uint32_t f = 0; f < frames; ++f) {
        float acc = 0.0f;
        uint32_t it = 0;
        do {
            stp.step(pos, vel, ids);
            if (dts && total < dts_cap) dts[total] = stp.last_dt;
            acc = acc + stp.last_dt;
            ++it;
            ++total;
        } while ((double)acc < frame_time && it < max_substeps);
        t += (double)acc;  // the frame's time, summed in float
    }
    if (sim_time) *sim_time = t;
    if (substeps) *substeps = total;
    return SF_OK;
}

// The frame accounting of Source/Simulator.cpp:44-56 on a given sequence of
// sub-step sizes: frames of sub-steps whose sizes, summed in float, reach
// frame_time, until the simulated time (the frames' float times summed in
// float) reaches stop_time.  Per frame: the sub-steps taken and the simulated
// time after it.  Returns SF_ERR_CAPACITY if more than cap frames would run
// or the sizes run out.
int sfo_frame_accounting(const float* dts, uint32_t ndts, double frame_time, float stop_time, uint32_t cap,
                         uint32_t* frame_substeps, float* sim_times, uint32_t* nframes) {
    if (!dts || !frame_substeps || !sim_times || !nframes) return SF_ERR_INVALID_ARGUMENT;
    float sim = 0.0f;
    uint32_t next = 0, nf = 0;
    while (sim < stop_time) {
        float acc = 0.0f;
        uint32_t it = 0;
        do {
            if (next >= ndts) return SF_ERR_CAPACITY;
            acc = acc + dts[next++];
            ++it;
        } while ((double)acc < frame_time);
        sim = sim + acc;
        if (nf >= cap) return SF_ERR_CAPACITY;
        frame_substeps[nf] = it;
        sim_times[nf] = sim;
        ++nf;
    }
    *nframes = nf;
    return SF_OK;
}

int sfo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
