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
    int eos, attractive, reach;
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
                const Real* inv_rho, const std::vector<uint32_t>& cs, Real* acc) {
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
        }
    }
}

template <typename Real>
void integrate_pass(const Derived<Real>& d, uint32_t n, Real* pos, Real* vel, const Real* acc) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        for (int a = 0; a < 3; ++a) {
            Real v = std::fma(d.dt, acc[3 * i + a], vel[3 * i + a]);
            Real x = std::fma(d.dt, v, pos[3 * i + a]);
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

template <typename Real>
int step_impl(const sf_params* p, uint32_t n, Real* pos, Real* vel, uint32_t* ids, uint32_t nsteps,
              int threads) {
    Derived<Real> d;
    int st = derive(p, &d);
    if (st) return st;
    if (n == 0) return SF_OK;
    if (!pos || !vel || !ids) return SF_ERR_INVALID_ARGUMENT;
    set_threads(threads);
    std::vector<uint32_t> keys, cs;
    std::vector<Real> prs(n), inv_rho(n), acc(3 * (size_t)n);
    for (uint32_t s = 0; s < nsteps; ++s) {
        sort_and_grid(d, n, pos, vel, ids, keys, cs);
        density_pass(d, n, pos, cs, (Real*)nullptr, prs.data(), inv_rho.data());
        accel_pass(d, n, pos, vel, prs.data(), inv_rho.data(), cs, acc.data());
        integrate_pass(d, n, pos, vel, acc.data());
    }
    return SF_OK;
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
        integrate_pass(d, n, pos, vel, acc);                                                                \
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

int sfo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
