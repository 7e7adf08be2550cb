// sf_scenes.cpp — SceneManager of the drop-in: initial particle states.
//
// The four scenes of the reference (SimulationScenes::Scene, Include/Common.h:49-60)
// follow Source/SceneManager.cpp:41-173: lattice spacing 2r, per-axis counts
// int((bMax - bMin) / spacing), loops i (x) -> j (y) -> k (z), positions
// bMin + spacing * (i, j, k) in float, except the second DoubleDambreak block
// which counts down from bMax (:165); SphereDrop keeps points with
// |p - c| <= 0.5 (:83); velocities are zero (:63,90,118,172).  The arithmetic is
// per component in float, like glm's vec3.
//
// The benchmark workloads live in the box [box_min, box_max] of the parameters
// and start at box_min + r (or box_max - r for blocks anchored at the far
// side).  Jittered workloads draw three offsets per particle, in emission
// order, from std::mt19937_64(seed): u = (draw >> 11) * 2^-53,
// offset = float((2u - 1) * 0.1 * spacing).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "sf_internal.h"

namespace sf {
namespace {

using Points = std::vector<float>;

inline void emit(Points& out, float x, float y, float z) {
    out.push_back(x);
    out.push_back(y);
    out.push_back(z);
}

inline int lattice_count(float lo, float hi, float spacing) { return (int)((hi - lo) / spacing); }

// Lattice of counts g[0] x g[1] x g[2] at `origin` stepping by sign[a]*spacing.
template <typename Keep>
void lattice(Points& out, const float origin[3], const int g[3], const float sign[3], float spacing, Keep&& keep) {
    for (int i = 0; i < g[0]; ++i)
        for (int j = 0; j < g[1]; ++j)
            for (int k = 0; k < g[2]; ++k) {
                const float t[3] = {spacing * (float)i, spacing * (float)j, spacing * (float)k};
                float q[3];
                for (int a = 0; a < 3; ++a) q[a] = sign[a] > 0.f ? origin[a] + t[a] : origin[a] - t[a];
                if (keep(q)) emit(out, q[0], q[1], q[2]);
            }
}

const float kUp[3] = {1.f, 1.f, 1.f};
auto keep_all = [](const float*) { return true; };

void reference_box_scene(Points& out, const float bmin[3], const float bmax[3], float spacing) {
    const int g[3] = {lattice_count(bmin[0], bmax[0], spacing), lattice_count(bmin[1], bmax[1], spacing),
                      lattice_count(bmin[2], bmax[2], spacing)};
    lattice(out, bmin, g, kUp, spacing, keep_all);
}

void scene_cube_drop(float r, Points& out) {
    const float bmin[3] = {-0.5f, -0.5f, -0.5f}, bmax[3] = {0.5f, 0.5f, 0.5f};
    reference_box_scene(out, bmin, bmax, 2.0f * r);
}

void scene_sphere_drop(float r, Points& out) {
    const float radius = 0.5f, spacing = 2.0f * r;
    const float bmin[3] = {0.0f - radius, 0.0f - radius, 0.0f - radius};
    const int m = (int)(2.0f * radius / spacing);
    const int g[3] = {m, m, m};
    lattice(out, bmin, g, kUp, spacing, [&](const float* q) {
        const float d0 = q[0] - 0.0f, d1 = q[1] - 0.0f, d2 = q[2] - 0.0f;
        return !(std::sqrt((d0 * d0 + d1 * d1) + d2 * d2) > radius);
    });
}

void scene_dambreak(float r, Points& out) {
    const float bmin[3] = {-1.0f + r, -1.0f + r, -1.0f + r}, bmax[3] = {0.4f, 0.4f, -0.5f};
    reference_box_scene(out, bmin, bmax, 2.0f * r);
}

void scene_double_dambreak(float r, Points& out) {
    scene_dambreak(r, out);
    const float spacing = 2.0f * r;
    const float bmin[3] = {-0.4f + 0.0f, -1.0f + r, 0.5f + 0.0f};
    const float bmax[3] = {1.0f - r, 0.4f - 0.0f, 1.0f - r};
    const int g[3] = {lattice_count(bmin[0], bmax[0], spacing), lattice_count(bmin[1], bmax[1], spacing),
                      lattice_count(bmin[2], bmax[2], spacing)};
    const float down[3] = {-1.f, -1.f, -1.f};
    lattice(out, bmax, g, down, spacing, keep_all);
}

struct JitterSource {
    std::mt19937_64 eng;
    double amp;
    JitterSource(uint64_t seed, float spacing) : eng(seed), amp(0.1 * (double)spacing) {}
    float operator()() {
        const double u = (double)(eng() >> 11) * (1.0 / 9007199254740992.0);
        return (float)((2.0 * u - 1.0) * amp);
    }
};

// Benchmark block anchored at box_min + r (sign +1) or box_max - r (sign -1).
void anchored_block(const sf_params& p, const int g[3], const float sign[3], JitterSource* jit, Points& out) {
    const float r = p.particle_radius, spacing = 2.0f * r;
    float origin[3];
    for (int a = 0; a < 3; ++a) origin[a] = sign[a] > 0.f ? p.box_min[a] + r : p.box_max[a] - r;
    const size_t first = out.size();
    lattice(out, origin, g, sign, spacing, keep_all);
    if (jit)
        for (size_t t = first; t < out.size(); ++t) out[t] = out[t] + (*jit)();
}

void scene_sphere_pool(const sf_params& p, uint64_t seed, Points& out) {
    const float r = p.particle_radius, spacing = 2.0f * r;
    JitterSource jit(seed, spacing);
    const int g[3] = {(int)(((double)p.box_max[0] - p.box_min[0]) / spacing), (int)(0.3 / (double)spacing),
                      (int)(((double)p.box_max[2] - p.box_min[2]) / spacing)};
    anchored_block(p, g, kUp, &jit, out);
    const float R = 0.15f;
    const float c[3] = {0.5f * (p.box_min[0] + p.box_max[0]), p.box_min[1] + 0.6f, 0.5f * (p.box_min[2] + p.box_max[2])};
    const int m = (int)(2.0f * R / spacing);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            for (int k = 0; k < m; ++k) {
                const float q[3] = {(c[0] - R) + spacing * ((float)i + 0.5f), (c[1] - R) + spacing * ((float)j + 0.5f),
                                    (c[2] - R) + spacing * ((float)k + 0.5f)};
                const float d0 = q[0] - c[0], d1 = q[1] - c[1], d2 = q[2] - c[2];
                if ((d0 * d0 + d1 * d1) + d2 * d2 > R * R) continue;
                const float a = jit(), b = jit(), e = jit();
                emit(out, q[0] + a, q[1] + b, q[2] + e);
            }
}

int build_scene(const sf_params& p, int scene, uint64_t seed, Points& out, const char** why) {
    out.clear();
    const float r = p.particle_radius;
    if (!(r > 0.f) || !std::isfinite(r)) {
        *why = "particle_radius must be positive";
        return SF_ERR_INVALID_ARGUMENT;
    }
    switch (scene) {
        case SF_SCENE_CUBE_DROP: scene_cube_drop(r, out); break;
        case SF_SCENE_SPHERE_DROP: scene_sphere_drop(r, out); break;
        case SF_SCENE_DAMBREAK: scene_dambreak(r, out); break;
        case SF_SCENE_DOUBLE_DAMBREAK: scene_double_dambreak(r, out); break;
        case SF_SCENE_DAMBREAK_16K: {
            const int g[3] = {20, 40, 20};
            anchored_block(p, g, kUp, nullptr, out);
            break;
        }
        case SF_SCENE_DAMBREAK_64K: {
            const int g[3] = {32, 64, 32};
            anchored_block(p, g, kUp, nullptr, out);
            break;
        }
        case SF_SCENE_DOUBLE_DAMBREAK_1M: {
            JitterSource jit(seed, 2.0f * r);
            const int g[3] = {64, 128, 64};
            const float far[3] = {-1.f, 1.f, -1.f};
            anchored_block(p, g, kUp, &jit, out);
            anchored_block(p, g, far, &jit, out);
            break;
        }
        case SF_SCENE_SPHERE_POOL: scene_sphere_pool(p, seed, out); break;
        default: *why = "unknown scene id"; return SF_ERR_INVALID_ARGUMENT;
    }
    if (out.size() / 3 > 0xffffffffull) {
        *why = "scene has more than 2^32-1 particles";
        return SF_ERR_CAPACITY;
    }
    return SF_OK;
}

}  // namespace

// Batched cube workload: scene s draws, in order from std::mt19937_64(seed),
// u_n, u_mu, u_k (each (draw >> 11) * 2^-53): particle count
// N_s = round(exp(ln 2000 + u_n (ln 65536 - ln 2000))) clamped to [2000, 65536],
// viscosity 0.005 + 0.045 u_mu, stiffness 20 + 80 u_k.  The scene is a lattice
// of spacing 2r with m = ceil(cbrt(N_s)) points per side (x outer, z inner; the
// first N_s points), anchored at m*r + r so the block sits centred in its box
// [0, 4 m r]^3, and drops under gravity.  Other parameters come from `base`.
int batch_cubes(uint64_t seed, uint32_t nscenes, const sf_params& base, std::vector<sf_params>& params,
                std::vector<uint32_t>& counts, std::vector<float>& pos, const char** why) {
    if (!(base.particle_radius > 0.f)) {
        *why = "particle_radius must be positive";
        return SF_ERR_INVALID_ARGUMENT;
    }
    std::mt19937_64 eng(seed);
    auto uni = [&eng]() { return (double)(eng() >> 11) * (1.0 / 9007199254740992.0); };
    params.assign(nscenes, base);
    counts.assign(nscenes, 0);
    pos.clear();
    const float r = base.particle_radius, spacing = 2.0f * r;
    for (uint32_t s = 0; s < nscenes; ++s) {
        const double un = uni(), umu = uni(), uk = uni();
        double nd = std::exp(std::log(2000.0) + un * (std::log(65536.0) - std::log(2000.0)));
        uint32_t n = (uint32_t)std::llround(nd);
        n = n < 2000 ? 2000 : (n > 65536 ? 65536 : n);
        uint32_t m = 1;
        while ((uint64_t)m * m * m < n) ++m;
        sf_params& p = params[s];
        p.viscosity = (float)(0.005 + 0.045 * umu);
        p.pressure_stiffness = (float)(20.0 + 80.0 * uk);
        p.scene = SF_SCENE_CUBE_DROP;
        const float ext = 4.0f * (float)m * r;
        for (int a = 0; a < 3; ++a) {
            p.box_min[a] = 0.0f;
            p.box_max[a] = ext;
        }
        const float origin = (float)m * r + r;
        uint32_t emitted = 0;
        for (uint32_t i = 0; i < m && emitted < n; ++i)
            for (uint32_t j = 0; j < m && emitted < n; ++j)
                for (uint32_t k = 0; k < m && emitted < n; ++k, ++emitted)
                    emit(pos, origin + spacing * (float)i, origin + spacing * (float)j, origin + spacing * (float)k);
        counts[s] = n;
    }
    return SF_OK;
}

int scene_points(const sf_params& p, int scene, uint64_t seed, std::vector<float>& out, const char** why) {
    return build_scene(p, scene, seed, out, why);
}

}  // namespace sf
