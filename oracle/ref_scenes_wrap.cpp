// C entry point around the reference's own SceneManager (compiled from the
// reference source by build_ref.sh).  TEST INFRASTRUCTURE ONLY: used to pin
// the scene generators of the oracle and of the product against the reference.
#include <cstdint>
#include <cstring>
#include <memory>
#include "SceneManager.h"

extern "C" int ref_setup_scene(int scene, float particle_radius, float* pos3, uint32_t cap, uint32_t* n_out) {
    auto params = std::make_shared<SPHParameters<float> >();
    params->particleRadius = particle_radius;
    params->scene = scene;
    SceneManager mgr(params);
    Vec_Vec3<float> particles, velocity;
    mgr.setupScene(particles, velocity);
    const uint32_t n = (uint32_t)particles.size();
    if (n_out) *n_out = n;
    if (velocity.size() != particles.size()) return 2;
    for (const auto& v : velocity)
        if (v[0] != 0.0f || v[1] != 0.0f || v[2] != 0.0f) return 3;
    if (!pos3) return 0;
    if (cap < n) return 1;
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) pos3[3 * i + a] = particles[i][a];
    return 0;
}
