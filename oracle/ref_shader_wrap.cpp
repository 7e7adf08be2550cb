// C entry points around the reference's own particle shaders
// (Shaders/particle.vs.glsl, particle.fs.glsl), compiled as C++ by
// build_ref.sh: each shader's text, with its qualifiers and uniform-block
// wrappers taken out, is included inside a struct, so that its uniforms,
// inputs and outputs are members the entry points set and read, and `discard`
// returns from main() with a flag set.  TEST INFRASTRUCTURE ONLY: it pins the
// oracle's restatement of the shader arithmetic against the reference.
#include <cstdint>
#include <cstring>

#include "glsl.h"

using namespace glsl;

#define discard              \
    {                        \
        discarded = true;    \
        return;              \
    }

struct ParticleVS : Builtins {
#include "particle_vs.inc"
};

struct ParticleFS : Builtins {
#include "particle_fs.inc"
};

#undef discard

namespace {
void set_mat(mat4& m, const float* a) {  // 16 floats, column-major
    for (int c = 0; c < 4; ++c) m.c[c] = vec4(a[4 * c], a[4 * c + 1], a[4 * c + 2], a[4 * c + 3]);
}
}  // namespace

// Vertex stage: view (V) and projection (P) matrices, column-major; outputs
// the eye-space centre, the point size and the clip position.
extern "C" void ref_particle_vs(const float* V, const float* P, float point_radius, float point_scale,
                                const float* position, float* view_center, float* point_size, float* clip) {
    ParticleVS s;
    set_mat(s.viewMatrix, V);
    set_mat(s.projectionMatrix, P);
    s.u_PointRadius = point_radius;
    s.u_PointScale = point_scale;
    s.v_Position = vec3(position[0], position[1], position[2]);
    s.v_Color = vec3(0.f, 0.f, 0.f);
    s.main();
    view_center[0] = s.f_ViewCenter.x;
    view_center[1] = s.f_ViewCenter.y;
    view_center[2] = s.f_ViewCenter.z;
    *point_size = s.gl_PointSize;
    clip[0] = s.gl_Position.x;
    clip[1] = s.gl_Position.y;
    clip[2] = s.gl_Position.z;
    clip[3] = s.gl_Position.w;
}

// Fragment stage.  lights: num_lights x (ambient, diffuse, specular, position)
// as 16 floats each; material: ambient, diffuse, specular (4 floats each) and
// shininess.  Returns 1 if the fragment is discarded, else 0 with rgba set.
extern "C" int ref_particle_fs(const float* lights, int num_lights, const float* material, float point_radius,
                               int has_vcolor, const float* color, const float* view_center, const float* point_coord,
                               float* rgba) {
    ParticleFS s;
    for (int l = 0; l < num_lights && l < 8; ++l) {
        const float* L = lights + 16 * l;
        s.lights[l].ambient = vec4(L[0], L[1], L[2], L[3]);
        s.lights[l].diffuse = vec4(L[4], L[5], L[6], L[7]);
        s.lights[l].specular = vec4(L[8], L[9], L[10], L[11]);
        s.lights[l].position = vec4(L[12], L[13], L[14], L[15]);
    }
    s.u_NumLights = num_lights;
    s.material.ambient = vec4(material[0], material[1], material[2], material[3]);
    s.material.diffuse = vec4(material[4], material[5], material[6], material[7]);
    s.material.specular = vec4(material[8], material[9], material[10], material[11]);
    s.material.shininess = material[12];
    s.u_HasVColor = has_vcolor;
    s.u_PointRadius = point_radius;
    s.f_Color = vec3(color[0], color[1], color[2]);
    s.f_ViewCenter = vec3(view_center[0], view_center[1], view_center[2]);
    s.gl_PointCoord = vec2(point_coord[0], point_coord[1]);
    s.main();
    if (s.discarded) return 1;
    rgba[0] = s.outColor.x;
    rgba[1] = s.outColor.y;
    rgba[2] = s.outColor.z;
    rgba[3] = s.outColor.w;
    return 0;
}
