// sf_render.h — constants of the headless particle renderer (sf_render.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/sf_capi.h"

namespace sf {

constexpr int kRampColors = 7;  // PARTICLE_COLOR_RAMP, Include/Common.h:31-40

// Everything the two render passes need, computed once on the host.
struct RenderConst {
    float V[16], P[16];  // view and projection matrices, column-major (glm layout)
    float scale;         // u_PointScale = height / tan(fovy / 2)
    float radius;        // u_PointRadius
    int width, height;
    int num_lights;
    float light_position[8][4], light_ambient[8][4], light_diffuse[8][4], light_specular[8][4];
    float mat_ambient[4], mat_diffuse[4], mat_specular[4];
    float mat_shininess;
    int color_mode;
    uint64_t color_seed;
    float ramp[kRampColors][3];
    float ramp_step;  // ramp segments per particle index: (kRampColors - 1) / (n - 1)
    float background[4];
};

// Fill `rc` from the render parameters (matrices in double, rounded).
void build_render_const(const sf_render_params& rp, float particle_radius, uint32_t n, RenderConst* rc);

void launch_render(const float4* pos, uint32_t n, const RenderConst& rc, unsigned long long* keys,
                   uint32_t* slot_of_id, float4* rgba, float* depth, uint32_t* owner, cudaStream_t s);

}  // namespace sf
