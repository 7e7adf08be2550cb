// sf_render.cu — headless sphere-impostor rendering of the particles
// (sm_103a), the arithmetic of the reference's point-sprite shaders without a
// graphics API:
//   Shaders/particle.vs.glsl:24-35  eye-space position, point size
//                                   radius * (scale / |eye|), clip position;
//   Shaders/particle.fs.glsl:46-83  gl_PointCoord -> normal.xy, disc test
//                                   (discard outside), normal.z, fragment
//                                   position, Blinn-Phong over the lights.
// Two passes: every particle splats its disc into a per-pixel 64-bit key
// (window depth of its centre, particle index) with atomicMin, which is the
// depth test of point sprites without depth correction with ties broken by
// index, independent of arrival order; then every pixel shades its winner.
// The CPU oracle (oracle/sph_oracle.cpp, render_impl) restates both passes.
#include "sf_device.cuh"
#include "sf_render.h"

namespace sf {
namespace {

__device__ __forceinline__ void eye_of(const RenderConst& rc, float x, float y, float z, float e[3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r) e[r] = ((rc.V[r] * x + rc.V[4 + r] * y) + rc.V[8 + r] * z) + rc.V[12 + r];
}

// Screen footprint of a particle; false when its centre is clipped.
struct Splat {
    float e[3];       // eye-space centre
    float x0, y0;     // top-left corner of the sprite square (pixels, rows down)
    float size;       // sprite edge (pixels)
    float depth;      // window depth of the centre
};

__device__ __forceinline__ bool splat_of(const RenderConst& rc, float x, float y, float z, Splat& s) {
    eye_of(rc, x, y, z, s.e);
    const float dist = sqrtf((s.e[0] * s.e[0] + s.e[1] * s.e[1]) + s.e[2] * s.e[2]);
    s.size = rc.radius * (rc.scale / dist);
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        c[r] = ((rc.P[r] * s.e[0] + rc.P[4 + r] * s.e[1]) + rc.P[8 + r] * s.e[2]) + rc.P[12 + r];
    if (!(c[3] > 0.f)) return false;
    if (c[0] < -c[3] || c[0] > c[3] || c[1] < -c[3] || c[1] > c[3] || c[2] < -c[3] || c[2] > c[3]) return false;
    const float nx = c[0] / c[3], ny = c[1] / c[3], nz = c[2] / c[3];
    const float wx = (nx * 0.5f + 0.5f) * (float)rc.width;
    const float wy = (ny * 0.5f + 0.5f) * (float)rc.height;
    s.depth = nz * 0.5f + 0.5f;
    s.x0 = wx - s.size * 0.5f;
    s.y0 = ((float)rc.height - wy) - s.size * 0.5f;
    return true;
}

// gl_PointCoord of pixel (px, row) -> impostor normal.xy and its squared length.
__device__ __forceinline__ float disc_of(const Splat& s, int px, int row, float& nx, float& ny) {
    const float u = (((float)px + 0.5f) - s.x0) / s.size;
    const float v = (((float)row + 0.5f) - s.y0) / s.size;
    nx = u * 2.0f + -1.0f;
    ny = v * -2.0f + 1.0f;
    return nx * nx + ny * ny;
}

__global__ void k_splat(const float4* __restrict__ pos, uint32_t n, RenderConst rc,
                        unsigned long long* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    Splat s;
    if (!splat_of(rc, p.x, p.y, p.z, s)) return;
    if (!(s.size > 0.f)) return;
    const int x_lo = max((int)ceilf(s.x0 - 0.5f), 0);
    const int x_hi = min((int)ceilf(s.x0 + s.size - 0.5f) - 1, rc.width - 1);
    const int y_lo = max((int)ceilf(s.y0 - 0.5f), 0);
    const int y_hi = min((int)ceilf(s.y0 + s.size - 0.5f) - 1, rc.height - 1);
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(s.depth) << 32) | (unsigned long long)__float_as_uint(p.w);
    for (int row = y_lo; row <= y_hi; ++row)
        for (int px = x_lo; px <= x_hi; ++px) {
            float nx, ny;
            if (disc_of(s, px, row, nx, ny) > 1.0f) continue;
            atomicMin(keys + (size_t)row * rc.width + px, key);
        }
}

__device__ __forceinline__ void normalize3(float v[3]) {
    const float len = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    v[0] = v[0] / len;
    v[1] = v[1] / len;
    v[2] = v[2] / len;
}

__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// Colour of particle `id` (caller index) in the random and ramp modes.
__device__ __forceinline__ void particle_color(const RenderConst& rc, uint32_t id, float col[3]) {
    if (rc.color_mode == SF_COLOR_RANDOM) {
        uint64_t z = rc.color_seed ^ ((uint64_t)id * 0x9E3779B97F4A7C15ull);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t q = z;
            q = (q ^ (q >> 30)) * 0xBF58476D1CE4E5B9ull;
            q = (q ^ (q >> 27)) * 0x94D049BB133111EBull;
            q ^= q >> 31;
            col[a] = (float)(q >> 40) * (1.0f / 16777216.0f);
        }
    } else {
        const float t = (float)id * rc.ramp_step;
        int k = (int)floorf(t);
        k = k < 0 ? 0 : (k > kRampColors - 2 ? kRampColors - 2 : k);
        const float f = t - (float)k;
#pragma unroll
        for (int a = 0; a < 3; ++a) col[a] = fmaf(f, rc.ramp[k + 1][a] - rc.ramp[k][a], rc.ramp[k][a]);
    }
}

__global__ void k_shade(const float4* __restrict__ pos, const unsigned long long* __restrict__ keys,
                        const uint32_t* __restrict__ slot_of_id, RenderConst rc, float4* __restrict__ rgba,
                        float* __restrict__ depth, uint32_t* __restrict__ owner) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (uint32_t)(rc.width * rc.height)) return;
    const unsigned long long key = keys[pix];
    if (key == ~0ull) {
        rgba[pix] = make_float4(rc.background[0], rc.background[1], rc.background[2], rc.background[3]);
        depth[pix] = 1.0f;
        owner[pix] = 0xffffffffu;
        return;
    }
    const uint32_t id = (uint32_t)(key & 0xffffffffull);
    const float4 p = pos[slot_of_id[id]];
    Splat s;
    splat_of(rc, p.x, p.y, p.z, s);
    const int px = (int)(pix % (uint32_t)rc.width), row = (int)(pix / (uint32_t)rc.width);
    float nrm[3];
    const float mag = disc_of(s, px, row, nrm[0], nrm[1]);
    nrm[2] = sqrtf(1.0f - mag);
    float view[3] = {s.e[0], s.e[1], s.e[2]};
    normalize3(view);
    const float frag[3] = {s.e[0] + nrm[0] * rc.radius, s.e[1] + nrm[1] * rc.radius, s.e[2] + nrm[2] * rc.radius};
    float surf[3] = {rc.mat_diffuse[0], rc.mat_diffuse[1], rc.mat_diffuse[2]};
    if (rc.color_mode != SF_COLOR_UNIFORM) particle_color(rc, id, surf);
    float shade[3] = {0.f, 0.f, 0.f};
    for (int l = 0; l < rc.num_lights; ++l) {
        float ld[3] = {rc.light_position[l][0] - frag[0], rc.light_position[l][1] - frag[1],
                       rc.light_position[l][2] - frag[2]};
        normalize3(ld);
        float hd[3] = {ld[0] - view[0], ld[1] - view[1], ld[2] - view[2]};
        normalize3(hd);
        const float diff = fmaxf(dot3(nrm, ld), 0.f);
        const float spec = powf(fmaxf(dot3(hd, nrm), 0.f), rc.mat_shininess);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float amb = rc.light_ambient[l][a] * rc.mat_ambient[a];
            const float dif = (rc.light_diffuse[l][a] * diff) * surf[a];
            const float spc = (rc.light_specular[l][a] * spec) * rc.mat_specular[a];
            shade[a] += (amb + dif) + spc;
        }
    }
    rgba[pix] = make_float4(shade[0], shade[1], shade[2], 1.0f);
    depth[pix] = s.depth;
    owner[pix] = id;
}

__global__ void k_slot_of_id(const float4* __restrict__ pos, uint32_t n, uint32_t* __restrict__ slot_of_id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(pos[i].w);
    if (id < n) slot_of_id[id] = i;
}

}  // namespace

void launch_render(const float4* pos, uint32_t n, const RenderConst& rc, unsigned long long* keys,
                   uint32_t* slot_of_id, float4* rgba, float* depth, uint32_t* owner, cudaStream_t s) {
    const uint32_t npix = (uint32_t)rc.width * (uint32_t)rc.height;
    cudaMemsetAsync(keys, 0xff, (size_t)npix * sizeof(unsigned long long), s);
    if (n) {
        k_slot_of_id<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, slot_of_id);
        k_splat<<<grid_for(n, kBlock), kBlock, 0, s>>>(pos, n, rc, keys);
    }
    k_shade<<<grid_for(npix, kBlock), kBlock, 0, s>>>(pos, keys, slot_of_id, rc, rgba, depth, owner);
}

}  // namespace sf
