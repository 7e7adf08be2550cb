// sf_frame.cu — sub-step control on the device: the adaptive (CFL) sub-step
// and the frame loop of Source/Simulator.cpp:46-51 ("while frameTime < 1/30:
// frameTime += advanceFrame()") as the body of a CUDA-graph conditional while
// node, so a whole frame is one graph launch with no host round trip.
//
// Adaptive sub-step: dt = min(time_step, 0.4 h / max|v|, 0.25 sqrt(h / max|a|))
// with both maxima taken over the previous sub-step (|v| after integration),
// which keeps forces and integration in one fused pass.  The density pass's
// first thread chooses dt (choose_dt in sf_device.cuh) before the force pass
// reads it.  The CPU oracle restates the same rule.
#include "sf_device.cuh"

namespace sf {
namespace {

// max |v|^2 of the state (non-negative floats order like their bits): one
// atomic per block of kMaxBlock threads.
constexpr uint32_t kMaxBlock = 1024;

__global__ void __launch_bounds__(kMaxBlock)
    k_init_maxima(const float4* __restrict__ vel, uint32_t n, FrameState* __restrict__ fs) {
    __shared__ uint32_t s_max[kMaxBlock / 32];
    const uint32_t i = blockIdx.x * kMaxBlock + threadIdx.x;
    uint32_t v2 = 0u;
    if (i < n) {
        const float4 v = vel[i];
        v2 = __float_as_uint(fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
    }
    v2 = __reduce_max_sync(0xffffffffu, v2);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x / 32] = v2;
    __syncthreads();
    if (threadIdx.x < 32) {
        const uint32_t m = __reduce_max_sync(0xffffffffu, s_max[threadIdx.x]);
        if (threadIdx.x == 0) atomicMax(&fs->v2max_bits, m);
    }
}

__global__ void k_frame_begin(FrameState* __restrict__ fs) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    fs->frame_acc = 0.f;
    fs->iter = 0u;
}

__global__ void k_frame_check(FrameState* __restrict__ fs, double frame_time, uint32_t max_substeps,
                              cudaGraphConditionalHandle h) {
    grid_dependency_wait();
    allow_dependents();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float dt = fs->dt;
    fs->frame_acc = fs->frame_acc + dt;
    fs->iter += 1u;
    fs->substeps += 1u;
    const bool more = (double)fs->frame_acc < frame_time && fs->iter < max_substeps;
    // a finished frame adds its time, summed in float as the reference's
    // frameTime is (Source/Simulator.cpp:46-50)
    if (!more) fs->sim_time += (double)fs->frame_acc;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

}  // namespace

void launch_init_maxima(const float4* vel, uint32_t n, FrameState* fs, cudaStream_t s) {
    cudaMemsetAsync(&fs->v2max_bits, 0, 2 * sizeof(uint32_t), s);
    if (n) k_init_maxima<<<grid_for(n, kMaxBlock), kMaxBlock, 0, s>>>(vel, n, fs);
}

void launch_frame_begin(FrameState* fs, cudaStream_t s) { k_frame_begin<<<1, 32, 0, s>>>(fs); }

void launch_frame_check(FrameState* fs, double frame_time, uint32_t max_substeps, cudaGraphConditionalHandle h,
                        cudaStream_t s) {
    launch_chained(k_frame_check, 1, 32, s, fs, frame_time, max_substeps, h);
}

}  // namespace sf
