// sf_noalloc.cu — density of caller-owned device positions with no device
// allocation: the uniform-grid sort works in a fixed scratch array compiled
// into this library.
//
// Who needs this: code that may not allocate device memory while it runs —
// a host application that owns a fixed device-memory budget (a renderer or a
// game engine embedding the fluid, a plugin inside another framework's memory
// pool), or a real-time loop where an allocation could block or fail.  Such a
// caller hands in its own position and output buffers; everything else this
// computation needs lives in g_sf_noalloc_scratch below.
//
// Scratch: one static __device__ array of kNoAllocScratchBytes (about 7.6 MB).
// Every GPU that loads this library holds it until the process exits.  It caps
// a call at kNoAllocMaxParticles particles and kNoAllocMaxCells grid cells;
// larger requests are rejected with SF_ERR_CAPACITY before any GPU work.
//
// Sharing: all calls on a device use the same scratch, which keeps the last
// call's contents.  The cell counters are cleared on every call.  Two calls
// whose GPU work overlaps (different streams, or different host threads
// without ordering) race on the scratch and produce garbage; serialise them on
// one stream.
//
// Set-up: the first call on a device looks up the scratch's device address
// with cudaGetSymbolAddress (with that device current) and caches it with the
// CUDA context that was current; make that first call before any stream
// capture.  The address belongs to that context: a call made under another
// context (after cudaDeviceReset, or with a driver-API context made current on
// the same device) repeats the set-up for it.
#include <cstdint>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "sf_internal.h"

namespace sf {
namespace {

constexpr uint32_t kNoAllocMaxParticles = 65536;
constexpr uint32_t kNoAllocMaxCells = 262144;  // e.g. a 64^3 grid
constexpr uint64_t kNoAllocCellsPad =
    ((uint64_t)kNoAllocMaxCells + 1 + kScanTile - 1) / kScanTile * kScanTile;
constexpr uint64_t kNoAllocTiles = kNoAllocCellsPad / kScanTile;

constexpr uint64_t align256(uint64_t x) { return (x + 255) / 256 * 256; }

// Byte offsets of each region inside the scratch array.
constexpr uint64_t kOffPos = 0;
constexpr uint64_t kOffVel = kOffPos + align256(16ull * kNoAllocMaxParticles);
constexpr uint64_t kOffPos2 = kOffVel + align256(16ull * kNoAllocMaxParticles);
constexpr uint64_t kOffVel2 = kOffPos2 + align256(16ull * kNoAllocMaxParticles);
constexpr uint64_t kOffPr = kOffVel2 + align256(16ull * kNoAllocMaxParticles);
constexpr uint64_t kOffRho = kOffPr + align256(8ull * kNoAllocMaxParticles);
constexpr uint64_t kOffKeySlot = kOffRho + align256(4ull * kNoAllocMaxParticles);
constexpr uint64_t kOffTmp = kOffKeySlot + align256(8ull * kNoAllocMaxParticles);
constexpr uint64_t kOffCounts = kOffTmp + align256(4ull * kNoAllocMaxParticles);
constexpr uint64_t kOffCellStart = kOffCounts + align256(4ull * kNoAllocCellsPad);
constexpr uint64_t kOffTileSums = kOffCellStart + align256(4ull * kNoAllocCellsPad);
constexpr uint64_t kNoAllocScratchBytes = kOffTileSums + align256(4ull * kNoAllocTiles);

static __device__ __align__(256) unsigned char g_sf_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
// Per device: the context the cached address was looked up in, and the address.
struct ScratchAddr {
    std::mutex m;
    CUcontext ctx = nullptr;
    unsigned char* addr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];

// The calling thread's current CUDA context (through the driver entry point
// the runtime hands out, so the library needs no link to the driver library).
cudaError_t current_context(CUcontext* out) {
    using GetCurrent = CUresult (*)(CUcontext*);
    static GetCurrent fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<GetCurrent>(p);
        else
            cudaGetLastError();
    });
    if (!fn) return cudaErrorNotSupported;
    return fn(out) == CUDA_SUCCESS ? cudaSuccess : cudaErrorDeviceUninitialized;
}

__global__ void k_density_to_caller_order(const float4* __restrict__ pos_sorted, const float* __restrict__ rho,
                                          const float2* __restrict__ pr, uint32_t n, float* __restrict__ out_rho,
                                          float* __restrict__ out_p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(pos_sorted[i].w);
    if (id >= n) return;
    if (out_rho) out_rho[id] = rho[i];
    if (out_p) out_p[id] = pr[i].x;
}

}  // namespace

// Device address of this device's scratch in the current context (looked up
// once per device and context).
static cudaError_t noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    CUcontext ctx = nullptr;
    e = current_context(&ctx);
    if (e != cudaSuccess) return e;
    ScratchAddr& s = g_scratch_addr[dev];
    std::lock_guard<std::mutex> lock(s.m);
    if (!ctx || !s.addr || s.ctx != ctx) {
        // the look-up also brings up the runtime's context when none is current
        void* addr = nullptr;
        e = cudaGetSymbolAddress(&addr, g_sf_noalloc_scratch);
        if (e != cudaSuccess) return e;
        e = current_context(&ctx);
        if (e != cudaSuccess) return e;
        s.addr = static_cast<unsigned char*>(addr);
        s.ctx = ctx;
    }
    *out = s.addr;
    return cudaSuccess;
}

int noalloc_density(const sf_params& p, const SimConst& c, const float* d_pos_xyz, uint32_t n, float* d_rho,
                    float* d_pressure, cudaStream_t stream, const char** why) {
    if (n > kNoAllocMaxParticles) {
        *why = "sf_density_noalloc: more than 65536 particles (the fixed scratch limit)";
        return SF_ERR_CAPACITY;
    }
    if (c.ncells > kNoAllocMaxCells) {
        *why = "sf_density_noalloc: grid has more than 262144 cells (the fixed scratch limit)";
        return SF_ERR_CAPACITY;
    }
    (void)p;
    if (n == 0) return SF_OK;
    unsigned char* base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) {
        *why = "sf_density_noalloc: cudaGetSymbolAddress of the scratch array failed";
        return SF_ERR_CUDA;
    }
    DeviceState d;
    d.n = n;
    d.cap = kNoAllocMaxParticles;
    d.pos = reinterpret_cast<float4*>(base + kOffPos);
    d.vel = reinterpret_cast<float4*>(base + kOffVel);
    d.pos2 = reinterpret_cast<float4*>(base + kOffPos2);
    d.vel2 = reinterpret_cast<float4*>(base + kOffVel2);
    d.pr = reinterpret_cast<float2*>(base + kOffPr);
    d.rho = reinterpret_cast<float*>(base + kOffRho);
    d.key_slot = reinterpret_cast<uint2*>(base + kOffKeySlot);
    d.tmp = reinterpret_cast<uint32_t*>(base + kOffTmp);
    d.counts = reinterpret_cast<uint32_t*>(base + kOffCounts);
    d.cell_start = reinterpret_cast<uint32_t*>(base + kOffCellStart);
    d.tile_sums = reinterpret_cast<uint32_t*>(base + kOffTileSums);
    d.ncells = c.ncells;
    d.ncells_pad = (uint32_t)(((uint64_t)c.ncells + 1 + kScanTile - 1) / kScanTile * kScanTile);
    d.ntiles = d.ncells_pad / kScanTile;
    // The counters (per cell and per scan tile) must start at zero; a previous
    // call normally leaves them zero, but an interrupted one may not.
    e = cudaMemsetAsync(d.counts, 0, (size_t)d.ncells_pad * sizeof(uint32_t), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.tile_sums, 0, (size_t)d.ntiles * sizeof(uint32_t), stream);
    if (e != cudaSuccess) {
        *why = "sf_density_noalloc: clearing the cell counters failed";
        return SF_ERR_CUDA;
    }
    launch_load_aos(d_pos_xyz, nullptr, n, d.pos2, d.vel2, stream);
    launch_hash_count(d, d.pos2, n, c, d.counts, d.key_slot, stream);
    enqueue_sort_tail(d, stream);
    launch_density(d, c, stream);
    k_density_to_caller_order<<<(n + 255) / 256, 256, 0, stream>>>(d.pos, d.rho, d.pr, n, d_rho, d_pressure);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        *why = "sf_density_noalloc: kernel launch failed";
        return SF_ERR_CUDA;
    }
    return SF_OK;
}

}  // namespace sf
