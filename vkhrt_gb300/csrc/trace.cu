// trace.cu -- the trace pass's host entry points: frame launches (kernels in trace_frames.cu),
// closest hit for explicit rays, and the no-allocation variant with its static scratch.
#include <mutex>

#define HRT_RAY_KERNEL
#include "trace_device.cuh"

namespace hrt {

// trace_frames.cu, compiled once per node mode: the frame kernels and their attributes (set once
// per context)
cudaError_t launch_frames_f(const TraceLaunch& L, cudaStream_t s, int sm_count);
cudaError_t launch_frames_q(const TraceLaunch& L, cudaStream_t s, int sm_count);
cudaError_t launch_frames_m(const TraceLaunch& L, cudaStream_t s, int sm_count);
cudaError_t prepare_frames_f();
cudaError_t prepare_frames_q();
cudaError_t prepare_frames_m();
cudaError_t prepare_frames() {
    cudaError_t e = prepare_frames_f();
    if (e == cudaSuccess) e = prepare_frames_q();
    return e == cudaSuccess ? prepare_frames_m() : e;
}

cudaError_t launch_trace(const TraceLaunch& L, int node_mode, cudaStream_t s, int sm_count) {
    switch (node_mode) {
        case kNodesQ: return launch_frames_q(L, s, sm_count);
        case kNodesPerInstance: return launch_frames_m(L, s, sm_count);
        default: return launch_frames_f(L, s, sm_count);
    }
}

cudaError_t launch_trace_rays(const DevInstance* inst, const TlasNode* tlas, uint32_t ninst, const float* rays,
                              uint64_t n, float tmin, float tmax, uint32_t fp64_resolve, RayBounds bounds,
                              hrt_hit* hits, TraceCounters* counters, cudaStream_t s, int sm_count) {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + kThreads - 1) / kThreads;
    unsigned grid = unsigned(blocks < uint64_t(sm_count) * 16 ? blocks : uint64_t(sm_count) * 16);
    trace_rays_kernel<<<grid, kThreads, 0, s>>>(inst, tlas, ninst, rays, n, tmin, tmax, fp64_resolve, bounds, hits,
                                                counters);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- no-allocation closest hit
// Scratch of hrt_trace_rays_noalloc: counters (error word, statistics), then the device
// staging of up to HRT_NOALLOC_MAX_RAYS rays (24 B each) and hits (16 B each).
namespace {
constexpr size_t kNoAllocRays = HRT_NOALLOC_MAX_RAYS;
constexpr size_t kNoAllocRayOff = 256;
constexpr size_t kNoAllocHitOff = kNoAllocRayOff + kNoAllocRays * 24;
static_assert(sizeof(TraceCounters) <= kNoAllocRayOff, "counters fit the header");
static_assert(kNoAllocHitOff + kNoAllocRays * sizeof(hrt_hit) == HRT_NOALLOC_SCRATCH_BYTES, "scratch size");
static __device__ __align__(256) unsigned char g_noalloc_scratch[HRT_NOALLOC_SCRATCH_BYTES];
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices];  // device address of g_noalloc_scratch per device (null until set up)
}  // namespace

cudaError_t trace_rays_noalloc(int device, const DevInstance* inst, const TlasNode* tlas, uint32_t ninst,
                               const float* host_rays, uint64_t n, float tmin, float tmax, uint32_t fp64_resolve,
                               RayBounds bounds, hrt_hit* host_hits, cudaStream_t s, int sm_count,
                               uint32_t* error_word) {
    *error_word = 0;
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    void* base = nullptr;
    {
        // set-up once per device, with that device current: the symbol's device address
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[device]) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return e;
            g_noalloc_ptr[device] = ptr;
        }
        base = g_noalloc_ptr[device];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    TraceCounters* ctr = reinterpret_cast<TraceCounters*>(b);
    float* drays = reinterpret_cast<float*>(b + kNoAllocRayOff);
    hrt_hit* dhits = reinterpret_cast<hrt_hit*>(b + kNoAllocHitOff);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(TraceCounters), s);  // the array keeps the last call's contents
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(drays, host_rays, n * 24, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n)
        e = launch_trace_rays(inst, tlas, ninst, drays, n, tmin, tmax, fp64_resolve, bounds, dhits, ctr, s, sm_count);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(host_hits, dhits, n * sizeof(hrt_hit), cudaMemcpyDeviceToHost, s);
    TraceCounters c;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, ctr, sizeof(c), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) *error_word = c.error;
    return e;
}

}  // namespace hrt
