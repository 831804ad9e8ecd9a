// trace_frames.cu -- the frame kernels for one node layout, compiled twice: with
// HRT_FRAMES_QUANT=0 (FP32 nodes) and =1 (8-bit nodes), so the two sets build in parallel.
#include "trace_device.cuh"

#ifndef HRT_FRAMES_QUANT
#error "compile with -DHRT_FRAMES_QUANT=0 or 1"
#endif

namespace hrt {

// variant: 0 default (4 resident blocks per SM), 1 = 4, 2 = 3 (more registers per thread),
// 3 = 5 (fewer). Launches the frame pass and, when Phantom candidates may need it, the FP64 pass.
#if HRT_FRAMES_QUANT
cudaError_t launch_frames_q(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    constexpr bool kQ = true;
#else
cudaError_t launch_frames_f(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    constexpr bool kQ = false;
#endif
    cudaError_t e;
    switch (L.variant) {
        case 2: e = launch_kind<kQ, 3>(L, s, sm_count); break;
        case 3: e = launch_kind<kQ, 5>(L, s, sm_count); break;
        default: e = launch_kind<kQ, 4>(L, s, sm_count); break;
    }
    if (e != cudaSuccess) return e;
    return launch_resolve<kQ>(L, s, sm_count);
}

#if HRT_FRAMES_QUANT
cudaError_t prepare_frames_q() { return prepare_frame_kernels<true>(); }
#else
cudaError_t prepare_frames_f() { return prepare_frame_kernels<false>(); }
#endif

}  // namespace hrt
