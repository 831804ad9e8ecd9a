// trace_frames.cu -- the frame kernels for one node mode, compiled three times: with
// HRT_FRAMES_QUANT=0 (FP32 nodes), =1 (8-bit nodes) and =2 (each instance's own format, for TLASes
// and batches that mix the two; the mixed-type kernel only), so the three sets build in parallel.
#include "trace_device.cuh"

#ifndef HRT_FRAMES_QUANT
#error "compile with -DHRT_FRAMES_QUANT=0, 1 or 2"
#endif

namespace hrt {

// variant: 0 default (4 resident blocks per SM), 1 = 4, 2 = 3 (more registers per thread),
// 3 = 5 (fewer). Launches the frame pass and, when Phantom candidates may need it, the FP64 pass.
#if HRT_FRAMES_QUANT == 2
cudaError_t launch_frames_m(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    constexpr int kN = kNodesPerInstance;
    cudaError_t e = launch_frame<kN, kMixed, 4, 1>(L, s, sm_count);
    if (e != cudaSuccess) return e;
    return launch_resolve<kN>(L, s, sm_count);
}
cudaError_t prepare_frames_m() { return prepare_frame_kernels<kNodesPerInstance>(); }
#else
#if HRT_FRAMES_QUANT
cudaError_t launch_frames_q(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    constexpr int kN = kNodesQ;
#else
cudaError_t launch_frames_f(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    constexpr int kN = kNodesF;
#endif
    cudaError_t e;
    switch (L.variant) {
        case 2: e = launch_kind<kN, 3>(L, s, sm_count); break;
        case 3: e = launch_kind<kN, 5>(L, s, sm_count); break;
        default: e = launch_kind<kN, 4>(L, s, sm_count); break;
    }
    if (e != cudaSuccess) return e;
    return launch_resolve<kN>(L, s, sm_count);
}

#if HRT_FRAMES_QUANT
cudaError_t prepare_frames_q() { return prepare_frame_kernels<kNodesQ>(); }
#else
cudaError_t prepare_frames_f() { return prepare_frame_kernels<kNodesF>(); }
#endif
#endif

}  // namespace hrt
