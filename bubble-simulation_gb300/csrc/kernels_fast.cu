// FP32 fused stage kernel in the fast arithmetic mode: FMA contraction,
// shared reciprocals and the hardware rcp/sqrt/rsqrt approximations.
#include "launchers.cuh"

namespace bubble {
namespace launch {

using namespace launch_detail;

cudaError_t stage_fused_f32_fast(const StageArgs<float> &A, const LatticeParams<float> &P,
                                 TileShape shape, bool mixed, cudaStream_t s) {
    if (shape.tx != 32) return cudaErrorInvalidValue;
    if (shape.ty == 8) {
        if (mixed) return stage_fused<float, true, true, 8>(A, P, shape.lz, s);
        return stage_fused<float, true, false, 8>(A, P, shape.lz, s);
    }
    if (shape.ty == 4) {
        if (mixed) return stage_fused<float, true, true, 4>(A, P, shape.lz, s);
        return stage_fused<float, true, false, 4>(A, P, shape.lz, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {

cudaError_t stage_v2_f32_fast(const StageArgs<float> &A, const LatticeParams<float> &P, TileShape shape,
                              bool mixed, const StageMaps &maps, int tma_ok, int *status, cudaStream_t s) {
    using namespace launch_detail;
    if (shape.tx != 32) return cudaErrorInvalidValue;
    if (shape.ty == 8) {
        if (mixed) return stage_v2<float, true, true, 8>(A, P, shape.lz, maps, tma_ok, status, s);
        return stage_v2<float, true, false, 8>(A, P, shape.lz, maps, tma_ok, status, s);
    }
    if (shape.ty == 4) {
        if (mixed) return stage_v2<float, true, true, 4>(A, P, shape.lz, maps, tma_ok, status, s);
        return stage_v2<float, true, false, 4>(A, P, shape.lz, maps, tma_ok, status, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble
