// FP32 fused stage kernel in the fast arithmetic mode: FMA contraction,
// shared reciprocals and the hardware rcp/sqrt/rsqrt approximations.
#include "launchers.cuh"

namespace bubble {
namespace launch {


cudaError_t stage_f32_fast(const StageArgs<float> &A, const LatticeParams<float> &P, TileShape shape, int mode,
                           const StageMaps &maps, int tma_ok, int *status, cudaStream_t s) {
    using namespace launch_detail;
    if (shape.tx != tile_x_for(shape.ty)) return cudaErrorInvalidValue;
    if (shape.ty == 16) {
        if (mode == dev::kThermal) return stage_column16<true, dev::kThermal>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kGamma) return stage_column16<true, dev::kGamma>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kPert) return stage_column16<true, dev::kPert>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kMixed) return stage_column16<true, dev::kMixed>(A, P, shape, maps, tma_ok, status, s);
        return stage_column16<true, dev::kPlain>(A, P, shape, maps, tma_ok, status, s);
    }
    if (mode != dev::kPlain && mode != dev::kMixed) return cudaErrorInvalidValue;
    if (shape.ty == 8) {
        if (mode == dev::kMixed) return stage_column<float, true, dev::kMixed, 8>(A, P, shape.lz, maps, tma_ok, status, s);
        return stage_column<float, true, dev::kPlain, 8>(A, P, shape.lz, maps, tma_ok, status, s);
    }
    if (shape.ty == 4) {
        if (mode == dev::kMixed) return stage_column<float, true, dev::kMixed, 4>(A, P, shape.lz, maps, tma_ok, status, s);
        return stage_column<float, true, dev::kPlain, 4>(A, P, shape.lz, maps, tma_ok, status, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {

int batch_max_grid(bool fast, int ty) {
    if (!fast) return batch_max_grid_strict(ty);
    if (ty == 16) return launch_detail::batch_max_grid<true, 16>();
    if (ty == 8) return launch_detail::batch_max_grid<true, 8>();
    return 0;
}
size_t batch_smem_bytes(int ty) {
    return ty == 16 ? dev::ColumnLayout<float, 16, dev::kBatchShared<16>>::bytes
                    : dev::ColumnLayout<float, 8, dev::kBatchShared<8>>::bytes;
}
cudaError_t batch_launch(bool fast, int ty, const void *lat, int n_lat, int n_items, int steps,
                         unsigned int *counters, int *status, int grid, unsigned int barrier_extra,
                         int barrier_shift, cudaStream_t s) {
    if (!fast)
        return batch_launch_strict(ty, lat, n_lat, n_items, steps, counters, status, grid, barrier_extra,
                                   barrier_shift, s);
    if (ty == 16)
        return launch_detail::batch_launch<true, 16>(lat, n_lat, n_items, steps, counters, status, grid,
                                                     barrier_extra, barrier_shift, s);
    if (ty == 8)
        return launch_detail::batch_launch<true, 8>(lat, n_lat, n_items, steps, counters, status, grid,
                                                    barrier_extra, barrier_shift, s);
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble
