// FP32 kernels in the strict arithmetic mode.  Built with --fmad=false and
// IEEE division / square root: every result is bit-identical with a plain
// IEEE single-precision restatement of the same operations on the CPU.
// Also holds the kernels whose results must not depend on the mode (init,
// nucleation, diagnostics).
#include "launchers.cuh"

namespace bubble {
namespace launch {

using namespace launch_detail;

cudaError_t init_f32(V2<float> *field, V4<float> *fluid, uint64_t n, float e_ref,
                     cudaStream_t s) {
    return init<float>(field, fluid, n, e_ref, s);
}
cudaError_t nucleate_f32(V2<float> *field, const V4<float> *bubbles, int count,
                         const LatticeParams<float> &P, cudaStream_t s) {
    return nucleate<float>(field, bubbles, count, P, s);
}
cudaError_t prim_f32(const V4<float> *fluid, V4<float> *out, uint64_t n,
                     const LatticeParams<float> &P, cudaStream_t s) {
    return prim<float>(fluid, out, n, P, s);
}
cudaError_t stage_ref_f32(const StageArgs<float> &A, const V4<float> *p,
                          const LatticeParams<float> &P, cudaStream_t s) {
    return stage_ref<float>(A, p, P, s);
}
cudaError_t diag_f32(const V2<float> *field, const V4<float> *fluid,
                     const LatticeParams<float> &P, int mode, void *partials,
                     unsigned int *ticket, DiagResult *out, cudaStream_t s) {
    if (mode == dev::kThermal) return diag<float, dev::kThermal>(field, fluid, P, partials, ticket, out, s);
    if (mode == dev::kGamma) return diag<float, dev::kGamma>(field, fluid, P, partials, ticket, out, s);
    if (mode == dev::kPert) return diag<float, dev::kPert>(field, fluid, P, partials, ticket, out, s);
    if (mode == dev::kMixed) return diag<float, dev::kMixed>(field, fluid, P, partials, ticket, out, s);
    return diag<float, dev::kPlain>(field, fluid, P, partials, ticket, out, s);
}

size_t diag_partials_bytes() { return sizeof(dev::DiagPartial) * dev::kDiagMaxBlocks; }
int diag_blocks_for(uint64_t cells) { return dev::diag_blocks(cells); }

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {

bool stage_shape_supported(int precision_double, int ty) {
    return precision_double ? (ty == 4 || ty == 16) : (ty == 4 || ty == 8 || ty == 16);
}
size_t stage_smem_bytes(int precision_double, int ty) {
    if (precision_double) return ty == 16 ? dev::ColumnLayout<double, 16>::bytes : dev::ColumnLayout<double, 4>::bytes;
    if (ty == 16) return dev::ColumnLayout<float, 16>::bytes;
    return ty == 4 ? dev::ColumnLayout<float, 4>::bytes : dev::ColumnLayout<float, 8>::bytes;
}

cudaError_t stage_f32_strict(const StageArgs<float> &A, const LatticeParams<float> &P, TileShape shape, int mode,
                             const StageMaps &maps, int tma_ok, int *status, cudaStream_t s) {
    using namespace launch_detail;
    if (shape.tx != tile_x_for(shape.ty)) return cudaErrorInvalidValue;
    if (shape.ty == 16) {
        if (mode == dev::kThermal)
            return stage_column16<false, dev::kThermal>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kGamma) return stage_column16<false, dev::kGamma>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kPert) return stage_column16<false, dev::kPert>(A, P, shape, maps, tma_ok, status, s);
        if (mode == dev::kMixed) return stage_column16<false, dev::kMixed>(A, P, shape, maps, tma_ok, status, s);
        return stage_column16<false, dev::kPlain>(A, P, shape, maps, tma_ok, status, s);
    }
    if (shape.ty == 8 && mode == dev::kMixed)
        return stage_column<float, false, dev::kMixed, 8>(A, P, shape.lz, maps, tma_ok, status, s);
    if (shape.ty == 8 && mode == dev::kPlain)
        return stage_column<float, false, dev::kPlain, 8>(A, P, shape.lz, maps, tma_ok, status, s);
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {

int batch_max_grid_strict(int ty) {
    if (ty != 16) return 0;
    return launch_detail::batch_max_grid<false, 16>();
}
cudaError_t batch_launch_strict(int ty, const void *lat, int n_lat, int n_items, int steps,
                                unsigned int *counters, int *status, int grid, unsigned int barrier_extra,
                                int barrier_shift, cudaStream_t s) {
    if (ty != 16) return cudaErrorInvalidValue;
    return launch_detail::batch_launch<false, 16>(lat, n_lat, n_items, steps, counters, status, grid, barrier_extra,
                                                 barrier_shift, s);
}

}  // namespace launch
}  // namespace bubble
