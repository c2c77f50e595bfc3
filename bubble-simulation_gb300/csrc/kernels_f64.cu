// FP64 instantiation of every kernel: the FP64 CUDA oracle against which the
// FP32 paths' rounding error is stated.  Built with --fmad=false, so it is
// bit-identical with a plain IEEE double restatement on the CPU.
#include "launchers.cuh"

namespace bubble {
namespace launch {

using namespace launch_detail;

cudaError_t init_f64(V2<double> *field, V4<double> *fluid, uint64_t n, double e_ref,
                     cudaStream_t s) {
    return init<double>(field, fluid, n, e_ref, s);
}
cudaError_t nucleate_f64(V2<double> *field, const V4<float> *bubbles, int count,
                         const LatticeParams<double> &P, cudaStream_t s) {
    return nucleate<double>(field, bubbles, count, P, s);
}
cudaError_t prim_f64(const V4<double> *fluid, V4<double> *out, uint64_t n,
                     const LatticeParams<double> &P, cudaStream_t s) {
    return prim<double>(fluid, out, n, P, s);
}
cudaError_t stage_ref_f64(const StageArgs<double> &A, const V4<double> *p,
                          const LatticeParams<double> &P, cudaStream_t s) {
    return stage_ref<double>(A, p, P, s);
}
cudaError_t diag_f64(const V2<double> *field, const V4<double> *fluid,
                     const LatticeParams<double> &P, void *partials, unsigned int *ticket,
                     DiagResult *out, cudaStream_t s) {
    return diag<double, false>(field, fluid, P, partials, ticket, out, s);
}

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {


cudaError_t stage_f64(const StageArgs<double> &A, const LatticeParams<double> &P, TileShape shape,
                      const StageMaps &maps, int tma_ok, int *status, cudaStream_t s) {
    using namespace launch_detail;
    if (shape.tx != tile_x_for(shape.ty)) return cudaErrorInvalidValue;
    if (shape.ty == 16) return stage_column<double, false, false, 16>(A, P, shape.lz, maps, tma_ok, status, s);
    if (shape.ty == 4) return stage_column<double, false, false, 4>(A, P, shape.lz, maps, tma_ok, status, s);
    return cudaErrorInvalidValue;
}

}  // namespace launch
}  // namespace bubble
