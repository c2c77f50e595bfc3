// Host-callable launchers of the kernels in kernels.cuh.
//
// Each function is defined in the translation unit whose compiler flags fix
// its arithmetic (kernels_strict.cu, kernels_fast.cu, kernels_f64.cu); this
// header is plain C++ so the host driver, compiled by the host compiler,
// can call them.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>

#include "params.h"
#include "tma.h"

namespace bubble {
namespace launch {

// ---- FP32 (strict translation unit: no FMA contraction) ----------------
cudaError_t init_f32(V2<float> *field, V4<float> *fluid, uint64_t n, float e_ref,
                     cudaStream_t s);
// `bubbles` is a host array of (cx, cy, cz, r0); it is passed by value.
cudaError_t nucleate_f32(V2<float> *field, const V4<float> *bubbles, int count,
                         const LatticeParams<float> &P, cudaStream_t s);
cudaError_t prim_f32(const V4<float> *fluid, V4<float> *prim, uint64_t n,
                     const LatticeParams<float> &P, cudaStream_t s);
cudaError_t stage_ref_f32(const StageArgs<float> &A, const V4<float> *prim,
                          const LatticeParams<float> &P, cudaStream_t s);

// `mode`: 0 plain, 1 mixed, 2 perturbation form, 3 gamma-law equation of
// state, 4 thermal potential (physics.cuh kPlain/kMixed/kPert/kGamma/kThermal).
cudaError_t diag_f32(const V2<float> *field, const V4<float> *fluid,
                     const LatticeParams<float> &P, int mode, void *partials,
                     unsigned int *ticket, DiagResult *out, cudaStream_t s);

// ---- FP64 (the FP64 CUDA oracle; no FMA contraction) --------------------
cudaError_t init_f64(V2<double> *field, V4<double> *fluid, uint64_t n, double e_ref,
                     cudaStream_t s);
cudaError_t nucleate_f64(V2<double> *field, const V4<float> *bubbles, int count,
                         const LatticeParams<double> &P, cudaStream_t s);
cudaError_t prim_f64(const V4<double> *fluid, V4<double> *prim, uint64_t n,
                     const LatticeParams<double> &P, cudaStream_t s);
cudaError_t stage_ref_f64(const StageArgs<double> &A, const V4<double> *prim,
                          const LatticeParams<double> &P, cudaStream_t s);
cudaError_t diag_f64(const V2<double> *field, const V4<double> *fluid,
                     const LatticeParams<double> &P, void *partials, unsigned int *ticket,
                     DiagResult *out, cudaStream_t s);

// Scratch of the diagnostics reduction: partials + ticket.
size_t diag_partials_bytes();
int diag_blocks_for(uint64_t cells);

// ---- fused stage kernel, column form (stage_column.cuh) -----------------------
// `maps` are the tensor maps of the stage input slot (tma.h); `tma_ok` says
// whether they are valid; bit 0 of *status is set if a bounded wait expired.
// Tile heights: 4 or 8 in FP32, 4 in FP64.  `mode`: 0 plain, 1 mixed, 2
// perturbation form, 3 gamma-law equation of state, 4 thermal potential; the
// last three and the strict arithmetic are built for ty = 8 only.
bool stage_shape_supported(int precision_double, int ty);
size_t stage_smem_bytes(int precision_double, int ty);
cudaError_t stage_f32_strict(const StageArgs<float> &A, const LatticeParams<float> &P, TileShape shape,
                                int mode, const StageMaps &maps, int tma_ok, int *status, cudaStream_t s);
cudaError_t stage_f32_fast(const StageArgs<float> &A, const LatticeParams<float> &P, TileShape shape,
                              int mode, const StageMaps &maps, int tma_ok, int *status, cudaStream_t s);
cudaError_t stage_f64(const StageArgs<double> &A, const LatticeParams<double> &P, TileShape shape,
                         const StageMaps &maps, int tma_ok, int *status, cudaStream_t s);

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {

// ---- batched persistent launch (batch.cuh) ---------------------------------
// lat: device array of BatchLattice; counters: 3 zeroed uint32 (barrier
// count, barrier generation, work counter).  Cooperative launch with `grid`
// CTAs, which must not exceed batch_max_grid(fast, ty).  The grid barrier
// between stages releases after grid + barrier_extra arrivals and waits at
// most 2^barrier_shift SM cycles: 0 and 32 in production; the test hook
// bubble_ext_test_expire_batch_barrier passes 1 (no arrival releases it) and
// a short limit.
int batch_max_grid(bool fast, int ty);
size_t batch_smem_bytes(int ty);
cudaError_t batch_launch(bool fast, int ty, const void *lat, int n_lat, int n_items, int steps,
                         unsigned int *counters, int *status, int grid, unsigned int barrier_extra,
                         int barrier_shift, cudaStream_t s);

}  // namespace launch
}  // namespace bubble

namespace bubble {
namespace launch {
// strict-mode halves of the batch entry points (kernels_strict.cu)
int batch_max_grid_strict(int ty);
cudaError_t batch_launch_strict(int ty, const void *lat, int n_lat, int n_items, int steps,
                                unsigned int *counters, int *status, int grid, unsigned int barrier_extra,
                                int barrier_shift, cudaStream_t s);
}  // namespace launch
}  // namespace bubble
