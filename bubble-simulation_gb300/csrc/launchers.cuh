// Launch helpers shared by the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <utility>
#include <vector>

#include "bubble_ext.h"
#include "kernels.cuh"
#include "launch.h"
#include "stage_column.cuh"

namespace bubble {
namespace launch_detail {

inline int grid_for(uint64_t n, int threads) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// cudaFuncSetAttribute once per (kernel, device), keyed on the kernel's
// address: every instantiation of a kernel template shares one function
// type, so the key must be the function itself.
inline cudaError_t ensure_smem_ptr(const void *k, size_t bytes) {
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    for (const auto &d : done)
        if (d.first == k && d.second == dev) return cudaSuccess;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done.emplace_back(k, dev);
    return e;
}
template <typename Kernel>
inline cudaError_t ensure_smem(Kernel k, size_t bytes) {
    return ensure_smem_ptr(reinterpret_cast<const void *>(k), bytes);
}

template <typename R>
cudaError_t init(V2<R> *field, V4<R> *fluid, uint64_t n, R e_ref, cudaStream_t s) {
    dev::init_kernel<R><<<grid_for(n, 256), 256, 0, s>>>(field, fluid, n, e_ref);
    return cudaGetLastError();
}

template <typename R>
cudaError_t nucleate(V2<R> *field, const V4<float> *bubbles, int count, const LatticeParams<R> &P,
                     cudaStream_t s) {
    const dim3 grid((unsigned)((P.nx + dev::kNucBx - 1) / dev::kNucBx), (unsigned)((P.ny + dev::kNucBy - 1) / dev::kNucBy),
                    (unsigned)((P.nz + dev::kNucBz - 1) / dev::kNucBz));
    for (int first = 0; first < count; first += dev::kNucleateBatch) {
        dev::BubbleBatch batch;
        batch.count = count - first < dev::kNucleateBatch ? count - first : dev::kNucleateBatch;
        batch._pad[0] = batch._pad[1] = batch._pad[2] = 0;
        for (int k = 0; k < batch.count; ++k) batch.b[k] = bubbles[first + k];
        dev::nucleate_kernel<R><<<grid, dev::kNucBx * dev::kNucBy, 0, s>>>(field, batch, P);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename R>
cudaError_t prim(const V4<R> *fluid, V4<R> *prim, uint64_t n, const LatticeParams<R> &P,
                 cudaStream_t s) {
    dev::prim_kernel<R><<<grid_for(n, 256), 256, 0, s>>>(fluid, prim, n, P);
    return cudaGetLastError();
}

template <typename R>
cudaError_t stage_ref(const StageArgs<R> &A, const V4<R> *prim, const LatticeParams<R> &P,
                      cudaStream_t s) {
    dim3 grid((P.nx + 63) / 64, P.ny, P.nz);
    dev::stage_ref_kernel<R><<<grid, 64, 0, s>>>(A, prim, P);
    return cudaGetLastError();
}

template <typename R, bool FAST, int FORM, int TY, bool LEAN = false>
cudaError_t stage_column(const StageArgs<R> &A, const LatticeParams<R> &P, int lz, const StageMaps &maps, int tma_ok,
                     int *status, cudaStream_t s) {
    using L = dev::ColumnLayout<R, TY, LEAN>;
    auto k = dev::stage_kernel<R, FAST, FORM, TY, LEAN>;
    cudaError_t e = ensure_smem(k, L::bytes);
    if (e != cudaSuccess) return e;
    if (lz < 1) lz = 1;
    const int ntx = (P.nx + L::TX - 1) / L::TX, nty = (P.ny + TY - 1) / TY;
    const int nzc = (P.nz + lz - 1) / lz;
    dim3 grid(ntx * nty, nzc);
    k<<<grid, L::NT, L::bytes, s>>>(A, P, lz, maps, tma_ok, status);
    return cudaGetLastError();
}

// Whether a 16 x 16 FP32 stage launch takes the shared form: on request, or
// (BUBBLE_STAGE_FORM_AUTO) when column_stage_cost (params.h) rates it cheaper
// at this chunk.  Measured per step, register vs shared form: 128^3 (256
// CTAs) 0.239 vs 0.261 ms, 256^3 (2048 CTAs) 1.549 vs 1.508 ms, 512^3 (4096
// CTAs) 11.38 vs 11.03 ms.
inline bool shared_form(const LatticeParams<float> &P, const TileShape &shape) {
    if (shape.form == BUBBLE_STAGE_FORM_SHARED) return true;
    if (shape.form == BUBBLE_STAGE_FORM_REGISTERS) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);  // the current device's
    if (sms < 1) sms = 1;
    const uint32_t nx = (uint32_t)P.nx, ny = (uint32_t)P.ny, nz = (uint32_t)P.nz;
    return column_stage_cost(nx, ny, nz, shape.lz, true, sms) < column_stage_cost(nx, ny, nz, shape.lz, false, sms);
}

// A 16 x 16 FP32 stage launch in the form shared_form() picks.
template <bool FAST, int FORM>
cudaError_t stage_column16(const StageArgs<float> &A, const LatticeParams<float> &P, const TileShape &shape,
                           const StageMaps &maps, int tma_ok, int *status, cudaStream_t s) {
    if (shared_form(P, shape)) return stage_column<float, FAST, FORM, 16, true>(A, P, shape.lz, maps, tma_ok, status, s);
    return stage_column<float, FAST, FORM, 16, false>(A, P, shape.lz, maps, tma_ok, status, s);
}

template <typename R, int MIXED>
cudaError_t diag(const V2<R> *field, const V4<R> *fluid, const LatticeParams<R> &P,
                 void *partials, unsigned int *ticket, DiagResult *out, cudaStream_t s) {
    const uint64_t n = (uint64_t)P.nx * P.ny * P.nz;
    const int blocks = dev::diag_blocks(n);
    dev::diag_kernel<R, MIXED><<<blocks, dev::kDiagThreads, 0, s>>>(
        field, fluid, P, reinterpret_cast<dev::DiagPartial *>(partials), ticket, out);
    return cudaGetLastError();
}

}  // namespace launch_detail
}  // namespace bubble

#include "batch.cuh"

namespace bubble {
namespace launch_detail {

template <bool FAST, int TY>
int batch_max_grid() {
    using L = dev::ColumnLayout<float, TY, dev::kBatchShared<TY>>;
    auto k = dev::batch_kernel<FAST, TY>;
    if (ensure_smem(k, L::bytes) != cudaSuccess) return 0;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, L::NT, L::bytes) != cudaSuccess) return 0;
    return per_sm * sms;
}

template <bool FAST, int TY>
cudaError_t batch_launch(const void *lat, int n_lat, int n_items, int steps, unsigned int *counters,
                         int *status, int grid, unsigned int barrier_extra, int barrier_shift, cudaStream_t s) {
    using L = dev::ColumnLayout<float, TY, dev::kBatchShared<TY>>;
    auto k = dev::batch_kernel<FAST, TY>;
    cudaError_t e = ensure_smem(k, L::bytes);
    if (e != cudaSuccess) return e;
    const BatchLattice *lp = static_cast<const BatchLattice *>(lat);
    void *args[] = {(void *)&lp,       (void *)&n_lat,  (void *)&n_items,       (void *)&steps,
                    (void *)&counters, (void *)&status, (void *)&barrier_extra, (void *)&barrier_shift};
    return cudaLaunchCooperativeKernel((const void *)k, dim3(grid), dim3(L::NT), args, L::bytes, s);
}

}  // namespace launch_detail
}  // namespace bubble
