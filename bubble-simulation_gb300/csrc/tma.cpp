// Tensor-map encoding: see tma.h.  The driver's cuTensorMapEncodeTiled is
// reached through the runtime's entry-point query, so the library needs no
// link-time dependency on the driver library.
#include "tma.h"

#include <cuda_runtime_api.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

namespace bubble {

namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}
}  // namespace

bool encode_stage_maps(StageMaps *out, const void *field, const void *fluid, int nx, int ny, int nz,
                       int tile_x, int tile_y, size_t elem_bytes) {
    std::memset(out, 0, sizeof(*out));
    auto fn = encode_fn();
    if (!fn) return false;
    if ((2 * (size_t)nx * elem_bytes) % 16 != 0) return false;
    if ((reinterpret_cast<uintptr_t>(field) | reinterpret_cast<uintptr_t>(fluid)) % 16 != 0) return false;
    const CUtensorMapDataType dt = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const cuuint32_t pw = (cuuint32_t)(tile_x + 4), ph = (cuuint32_t)(tile_y + 4);
    {
        const cuuint64_t dims[4] = {4, (cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
        const cuuint64_t strides[3] = {4 * elem_bytes, 4 * elem_bytes * (cuuint64_t)nx,
                                       4 * elem_bytes * (cuuint64_t)nx * (cuuint64_t)ny};
        const cuuint32_t box[4] = {4, pw, ph, 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        if (fn(&out->fluid, dt, 4, const_cast<void *>(fluid), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    {
        const cuuint64_t dims[3] = {2 * (cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
        const cuuint64_t strides[2] = {2 * elem_bytes * (cuuint64_t)nx,
                                       2 * elem_bytes * (cuuint64_t)nx * (cuuint64_t)ny};
        const cuuint32_t box[3] = {2 * pw, ph, 1};
        const cuuint32_t es[3] = {1, 1, 1};
        if (fn(&out->field, dt, 3, const_cast<void *>(field), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

}  // namespace bubble
