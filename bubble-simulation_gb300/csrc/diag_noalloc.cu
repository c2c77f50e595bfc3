// Diagnostics reduction for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: an engine that owns every byte of
// device memory through its own pool and forbids allocations behind its
// back, a real-time loop that must not take the allocator's locks or risk
// an out-of-memory failure in the middle of a run, or a host with a fixed
// memory budget.  They already hold the lattice (and a place for the
// result) in their own device buffers; what the reduction needs beyond
// that is a small scratch area for per-block partial sums and a completion
// counter.  This file keeps that scratch in a statically sized __device__
// array, so the entry point below allocates nothing.
//
// Cost and limits:
//   * the array is 1024 block partials (48 B each) plus a 256 B counter
//     area, 49,408 bytes; every GPU that loads this library holds it until
//     the process exits;
//   * the reduction grid-strides over at most 1024 blocks, so any lattice
//     the library accepts (axes 8..2048) fits; larger requests are rejected;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress), which also loads this module on that device:
//     make that first call before any stream capture;
//   * every call shares the one array and the array keeps the last call's
//     contents; the counter is cleared on the caller's stream before each
//     launch, and calls that overlap on the GPU (different streams, no
//     ordering between them) race on the scratch.
// The kernel, its launch shape and its arithmetic are those of
// bubble_diagnostics, so the results are identical.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/bubble.h"
#include "../../include/bubble_ext.h"
#include "launchers.cuh"
#include "physics.h"

namespace {

using bubble::dev::DiagPartial;
constexpr int kPartials = bubble::dev::kDiagMaxBlocks;  // 1024
constexpr size_t kPartialBytes = sizeof(DiagPartial) * kPartials;
constexpr size_t kScratchBytes = kPartialBytes + 256;  // partials + counter area

static __device__ __align__(256) unsigned char g_diag_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch[kMaxDevices] = {};

int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);  // read back with bubble_last_error()
    return code;
}

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(BUBBLE_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= kMaxDevices) return fail(BUBBLE_ERR_CUDA, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_diag_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return fail(BUBBLE_ERR_CUDA, std::string("cudaGetSymbolAddress of the reduction scratch: ") +
                                             cudaGetErrorString(e));
        }
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return BUBBLE_OK;
}

template <typename R>
bubble::LatticeParams<R> params_of(const bubble_model &m, const uint32_t grid[3]) {
    const bubble::SimParamsHost h = bubble::sim_params(m, grid);
    bubble::LatticeParams<R> p{};
    p.nx = (int)h.nx;
    p.ny = (int)h.ny;
    p.nz = (int)h.nz;
    p.dx = h.dx;
    p.inv_dx = h.inv_dx;
    p.eta = h.eta;
    p.lambda = h.lambda;
    p.phi_b = h.phi_b;
    p.m2 = h.m2;
    p.delta = h.delta;
    p.wall_width = h.wall_width;
    p.p_floor = h.p_floor;
    p.e_floor = h.e_floor;
    p.z_max = h.z_max;
    p.e_ref = h.e_ref;
    return p;
}

}  // namespace

extern "C" {

int bubble_diagnostics_noalloc(const void *field, const void *fluid, const uint32_t grid[3],
                               const bubble_model *model, int32_t precision, void *result,
                               void *stream) {
    if (!field || !fluid || !grid || !model || !result)
        return fail(BUBBLE_ERR_INVALID, "field, fluid, grid, model and result must be non-NULL");
    for (int a = 0; a < 3; ++a)
        if (grid[a] < BUBBLE_MIN_GRID || grid[a] > BUBBLE_MAX_GRID)
            return fail(BUBBLE_ERR_INVALID, "grid axis " + std::to_string(a) + " is " +
                                                std::to_string(grid[a]) + "; accepted axes are 8..2048");
    if (precision < BUBBLE_PRECISION_SINGLE || precision > BUBBLE_PRECISION_DOUBLE)
        return fail(BUBBLE_ERR_INVALID, "precision must be SINGLE, MIXED or DOUBLE");
    const std::string msg = bubble::validate_model(*model);
    if (!msg.empty()) return fail(BUBBLE_ERR_INVALID, msg);
    const uint64_t cells = (uint64_t)grid[0] * grid[1] * grid[2];
    if (bubble::launch::diag_blocks_for(cells) > kPartials)
        return fail(BUBBLE_ERR_INVALID, "the reduction needs more block partials than the 1024 the "
                                        "static scratch holds");
    void *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != BUBBLE_OK) return rc;
    void *partials = scratch;
    unsigned int *ticket = reinterpret_cast<unsigned int *>(static_cast<char *>(scratch) + kPartialBytes);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        auto *out = static_cast<bubble::DiagResult *>(result);
        if (precision == BUBBLE_PRECISION_DOUBLE)
            e = bubble::launch_detail::diag<double, false>(
                static_cast<const bubble::V2<double> *>(field), static_cast<const bubble::V4<double> *>(fluid),
                params_of<double>(*model, grid), partials, ticket, out, s);
        else if (precision == BUBBLE_PRECISION_MIXED)
            e = bubble::launch_detail::diag<float, true>(
                static_cast<const bubble::V2<float> *>(field), static_cast<const bubble::V4<float> *>(fluid),
                params_of<float>(*model, grid), partials, ticket, out, s);
        else
            e = bubble::launch_detail::diag<float, false>(
                static_cast<const bubble::V2<float> *>(field), static_cast<const bubble::V4<float> *>(fluid),
                params_of<float>(*model, grid), partials, ticket, out, s);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(BUBBLE_ERR_CUDA, std::string("diagnostics launch: ") + cudaGetErrorString(e));
    }
    return BUBBLE_OK;
}

}  // extern "C"
