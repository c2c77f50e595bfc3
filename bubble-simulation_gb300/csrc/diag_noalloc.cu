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
//   * the reduction grid-strides over at most 1024 blocks, so every lattice
//     the library accepts fits: the only size limit is the axis range
//     8..2048, and other sizes are rejected;
//   * the array's device address is looked up (cudaGetSymbolAddress) with
//     the caller's device current on every call; the first call on a device
//     also loads this module there, so make that first call before any
//     stream capture;
//   * every call shares the one array and the array keeps the last call's
//     contents; the counter is cleared on the caller's stream before each
//     launch, and calls that overlap on the GPU (different streams, no
//     ordering between them) race on the scratch.
// The lattice is described by its bubble_spec (grid, model, precision form,
// equation of state), and the kernel, its launch shape, its constants and
// its arithmetic are those bubble_diagnostics uses for that spec, so the
// results are identical.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/bubble.h"
#include "../../include/bubble_ext.h"
#include "launchers.cuh"
#include "physics.h"
#include "simulation.h"

namespace {

using bubble::dev::DiagPartial;
constexpr int kPartials = bubble::dev::kDiagMaxBlocks;  // 1024
constexpr size_t kPartialBytes = sizeof(DiagPartial) * kPartials;
constexpr size_t kScratchBytes = kPartialBytes + 256;  // partials + counter area

static __device__ __align__(256) unsigned char g_diag_scratch[kScratchBytes];

int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);  // read back with bubble_last_error()
    return code;
}

// Device address of the scratch array on the current device.  Looked up on
// every call (cheap once the module is loaded), so the pointer can never
// outlive the context it was taken in.
int scratch_address(void **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return fail(BUBBLE_ERR_CUDA,
                    std::string("cudaGetSymbolAddress of the reduction scratch: ") + cudaGetErrorString(e));
    }
    *out = p;
    return BUBBLE_OK;
}

// The perturbation form stores E - e_ref: bubble_diagnostics adds the
// background N e_ref to the energy sums on the host; here the result lives
// on the device, so one thread adds it after the reduction, in FP64.
__global__ void add_background_kernel(bubble::DiagResult *out, double bg) {
    out->sums[0] += bg;
    out->sums[3] += bg;
}

template <int MODE>
cudaError_t diag_f32(const void *field, const void *fluid, const bubble_spec &spec, void *partials,
                     unsigned int *ticket, bubble::DiagResult *out, cudaStream_t s) {
    return bubble::launch_detail::diag<float, MODE>(static_cast<const bubble::V2<float> *>(field),
                                                    static_cast<const bubble::V4<float> *>(fluid),
                                                    bubble::lattice_params_f32(spec), partials, ticket, out, s);
}

}  // namespace

extern "C" {

int bubble_diagnostics_noalloc(const void *field, const void *fluid, const bubble_spec *spec, void *result,
                               void *stream) {
    if (!field || !fluid || !spec || !result)
        return fail(BUBBLE_ERR_INVALID, "field, fluid, spec and result must be non-NULL");
    for (int a = 0; a < 3; ++a)
        if (spec->grid[a] < BUBBLE_MIN_GRID || spec->grid[a] > BUBBLE_MAX_GRID)
            return fail(BUBBLE_ERR_INVALID, "grid axis " + std::to_string(a) + " is " +
                                                std::to_string(spec->grid[a]) + "; accepted axes are 8..2048");
    if (spec->precision < BUBBLE_PRECISION_SINGLE || spec->precision > BUBBLE_PRECISION_PERTURBATION)
        return fail(BUBBLE_ERR_INVALID, "unknown precision");
    {
        const std::string msg = bubble::validate_model(spec->model);
        if (!msg.empty()) return fail(BUBBLE_ERR_INVALID, msg);
        const std::string emsg = bubble::validate_eos(*spec);
        if (!emsg.empty()) return fail(BUBBLE_ERR_INVALID, emsg);
    }
    static_assert(bubble::dev::kDiagMaxBlocks == kPartials,
                  "the reduction launches at most kDiagMaxBlocks blocks, one partial each");
    void *scratch = nullptr;
    const int rc = scratch_address(&scratch);
    if (rc != BUBBLE_OK) return rc;
    void *partials = scratch;
    unsigned int *ticket = reinterpret_cast<unsigned int *>(static_cast<char *>(scratch) + kPartialBytes);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto *out = static_cast<bubble::DiagResult *>(result);
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        if (spec->precision == BUBBLE_PRECISION_DOUBLE) {
            e = bubble::launch_detail::diag<double, bubble::dev::kPlain>(
                static_cast<const bubble::V2<double> *>(field), static_cast<const bubble::V4<double> *>(fluid),
                bubble::lattice_params_f64(*spec), partials, ticket, out, s);
        } else {
            switch (bubble::arith_mode(*spec)) {
                case bubble::dev::kMixed:
                    e = diag_f32<bubble::dev::kMixed>(field, fluid, *spec, partials, ticket, out, s);
                    break;
                case bubble::dev::kPert:
                    e = diag_f32<bubble::dev::kPert>(field, fluid, *spec, partials, ticket, out, s);
                    if (e == cudaSuccess) {
                        const bubble::LatticeParams<float> P = bubble::lattice_params_f32(*spec);
                        const uint64_t cells = (uint64_t)spec->grid[0] * spec->grid[1] * spec->grid[2];
                        add_background_kernel<<<1, 1, 0, s>>>(out, (double)P.e_bg * (double)cells);
                        e = cudaGetLastError();
                    }
                    break;
                case bubble::dev::kGamma:
                    e = diag_f32<bubble::dev::kGamma>(field, fluid, *spec, partials, ticket, out, s);
                    break;
                case bubble::dev::kThermal:
                    e = diag_f32<bubble::dev::kThermal>(field, fluid, *spec, partials, ticket, out, s);
                    break;
                default:
                    e = diag_f32<bubble::dev::kPlain>(field, fluid, *spec, partials, ticket, out, s);
                    break;
            }
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(BUBBLE_ERR_CUDA, std::string("diagnostics launch: ") + cudaGetErrorString(e));
    }
    return BUBBLE_OK;
}

}  // extern "C"
