// Host-callable launchers of the visualisation kernels (render.cu).
#pragma once

#include <cuda_runtime_api.h>
#include <vector_types.h>

#include <cstdint>

#include "../../include/bubble_render.h"
#include "params.h"

namespace bubble {
namespace launch {

// vis pack of one slot into the half4 surface `surf` (nx x ny x nz texels);
// `dof_ratio` != 1 makes the radiation constant phase dependent.
cudaError_t vis_f32(const V2<float> *field, const V4<float> *fluid, const LatticeParams<float> &P, float a_rad,
                    float t_ref, float dof_ratio, int mode, cudaSurfaceObject_t surf, cudaStream_t s);
cudaError_t vis_f64(const V2<double> *field, const V4<double> *fluid, const LatticeParams<double> &P,
                    double a_rad, double t_ref, float dof_ratio, cudaSurfaceObject_t surf, cudaStream_t s);
// One frame: width x height RGBA8 pixels into device memory `out`.
cudaError_t render(const bubble_view &view, cudaTextureObject_t tex, uchar4 *out, int width, int height,
                   cudaStream_t s);

}  // namespace launch
}  // namespace bubble
