// Launchers of the visualisation kernels (render.cuh).  Built with
// --fmad=false and IEEE division / square root, so the vis pack is
// bit-identical with a plain IEEE restatement on the CPU, and the
// ray-march's arithmetic differs from one only through the library
// functions (expf, powf) and the texture unit's filter.
#include "launch_render.h"
#include "render.cuh"

namespace bubble {
namespace launch {

namespace {
int vis_grid(uint64_t n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t blocks = (n + 255) / 256;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 16;
    return (int)(blocks < cap ? blocks : cap);
}
}  // namespace

cudaError_t vis_f32(const V2<float> *field, const V4<float> *fluid, const LatticeParams<float> &P, float a_rad,
                    float t_ref, float dof_ratio, int mode, cudaSurfaceObject_t surf, cudaStream_t s) {
    const uint64_t n = (uint64_t)P.nx * P.ny * P.nz;
    const dev::VisConsts<float> C{a_rad, t_ref, dof_ratio};
    if (mode == dev::kThermal)
        dev::vis_kernel<float, dev::kThermal><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    else if (mode == dev::kGamma)
        dev::vis_kernel<float, dev::kGamma><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    else if (mode == dev::kPert) dev::vis_kernel<float, dev::kPert><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    else if (mode == dev::kMixed) dev::vis_kernel<float, dev::kMixed><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    else dev::vis_kernel<float, dev::kPlain><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    return cudaGetLastError();
}

cudaError_t vis_f64(const V2<double> *field, const V4<double> *fluid, const LatticeParams<double> &P,
                    double a_rad, double t_ref, float dof_ratio, cudaSurfaceObject_t surf, cudaStream_t s) {
    const uint64_t n = (uint64_t)P.nx * P.ny * P.nz;
    const dev::VisConsts<double> C{a_rad, t_ref, (double)dof_ratio};
    dev::vis_kernel<double, dev::kPlain><<<vis_grid(n), 256, 0, s>>>(field, fluid, P, C, surf);
    return cudaGetLastError();
}

cudaError_t render(const bubble_view &view, cudaTextureObject_t tex, uchar4 *out, int width, int height,
                   cudaStream_t s) {
    dev::ViewArgs A;
    A.v = view;
    A.tex = tex;
    A.out = out;
    A.width = width;
    A.height = height;
    const dim3 grid((unsigned)((width + 15) / 16), (unsigned)((height + 7) / 8));
    dev::render_kernel<<<grid, 128, 0, s>>>(A);
    return cudaGetLastError();
}

}  // namespace launch
}  // namespace bubble
