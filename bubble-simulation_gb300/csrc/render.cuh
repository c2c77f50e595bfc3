// Headless visualisation kernels: the vis pack and the volume ray-march.
//
// vis_kernel restates shaders/vis.wgsl:30-55 with the primitive recovery of
// shaders/primitives.wgsl:16-23 fused in (there is no primitive cache): per
// cell (phi/phi_b, |v|, T/T_ref - 1, (E+p)v^2/e_ref), rounded to f32 and
// then to binary16 (round to nearest even), written through a surface into
// a half4 CUDA array.
//
// render_kernel restates the fragment shader shaders/volume.wgsl:229-381 as
// one thread per pixel: unproject, background gradient, slab test, cutaway
// plane, box wireframe, then the march with the isosurface crossing test,
// gradient-shaded wall and emissive plasma, the tonemap and the gamma
// curve.  The texture is sampled by the texture unit with trilinear
// filtering, clamp to edge and normalised coordinates -- the sampler of
// src/gpu/render.rs:206-218 -- so the fixed-point filter weights that the
// reference's `<= 0` crossing test accounts for are the same here.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/bubble_render.h"
#include "physics.cuh"

namespace bubble {
namespace dev {

// ---------------------------------------------------------------------------
//  vis pack
// ---------------------------------------------------------------------------
template <typename R>
struct VisConsts {
    R a_rad, t_ref;
    // Phase-dependent radiation constant (docs/EOS.md:58-84):
    // a(phi) = a_rad (1 + (r - 1) smoothstep(phi / phi_b)); r = 1 is the bag model.
    R dof_ratio;
};

BUBBLE_DEV unsigned short half_bits(float x) { return __half_as_ushort(__float2half_rn(x)); }

template <typename R, int MIXED>
__global__ void __launch_bounds__(256) vis_kernel(const V2<R> *__restrict__ field, const V4<R> *__restrict__ fluid,
                                                  LatticeParams<R> P, VisConsts<R> C, cudaSurfaceObject_t surf) {
    const uint64_t n = (uint64_t)P.nx * P.ny * P.nz;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % (uint64_t)P.nx);
        const uint64_t yz = i / (uint64_t)P.nx;
        const int y = (int)(yz % (uint64_t)P.ny);
        const int z = (int)(yz / (uint64_t)P.ny);
        const R phi = field[i].x;
        const V4<R> u = fluid[i];
        const V4<R> q = recover<R, false, MIXED>(u, P, phi);
        // the full p and max(E, e_floor); the perturbation form adds its backgrounds
        const R p = MIXED == kPert ? P.p_bg + q.w : q.w;
        const R e_lab = MIXED == kPert ? P.e_bg + vmax(u.x, P.e_floor) : vmax(u.x, P.e_floor);
        const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
        const R speed = sqrt(v2);
        // eos_temperature (shaders/eos.wgsl:65-69)
        const R pt = MIXED == kPert ? P.p_bg + vmax(q.w, P.p_floor) : vmax(p, P.p_floor);
        R a = C.a_rad;
        if (C.dof_ratio != R(1.0)) {
            const R h = vmin(vmax(phi / P.phi_b, R(0.0)), R(1.0));
            const R smooth = h * h * (R(3.0) - R(2.0) * h);
            a = C.a_rad * (R(1.0) + (C.dof_ratio - R(1.0)) * smooth);
        }
        R temp;
        if constexpr (MIXED == kThermal) temp = thermal_temperature<R, false>(pt, phi, P);
        else temp = sqrt(sqrt(R(3.0) * pt / a));
        const R kinetic = (e_lab + p) * v2;
        ushort4 t;
        t.x = half_bits((float)(phi / P.phi_b));
        t.y = half_bits((float)speed);
        t.z = half_bits((float)(temp / C.t_ref - R(1.0)));
        t.w = half_bits((float)(kinetic / P.e_ref));
        surf3Dwrite(t, surf, x * (int)sizeof(ushort4), y, z, cudaBoundaryModeZero);
    }
}

// ---------------------------------------------------------------------------
//  ray-march
// ---------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
BUBBLE_DEV f3 mk(float x, float y, float z) { return f3{x, y, z}; }
BUBBLE_DEV f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
BUBBLE_DEV f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
BUBBLE_DEV f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
BUBBLE_DEV f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
BUBBLE_DEV f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
BUBBLE_DEV f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
BUBBLE_DEV f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
BUBBLE_DEV float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BUBBLE_DEV f3 normalise(f3 a) { return a / sqrtf(dot3(a, a)); }
BUBBLE_DEV float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
// WGSL mix: e1 (1 - t) + e2 t
BUBBLE_DEV float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
BUBBLE_DEV f3 mix3(f3 a, f3 b, float t) { return mk(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
BUBBLE_DEV float fractf(float x) { return x - floorf(x); }
BUBBLE_DEV float smooth_step(float lo, float hi, float x) {
    const float t = clampf((x - lo) / (hi - lo), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// Colour maps of shaders/volume.wgsl:37-78 (11 control points each):
// viridis, inferno and the signed map with a near-black centre.
__constant__ float kColormaps[3][11][3] = {
    {{0.267f, 0.005f, 0.329f}, {0.283f, 0.141f, 0.458f}, {0.254f, 0.265f, 0.530f}, {0.207f, 0.372f, 0.553f},
     {0.164f, 0.471f, 0.558f}, {0.128f, 0.567f, 0.551f}, {0.135f, 0.659f, 0.518f}, {0.267f, 0.749f, 0.441f},
     {0.478f, 0.821f, 0.318f}, {0.741f, 0.873f, 0.150f}, {0.993f, 0.906f, 0.144f}},
    {{0.001f, 0.000f, 0.014f}, {0.078f, 0.044f, 0.214f}, {0.225f, 0.036f, 0.388f}, {0.373f, 0.074f, 0.432f},
     {0.522f, 0.128f, 0.420f}, {0.665f, 0.182f, 0.370f}, {0.798f, 0.280f, 0.270f}, {0.902f, 0.413f, 0.144f},
     {0.969f, 0.579f, 0.032f}, {0.988f, 0.762f, 0.135f}, {0.988f, 0.998f, 0.645f}},
    {{0.30f, 0.55f, 1.00f}, {0.22f, 0.42f, 0.85f}, {0.15f, 0.30f, 0.66f}, {0.09f, 0.19f, 0.45f},
     {0.04f, 0.09f, 0.24f}, {0.02f, 0.02f, 0.03f}, {0.26f, 0.09f, 0.04f}, {0.48f, 0.17f, 0.06f},
     {0.72f, 0.29f, 0.08f}, {0.92f, 0.48f, 0.14f}, {1.00f, 0.72f, 0.32f}},
};

// ramp (shaders/volume.wgsl:80-90): 0 viridis, 1 inferno, anything else signed.
BUBBLE_DEV f3 ramp(float t, int which) {
    const float x = clampf(t, 0.0f, 1.0f) * 10.0f;
    const int i0 = (int)floorf(x);
    const int i1 = min(i0 + 1, 10);
    const float f = x - floorf(x);
    const int m = (which == 0) ? 0 : (which == 1 ? 1 : 2);
    const f3 a = mk(kColormaps[m][i0][0], kColormaps[m][i0][1], kColormaps[m][i0][2]);
    const f3 b = mk(kColormaps[m][i1][0], kColormaps[m][i1][1], kColormaps[m][i1][2]);
    return mix3(a, b, f);
}

// safe_inv (shaders/volume.wgsl:96-99)
BUBBLE_DEV float safe_inv(float x) {
    const float s = x < 0.0f ? -1.0f : 1.0f;
    return s / fmaxf(fabsf(x), 1e-9f);
}

struct ViewArgs {
    bubble_view v;
    cudaTextureObject_t tex;
    uchar4 *out;
    int width, height;
};

BUBBLE_DEV float4 sample_state(const ViewArgs &A, f3 p) {
    const float *bh = A.v.box_half;
    const float u = (p.x / bh[0]) * 0.5f + 0.5f;
    const float v = (p.y / bh[1]) * 0.5f + 0.5f;
    const float w = (p.z / bh[2]) * 0.5f + 0.5f;
    return tex3D<float4>(A.tex, u, v, w);
}

// grad_phi (shaders/volume.wgsl:123-134)
BUBBLE_DEV f3 grad_phi(const ViewArgs &A, f3 p) {
    const float h = A.v.box_half[3];
    const f3 dx = mk(h, 0.0f, 0.0f), dy = mk(0.0f, h, 0.0f), dz = mk(0.0f, 0.0f, h);
    const f3 g = mk(sample_state(A, p + dx).x - sample_state(A, p - dx).x,
                    sample_state(A, p + dy).x - sample_state(A, p - dy).x,
                    sample_state(A, p + dz).x - sample_state(A, p - dz).x);
    return g / (2.0f * h);
}

// hash12 (shaders/volume.wgsl:136-140)
BUBBLE_DEV float hash12(float px, float py) {
    f3 p3 = mk(fractf(px * 0.1031f), fractf(py * 0.1031f), fractf(px * 0.1031f));
    const float d = dot3(p3, mk(p3.y + 33.33f, p3.z + 33.33f, p3.x + 33.33f));
    p3 = mk(p3.x + d, p3.y + d, p3.z + d);
    return fractf((p3.x + p3.y) * p3.z);
}

// map_field (shaders/volume.wgsl:152-185)
BUBBLE_DEV void map_field(const bubble_view &V, float4 s, float &t, float &intensity, int &ramp_id) {
    const int mode = (int)V.render1[0];
    const float gain = V.render2[0];
    ramp_id = (int)V.render1[3];
    if (mode == 0) {
        const float x = clampf(s.x, 0.0f, 1.0f);
        t = x;
        intensity = x * gain;
    } else if (mode == 1) {
        const float x = clampf(s.y * gain, 0.0f, 1.0f);
        t = x;
        intensity = x;
    } else if (mode == 2) {
        const float x = clampf(s.z * gain, -1.0f, 1.0f);
        t = 0.5f + 0.5f * x;
        intensity = fabsf(x);
        ramp_id = 2;
    } else {
        const float x = clampf(s.w * gain, 0.0f, 1.0f);
        t = x;
        intensity = x;
    }
}

constexpr int kMaxMarchSteps = 2048;

BUBBLE_DEV f3 shade_pixel(const ViewArgs &A, float px, float py, float ndc_x, float ndc_y) {
    const bubble_view &V = A.v;
    const f3 ro = mk(V.cam_pos[0], V.cam_pos[1], V.cam_pos[2]);
    // far = inv_view_proj * (ndc, 1, 1), column-major
    const float *M = V.inv_view_proj;
    float far4[4];
    for (int r = 0; r < 4; ++r) far4[r] = M[0 * 4 + r] * ndc_x + M[1 * 4 + r] * ndc_y + M[2 * 4 + r] * 1.0f + M[3 * 4 + r] * 1.0f;
    const f3 rd = normalise(mk(far4[0] / far4[3], far4[1] / far4[3], far4[2] / far4[3]) - ro);

    const float horizon = clampf(rd.y * 0.5f + 0.5f, 0.0f, 1.0f);
    f3 color = mix3(mk(0.015f, 0.017f, 0.028f), mk(0.045f, 0.055f, 0.085f), horizon) * V.render3[2];

    const f3 inv_rd = mk(safe_inv(rd.x), safe_inv(rd.y), safe_inv(rd.z));
    const f3 half = mk(V.box_half[0], V.box_half[1], V.box_half[2]);
    // intersect_box (shaders/volume.wgsl:103-111)
    const f3 t0 = (-half - ro) * inv_rd;
    const f3 t1 = (half - ro) * inv_rd;
    const float tn = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z));
    const float tf = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z));
    float t_near = fmaxf(tn, 0.0f);
    float t_far = tf;
    if (t_near >= t_far) return color;

    const int clip_axis = (int)V.render1[1];
    if (clip_axis >= 0 && clip_axis <= 2) {
        const float ro_a = clip_axis == 0 ? ro.x : (clip_axis == 1 ? ro.y : ro.z);
        const float rd_a = clip_axis == 0 ? rd.x : (clip_axis == 1 ? rd.y : rd.z);
        const float plane = V.render1[2] * V.box_half[clip_axis];
        const float denom = rd_a;
        const float dist = plane - ro_a;
        if (fabsf(denom) < 1e-6f) {
            if (dist < 0.0f) return color;
        } else {
            const float t_plane = dist / denom;
            if (denom > 0.0f) t_far = fminf(t_far, t_plane);
            else t_near = fmaxf(t_near, t_plane);
            if (t_near >= t_far) return color;
        }
    }

    if (V.render3[1] > 0.5f) {
        const float w = 0.004f * V.box_half[3] * V.grid[0];
        float edge = 0.0f;
        for (int k = 0; k < 2; ++k) {
            const f3 p = ro + rd * (k == 0 ? t_near : t_far);
            const f3 d = mk(half.x - fabsf(p.x), half.y - fabsf(p.y), half.z - fabsf(p.z));
            const float median = fmaxf(fminf(d.x, d.y), fminf(fmaxf(d.x, d.y), d.z));
            edge = fmaxf(edge, 1.0f - smooth_step(0.0f, w, median));
        }
        color = color + mk(0.20f, 0.26f, 0.34f) * edge;
    }

    const float cell = V.box_half[3];
    const float samples_per_cell = fmaxf(V.render0[2], 0.25f);
    float ds = cell / samples_per_cell;
    const float span = t_far - t_near;
    if (span / ds > (float)kMaxMarchSteps) ds = span / (float)kMaxMarchSteps;
    const int n_steps = min((int)ceilf(span / ds), kMaxMarchSteps);

    const float jitter = hash12(px + V.render3[0], py + V.render3[0]);
    const float iso = V.render0[0];
    const float wall_opacity = V.render0[1];
    const float exposure = V.render0[3];
    const float absorption = V.render2[1];
    const bool show_iso = V.render2[2] > 0.5f;
    const bool show_vol = V.render2[3] > 0.5f;

    f3 accum = mk(0.0f, 0.0f, 0.0f);
    float alpha = 0.0f;
    float t = t_near + jitter * ds;
    float prev_phi = sample_state(A, ro + rd * t_near).x;
    float prev_t = t_near;
    const f3 l1 = normalise(mk(0.55f, 0.72f, 0.42f));
    const f3 l2 = normalise(mk(-0.5f, -0.2f, -0.7f));

    for (int i = 0; i < n_steps; ++i) {
        if (t > t_far || alpha > 0.995f) break;
        const f3 p = ro + rd * t;
        const float4 s = sample_state(A, p);

        const float d_prev = prev_phi - iso;
        const float d_cur = s.x - iso;
        if (show_iso && d_prev != 0.0f && d_prev * d_cur <= 0.0f) {
            const float denom = s.x - prev_phi;
            const float frac = fabsf(denom) > 1e-6f ? (iso - prev_phi) / denom : 0.5f;
            const float t_hit = mixf(prev_t, t, clampf(frac, 0.0f, 1.0f));
            const f3 p_hit = ro + rd * t_hit;
            const f3 g = grad_phi(A, p_hit);
            const f3 n = normalise(-g - rd * 1e-6f);
            const float4 hs = sample_state(A, p_hit);
            const float drive = clampf(hs.y * 4.0f, 0.0f, 1.0f);
            const f3 base = mix3(mk(0.16f, 0.62f, 0.72f), mk(1.00f, 0.72f, 0.28f), drive);
            const f3 view = -rd;
            const float diff = fmaxf(dot3(n, l1), 0.0f) + 0.35f * fmaxf(dot3(n, l2), 0.0f);
            const f3 h = normalise(l1 + view + mk(0.0f, 1e-5f, 0.0f));
            const float spec = powf(fmaxf(dot3(n, h), 0.0f), 48.0f);
            const float fres = powf(1.0f - fabsf(dot3(n, view)), 3.0f);
            const f3 shaded = base * (0.22f + 0.85f * diff) + mk(1.0f, 1.0f, 1.0f) * spec * 0.35f + base * fres * 0.9f;
            const float a = wall_opacity;
            accum = accum + (1.0f - alpha) * shaded * a;
            alpha = alpha + (1.0f - alpha) * a;
        }

        if (show_vol) {
            float mt, mi;
            int rid;
            map_field(V, s, mt, mi, rid);
            if (mi > 1e-4f) {
                const float weight = mi * mi;
                const float a = 1.0f - expf(-absorption * weight * ds);
                const f3 emit = ramp(mt, rid) * exposure;
                accum = accum + (1.0f - alpha) * emit * a;
                alpha = alpha + (1.0f - alpha) * a;
            }
        }
        prev_phi = s.x;
        prev_t = t;
        t = t + ds;
    }
    color = color * (1.0f - alpha) + accum;
    return color;
}

// One thread per pixel; row 0 is the top of the image.
__global__ void __launch_bounds__(128) render_kernel(ViewArgs A) {
    const int px = blockIdx.x * 16 + (threadIdx.x & 15);
    const int py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= A.width || py >= A.height) return;
    const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
    const float ndc_x = fx / (float)A.width * 2.0f - 1.0f;
    const float ndc_y = 1.0f - fy / (float)A.height * 2.0f;
    f3 c = shade_pixel(A, fx, fy, ndc_x, ndc_y);
    // tonemap + gamma (shaders/volume.wgsl:374-378)
    c = mk(c.x / (1.0f + c.x), c.y / (1.0f + c.y), c.z / (1.0f + c.z));
    const float g = 1.0f / 2.2f;
    c = mk(powf(fmaxf(c.x, 0.0f), g), powf(fmaxf(c.y, 0.0f), g), powf(fmaxf(c.z, 0.0f), g));
    // Rgba8Unorm store: round to nearest
    auto unorm = [](float x) { return (unsigned char)__float2int_rn(clampf(x, 0.0f, 1.0f) * 255.0f); };
    A.out[(size_t)py * A.width + px] = make_uchar4(unorm(c.x), unorm(c.y), unorm(c.z), 255);
}

}  // namespace dev
}  // namespace bubble
