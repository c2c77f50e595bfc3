// Device-side physics of one lattice cell and one cell face.
//
// Restates, for CUDA, the per-cell arithmetic of the reference shaders:
//   potential / dpotential         shaders/potential.wgsl:38-47
//   bag EOS, con2prim, fluxes      shaders/eos.wgsl:94-176
//   MC limiter                     shaders/common.wgsl:114-136
//   sanitise, HLL                  shaders/step.wgsl:61-90
//   nucleation profile             shaders/nucleate.wgsl:51-85
//
// Two arithmetic modes share this file:
//   FAST = false  the WGSL evaluation order with IEEE division and square
//                 root; the translation units that instantiate it are built
//                 with --fmad=false, so every result is bit-identical with a
//                 plain IEEE restatement on the CPU.
//   FAST = true   the same formulas with shared reciprocals and hardware
//                 approximate rcp/sqrt/rsqrt (MUFU), built with FMA
//                 contraction.  Results differ from the strict mode by
//                 rounding only.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "params.h"

namespace bubble {
namespace dev {

#define BUBBLE_DEV __device__ __forceinline__

template <typename R>
BUBBLE_DEV R vmax(R a, R b) {
    return fmax(a, b);
}
template <typename R>
BUBBLE_DEV R vmin(R a, R b) {
    return fmin(a, b);
}
template <>
BUBBLE_DEV float vmax<float>(float a, float b) {
    return fmaxf(a, b);
}
template <>
BUBBLE_DEV float vmin<float>(float a, float b) {
    return fminf(a, b);
}

// Hardware approximations used by the FAST mode (float only).
BUBBLE_DEV float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
BUBBLE_DEV float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
BUBBLE_DEV float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Paired FP32 arithmetic of sm_100+ (two IEEE operations per instruction),
// used by the FAST mode on the (x, y) and (z, w) halves of 4-vectors.
BUBBLE_DEV float2 lo2(const V4<float> &v) { return make_float2(v.x, v.y); }
BUBBLE_DEV float2 hi2(const V4<float> &v) { return make_float2(v.z, v.w); }
BUBBLE_DEV V4<float> v4of(float2 a, float2 b) { return V4<float>{a.x, a.y, b.x, b.y}; }
BUBBLE_DEV float2 bc2(float s) { return make_float2(s, s); }
BUBBLE_DEV float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as a + b * (-1): exact product, one rounding
BUBBLE_DEV float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.0f), a); }
BUBBLE_DEV float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
BUBBLE_DEV float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// x^2 + y^2 + z^2 with fixed roundings (the FAST mode's contraction of it)
BUBBLE_DEV float dot3_rn(float x, float y, float z) { return __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x))); }
BUBBLE_DEV double dot3_rn(double x, double y, double z) { return __fma_rn(z, z, __fma_rn(y, y, __dmul_rn(x, x))); }

// ---------------------------------------------------------------------------
//  Potential (shaders/potential.wgsl:38-47)
// ---------------------------------------------------------------------------
template <typename R>
BUBBLE_DEV R potential(R phi, const LatticeParams<R> &P) {
    const R p2 = phi * phi;
    return R(0.5) * P.m2 * p2 - P.delta * p2 * phi / R(3.0) + R(0.25) * P.lambda * p2 * p2;
}
template <typename R>
BUBBLE_DEV R dpotential(R phi, const LatticeParams<R> &P) {
    return phi * (P.m2 - P.delta * phi + P.lambda * phi * phi);
}

// ---------------------------------------------------------------------------
//  Limiter (shaders/common.wgsl:114-136)
// ---------------------------------------------------------------------------
// minmod3(0.5 (dm + dp), 2 dm, 2 dp) with WGSL sign() semantics.  The three
// signs agree exactly when dm and dp are both non-zero with one sign (the
// half-sum of two same-signed floats cannot round to zero and doubling keeps
// the sign), and then sign(a) * min(|a|, |b|, |c|) is that sign applied to
// the minimum; every other case returns zero.  Same values, fewer
// instructions.
template <typename R, bool FAST = false>
BUBBLE_DEV R limit_slope(R dm, R dp) {
    if constexpr (FAST) {
        // Same limiter with the sign test folded into one product (differs
        // only when dm*dp underflows, i.e. for slopes below 1e-19).
        const R m = vmin(fabs(R(0.5) * (dm + dp)), R(2.0) * vmin(fabs(dm), fabs(dp)));
        return dm * dp > R(0) ? copysign(m, dm) : R(0);
    } else {
        const bool same = (dm > R(0) && dp > R(0)) || (dm < R(0) && dp < R(0));
        const R a = fabs(R(0.5) * (dm + dp));
        const R m = vmin(a, vmin(fabs(R(2.0) * dm), fabs(R(2.0) * dp)));
        return same ? copysign(m, dm) : R(0);
    }
}

// ---------------------------------------------------------------------------
//  Bag EOS (shaders/eos.wgsl:94-123): conserved -> primitive
// ---------------------------------------------------------------------------
// eos_prim_from_cons(eos_regularise(u)) -> (vx, vy, vz, p).
template <typename R, bool FAST>
BUBBLE_DEV V4<R> prim_from_cons(const V4<R> &u, const LatticeParams<R> &P) {
    const R e_lab = vmax(u.x, P.e_floor);
    R zx = u.y, zy = u.z, zz = u.w;
    const R zcap = P.z_max * e_lab;
    if constexpr (FAST) {
        // Explicit roundings (no contraction left to the compiler): the
        // recovery runs at two sites of the stage kernel (chunk prologue and
        // z-march), which must give the same bits for every z chunking.
        R z2 = dot3_rn(zx, zy, zz);
        if (z2 > __fmul_rn(zcap, zcap)) {
            const R s = __fmul_rn(zcap, rsqrt_approx(z2));
            zx = __fmul_rn(zx, s);
            zy = __fmul_rn(zy, s);
            zz = __fmul_rn(zz, s);
            z2 = dot3_rn(zx, zy, zz);
        }
        const R disc = vmax(__fmaf_rn(__fmul_rn(R(4.0), e_lab), e_lab, __fmul_rn(R(-3.0), z2)), R(0.0));
        R p = __fmul_rn(__fmaf_rn(e_lab, e_lab, -z2), rcp_approx(__fadd_rn(e_lab, sqrt_approx(disc))));
        p = vmax(p, P.p_floor);
        const R inv = rcp_approx(vmax(__fadd_rn(e_lab, p), R(1e-30)));
        return V4<R>{__fmul_rn(zx, inv), __fmul_rn(zy, inv), __fmul_rn(zz, inv), p};
    } else {
        const R zlen = sqrt(zx * zx + zy * zy + zz * zz);
        if (zlen > zcap) {
            const R s = zcap / vmax(zlen, R(1e-30));
            zx = zx * s;
            zy = zy * s;
            zz = zz * s;
        }
        const R z2 = zx * zx + zy * zy + zz * zz;
        const R disc = vmax(R(4.0) * e_lab * e_lab - R(3.0) * z2, R(0.0));
        R p = (e_lab * e_lab - z2) / (e_lab + sqrt(disc));
        p = vmax(p, P.p_floor);
        const R s = vmax(e_lab + p, R(1e-30));
        return V4<R>{zx / s, zy / s, zz / s, p};
    }
}

// FP64 recovery of one FP32 cell, used where the Lorentz factor exceeds 3
// (v^2 > 8/9), the regime where E^2 - Z^2 cancels.  Rarely taken and long
// (FP64 division and square root are multi-instruction sequences).  It takes
// the FP32 state and constants by value, so it can also be compiled out of
// line (BUBBLE_F64_RECOVERY_LINKAGE): one copy per kernel was 1.6 % faster
// for the register-form stage kernel at 512^3 (fewer instruction-fetch
// stalls), inlined is 0.6 % faster for the shared form, which now runs every
// large lattice.
#define BUBBLE_F64_RECOVERY_LINKAGE __device__ __forceinline__
template <bool FAST = false>
BUBBLE_F64_RECOVERY_LINKAGE V4<float> prim_from_cons_f64_x(V4<float> u, float e_floor, float z_max, float p_floor);
template <bool FAST = false>
BUBBLE_DEV V4<float> prim_from_cons_f64(const V4<float> &u, const LatticeParams<float> &P) {
    return prim_from_cons_f64_x<FAST>(u, P.e_floor, P.z_max, P.p_floor);
}
template <bool FAST>
BUBBLE_F64_RECOVERY_LINKAGE V4<float> prim_from_cons_f64_x(V4<float> u, float e_floor_f, float z_max_f, float p_floor_f) {
    struct {
        float e_floor, z_max, p_floor;
    } P{e_floor_f, z_max_f, p_floor_f};
    const double e_lab = fmax((double)u.x, (double)P.e_floor);
    double zx = u.y, zy = u.z, zz = u.w;
    if constexpr (FAST) {
        // explicit roundings, so every call site computes the same bits
        const double zcap = __dmul_rn((double)P.z_max, e_lab);
        const double zlen = __dsqrt_rn(dot3_rn(zx, zy, zz));
        if (zlen > zcap) {
            const double s = __ddiv_rn(zcap, fmax(zlen, 1e-30));
            zx = __dmul_rn(zx, s);
            zy = __dmul_rn(zy, s);
            zz = __dmul_rn(zz, s);
        }
        const double z2 = dot3_rn(zx, zy, zz);
        const double disc = fmax(__fma_rn(__dmul_rn(4.0, e_lab), e_lab, __dmul_rn(-3.0, z2)), 0.0);
        double p = __ddiv_rn(__fma_rn(e_lab, e_lab, -z2), __dadd_rn(e_lab, __dsqrt_rn(disc)));
        p = fmax(p, (double)P.p_floor);
        const double s = fmax(__dadd_rn(e_lab, p), 1e-30);
        return V4<float>{(float)__ddiv_rn(zx, s), (float)__ddiv_rn(zy, s), (float)__ddiv_rn(zz, s), (float)p};
    } else {
        const double zcap = (double)P.z_max * e_lab;
        const double zlen = sqrt(zx * zx + zy * zy + zz * zz);
        if (zlen > zcap) {
            const double s = zcap / fmax(zlen, 1e-30);
            zx *= s;
            zy *= s;
            zz *= s;
        }
        const double z2 = zx * zx + zy * zy + zz * zz;
        const double disc = fmax(4.0 * e_lab * e_lab - 3.0 * z2, 0.0);
        double p = (e_lab * e_lab - z2) / (e_lab + sqrt(disc));
        p = fmax(p, (double)P.p_floor);
        const double s = fmax(e_lab + p, 1e-30);
        return V4<float>{(float)(zx / s), (float)(zy / s), (float)(zz / s), (float)p};
    }
}

// ---------------------------------------------------------------------------
//  Perturbation form: the fluid energy is stored as E - e_bg (e_bg = e_ref)
// ---------------------------------------------------------------------------
// For weak transitions the fluid's departure from the background is a small
// signal on an O(1) E, and FP32 totals lose its digits.  Storing E - e_bg
// keeps them.  p = (E^2 - Z^2) / (E + s), s = sqrt(4E^2 - 3Z^2), equals
// E/3 - Z^2 / (s + 2E) exactly, so with p_bg = e_bg/3
//     p - p_bg = (E - e_bg)/3 - Z^2 / (s + 2E),
// in which the background cancels analytically; E itself is needed only in
// the small Z^2 term and in E + p.  The primitive's w component is p - p_bg,
// and the floors in LatticeParams hold e_floor - e_bg and p_floor - p_bg.
template <typename R, bool FAST>
BUBBLE_DEV V4<R> prim_from_cons_pert(const V4<R> &u, const LatticeParams<R> &P) {
    const R de = vmax(u.x, P.e_floor);
    const R e_lab = P.e_bg + de;
    R zx = u.y, zy = u.z, zz = u.w;
    const R zcap = P.z_max * e_lab;
    if constexpr (FAST) {
        // explicit roundings, as prim_from_cons<FAST>: same bits at every call site
        R z2 = dot3_rn(zx, zy, zz);
        if (z2 > __fmul_rn(zcap, zcap)) {
            const R sc = __fmul_rn(zcap, rsqrt_approx(z2));
            zx = __fmul_rn(zx, sc);
            zy = __fmul_rn(zy, sc);
            zz = __fmul_rn(zz, sc);
            z2 = dot3_rn(zx, zy, zz);
        }
        const R sq = sqrt_approx(vmax(__fmaf_rn(__fmul_rn(R(4.0), e_lab), e_lab, __fmul_rn(R(-3.0), z2)), R(0.0)));
        R dp = __fmaf_rn(de, R(1.0 / 3.0), -__fmul_rn(z2, rcp_approx(__fmaf_rn(R(2.0), e_lab, sq))));
        dp = vmax(dp, P.p_floor);
        const R inv = rcp_approx(vmax(__fadd_rn(__fadd_rn(e_lab, P.p_bg), dp), R(1e-30)));
        return V4<R>{__fmul_rn(zx, inv), __fmul_rn(zy, inv), __fmul_rn(zz, inv), dp};
    } else {
        const R zlen = sqrt(zx * zx + zy * zy + zz * zz);
        if (zlen > zcap) {
            const R sc = zcap / vmax(zlen, R(1e-30));
            zx = zx * sc;
            zy = zy * sc;
            zz = zz * sc;
        }
        const R z2 = zx * zx + zy * zy + zz * zz;
        const R sq = sqrt(vmax(R(4.0) * e_lab * e_lab - R(3.0) * z2, R(0.0)));
        R dp = de / R(3.0) - z2 / (sq + R(2.0) * e_lab);
        dp = vmax(dp, P.p_floor);
        const R d = vmax(e_lab + P.p_bg + dp, R(1e-30));
        return V4<R>{zx / d, zy / d, zz / d, dp};
    }
}

// FP64 recovery of one FP32 cell in the perturbation form (gamma > 3),
// compiled like prim_from_cons_f64.
template <bool FAST = false>
BUBBLE_F64_RECOVERY_LINKAGE V4<float> prim_from_cons_pert_f64_x(V4<float> u, float e_floor, float z_max, float p_floor,
                                                            float e_bg, float p_bg);
template <bool FAST = false>
BUBBLE_DEV V4<float> prim_from_cons_pert_f64(const V4<float> &u, const LatticeParams<float> &P) {
    return prim_from_cons_pert_f64_x<FAST>(u, P.e_floor, P.z_max, P.p_floor, P.e_bg, P.p_bg);
}
template <bool FAST>
BUBBLE_F64_RECOVERY_LINKAGE V4<float> prim_from_cons_pert_f64_x(V4<float> u, float e_floor_f, float z_max_f,
                                                            float p_floor_f, float e_bg_f, float p_bg_f) {
    struct {
        float e_floor, z_max, p_floor, e_bg, p_bg;
    } P{e_floor_f, z_max_f, p_floor_f, e_bg_f, p_bg_f};
    const double de = fmax((double)u.x, (double)P.e_floor);
    const double e_lab = (double)P.e_bg + de;
    double zx = u.y, zy = u.z, zz = u.w;
    if constexpr (FAST) {
        // explicit roundings, so every call site computes the same bits
        const double zcap = __dmul_rn((double)P.z_max, e_lab);
        const double zlen = __dsqrt_rn(dot3_rn(zx, zy, zz));
        if (zlen > zcap) {
            const double sc = __ddiv_rn(zcap, fmax(zlen, 1e-30));
            zx = __dmul_rn(zx, sc);
            zy = __dmul_rn(zy, sc);
            zz = __dmul_rn(zz, sc);
        }
        const double z2 = dot3_rn(zx, zy, zz);
        const double sq = __dsqrt_rn(fmax(__fma_rn(__dmul_rn(4.0, e_lab), e_lab, __dmul_rn(-3.0, z2)), 0.0));
        double dp = __dsub_rn(__ddiv_rn(de, 3.0), __ddiv_rn(z2, __fma_rn(2.0, e_lab, sq)));
        dp = fmax(dp, (double)P.p_floor);
        const double d = fmax(__dadd_rn(__dadd_rn(e_lab, (double)P.p_bg), dp), 1e-30);
        return V4<float>{(float)__ddiv_rn(zx, d), (float)__ddiv_rn(zy, d), (float)__ddiv_rn(zz, d), (float)dp};
    } else {
        const double zcap = (double)P.z_max * e_lab;
        const double zlen = sqrt(zx * zx + zy * zy + zz * zz);
        if (zlen > zcap) {
            const double sc = zcap / fmax(zlen, 1e-30);
            zx *= sc;
            zy *= sc;
            zz *= sc;
        }
        const double z2 = zx * zx + zy * zy + zz * zz;
        const double sq = sqrt(fmax(4.0 * e_lab * e_lab - 3.0 * z2, 0.0));
        double dp = de / 3.0 - z2 / (sq + 2.0 * e_lab);
        dp = fmax(dp, (double)P.p_floor);
        const double d = fmax(e_lab + (double)P.p_bg + dp, 1e-30);
        return V4<float>{(float)(zx / d), (float)(zy / d), (float)(zz / d), (float)dp};
    }
}

// ---------------------------------------------------------------------------
//  Gamma-law equation of state e = p / (Gamma - 1) + e0 (docs/EOS.md:86-118)
// ---------------------------------------------------------------------------
// c_s^2 = dp/de = Gamma - 1 (P.eos_c2), w = e + p = p / c2 + p + e0.  With
// s = E + p the closure leaves f(p) = p - c2 (E - Z^2 / s - e0) = 0, monotone
// (f' = 1 - c2 Z^2 / s^2 > 0 for |Z| < E), solved by a fixed eight Newton
// steps from the Z = 0 root c2 (E - e0), floored at p_floor after each step:
// a fixed count, so no cell can stall its warp.  Gamma = 4/3, e0 = 0 is the
// bag model.
constexpr int kGammaNewtonSteps = 8;

template <typename R>
BUBBLE_DEV R gamma_enthalpy(R p, const LatticeParams<R> &P) {
    return p / P.eos_c2 + p + P.eos_e0;
}

template <typename R, bool FAST>
BUBBLE_DEV V4<R> prim_from_cons_gamma(const V4<R> &u, const LatticeParams<R> &P) {
    const R e_lab = vmax(u.x, P.e_floor);
    R zx = u.y, zy = u.z, zz = u.w;
    const R zcap = P.z_max * e_lab;
    const R zlen = sqrt(zx * zx + zy * zy + zz * zz);
    if (zlen > zcap) {
        const R sc = zcap / vmax(zlen, R(1e-30));
        zx = zx * sc;
        zy = zy * sc;
        zz = zz * sc;
    }
    const R z2 = zx * zx + zy * zy + zz * zz;
    const R c2 = P.eos_c2;
    R p = vmax(c2 * (e_lab - P.eos_e0), P.p_floor);
#pragma unroll
    for (int it = 0; it < kGammaNewtonSteps; ++it) {
        const R sp = e_lab + p;
        if constexpr (FAST) {
            const R inv = rcp_approx(sp);
            const R r = p - c2 * (e_lab - z2 * inv - P.eos_e0);
            const R d = R(1.0) - c2 * z2 * (inv * inv);
            p = vmax(p - r * rcp_approx(d), P.p_floor);
        } else {
            const R r = p - c2 * (e_lab - z2 / sp - P.eos_e0);
            const R d = R(1.0) - c2 * z2 / (sp * sp);
            p = vmax(p - r / d, P.p_floor);
        }
    }
    const R d = vmax(e_lab + p, R(1e-30));
    return V4<R>{zx / d, zy / d, zz / d, p};
}

// ---------------------------------------------------------------------------
//  Thermal potential (docs/EOS.md:120-150, shaders/potential.wgsl:29-37)
// ---------------------------------------------------------------------------
// V(phi, T) = V(phi) + gamma/2 (T^2 - T_ref^2) phi^2 - A/3 (T - T_ref) phi^3
// equals the reference's V(phi) at T = T_ref, and is the finite-temperature
// form gamma/2 (T^2 - T0^2) phi^2 - A/3 T phi^3 + lambda/4 phi^4 of the
// reference's recipe when A = delta / T_ref and gamma T0^2 = gamma T_ref^2 - m2.
// The field keeps the zero-temperature part V(phi, 0); the plasma carries
// dV = gamma/2 T^2 phi^2 - A/3 T phi^3 in its free energy:
//     p(T, phi) = a/3 T^4 - dV,   e = T dp/dT - p = a T^4 - gamma/2 T^2 phi^2,
//     c_s^2 = (dp/dT) / (de/dT)   (at fixed phi),
// and d(dV)/dphi passes between field and plasma the way the friction does
// (dE += dV' pi, dZ -= dV' grad phi), so the conserved total is
// 1/2 pi^2 + 1/2 |grad phi|^2 + V(phi, 0) + E.  On the physical branch
// T >= th_lo |phi| (th_lo = sqrt(3 gamma / (4a))), e, de/dT and, for A >= 0
// and phi >= 0, dp/dT are positive and p(T) is convex, so the inversions
// below are fixed Newton counts with floors, like the gamma law's.
constexpr int kThermalNewtonSteps = 8;

template <typename R>
BUBBLE_DEV R thermal_pressure(R T, R phi, const LatticeParams<R> &P) {
    const R t2 = T * T, f2 = phi * phi;
    return P.th_k * (t2 * t2) - (R(0.5) * P.th_g) * (t2 * f2) + P.th_h * (T * (f2 * phi));
}
template <typename R>
BUBBLE_DEV R thermal_energy(R T, R phi, const LatticeParams<R> &P) {
    const R t2 = T * T;
    return P.a_rad * (t2 * t2) - (R(0.5) * P.th_g) * (t2 * (phi * phi));
}
// c_s^2 = (dp/dT) / (de/dT), held in [1e-4, 1] (an outer bound for HLL off the branch)
template <typename R, bool FAST>
BUBBLE_DEV R thermal_cs2(R T, R phi, const LatticeParams<R> &P) {
    const R t2 = T * T, f2 = phi * phi;
    const R dp = T * (R(4.0) * P.th_k * t2 - P.th_g * f2) + P.th_h * (f2 * phi);
    const R de = vmax(T * (R(4.0) * P.a_rad * t2 - P.th_g * f2), R(1e-30));
    R c2;
    if constexpr (FAST) c2 = dp * rcp_approx(de);
    else c2 = dp / de;
    return vmin(vmax(c2, R(1e-4)), R(1.0));
}
// eos_temperature(p, phi): the root of p(T, phi) = p from the phi = 0 root,
// each step held to [max(T_lo, T/2), 2T].
template <typename R, bool FAST>
BUBBLE_DEV R thermal_temperature(R p, R phi, const LatticeParams<R> &P) {
    const R pp = vmax(p, P.p_floor);
    const R lo = P.th_lo * fabs(phi);
    const R f2 = phi * phi, h = P.th_h * (f2 * phi);
    R T;
    if constexpr (FAST) T = vmax(sqrt_approx(sqrt_approx(pp * rcp_approx(P.th_k))), lo);
    else T = vmax(sqrt(sqrt(pp / P.th_k)), lo);
#pragma unroll
    for (int it = 0; it < kThermalNewtonSteps; ++it) {
        const R t2 = T * T;
        const R g = P.th_k * (t2 * t2) - (R(0.5) * P.th_g) * (t2 * f2) + P.th_h * (T * (f2 * phi)) - pp;
        const R d = vmax(T * (R(4.0) * P.th_k * t2 - P.th_g * f2) + h, R(1e-30));
        R tn;
        if constexpr (FAST) tn = T - g * rcp_approx(d);
        else tn = T - g / d;
        T = vmin(vmax(tn, vmax(lo, R(0.5) * T)), R(2.0) * T);
    }
    return T;
}
// dV/dphi of the thermal potential at (phi, T) and its plasma part d(dV)/dphi
template <typename R>
BUBBLE_DEV R thermal_dpotential(R phi, R T, const LatticeParams<R> &P) {
    return dpotential(phi, P) + phi * (P.th_g * (T * T - P.t_ref * P.t_ref) - P.th_a * ((T - P.t_ref) * phi));
}
template <typename R>
BUBBLE_DEV R thermal_exchange(R phi, R T, const LatticeParams<R> &P) {
    return phi * (P.th_g * (T * T) - P.th_a * (T * phi));
}
// V(phi, 0), the field's share of the potential (diagnostics)
template <typename R>
BUBBLE_DEV R thermal_potential0(R phi, const LatticeParams<R> &P) {
    const R f2 = phi * phi;
    return potential(phi, P) + f2 * (P.th_h * (P.t_ref * phi) - (R(0.5) * P.th_g) * (P.t_ref * P.t_ref));
}
// con2prim: f(p) = p - p(T(e), phi) = 0 with e = E - Z^2 / (E + p) and
// T^2 = (gamma/2 phi^2 + sqrt((gamma/2 phi^2)^2 + 4 a e)) / (2a), the root of
// e(T) = e on the branch; f' = 1 - c_s^2 Z^2 / (E + p)^2 > 0.
template <typename R, bool FAST>
BUBBLE_DEV V4<R> prim_from_cons_thermal(const V4<R> &u, R phi, const LatticeParams<R> &P) {
    const R e_lab = vmax(u.x, P.e_floor);
    R zx = u.y, zy = u.z, zz = u.w;
    const R zcap = P.z_max * e_lab;
    const R zlen = sqrt(zx * zx + zy * zy + zz * zz);
    if (zlen > zcap) {
        const R sc = zcap / vmax(zlen, R(1e-30));
        zx = zx * sc;
        zy = zy * sc;
        zz = zz * sc;
    }
    const R z2 = zx * zx + zy * zy + zz * zz;
    const R f2 = phi * phi;
    const R g = (R(0.5) * P.th_g) * f2;
    const R h = P.th_h * (f2 * phi);
    const R a4 = R(4.0) * P.a_rad;
    R X = (g + sqrt(g * g + a4 * e_lab)) * P.th_i2a;
    R p = vmax(P.th_k * (X * X) - g * X + h * sqrt(X), P.p_floor);
#pragma unroll
    for (int it = 0; it < kThermalNewtonSteps; ++it) {
        const R sp = e_lab + p;
        R e, c2, r, d;
        if constexpr (FAST) {
            const R isp = rcp_approx(sp);
            e = e_lab - z2 * isp;
            X = (g + sqrt_approx(g * g + a4 * e)) * P.th_i2a;
            const R T = sqrt_approx(X);
            const R dp = T * (R(4.0) * P.th_k * X - P.th_g * f2) + h;
            const R de = vmax(T * (a4 * X - P.th_g * f2), R(1e-30));
            c2 = vmin(vmax(dp * rcp_approx(de), R(1e-4)), R(1.0));
            r = p - (P.th_k * (X * X) - g * X + h * T);
            d = R(1.0) - c2 * z2 * (isp * isp);
            p = vmax(p - r * rcp_approx(d), P.p_floor);
        } else {
            e = e_lab - z2 / sp;
            X = (g + sqrt(g * g + a4 * e)) * P.th_i2a;
            const R T = sqrt(X);
            const R dp = T * (R(4.0) * P.th_k * X - P.th_g * f2) + h;
            const R de = vmax(T * (a4 * X - P.th_g * f2), R(1e-30));
            c2 = vmin(vmax(dp / de, R(1e-4)), R(1.0));
            r = p - (P.th_k * (X * X) - g * X + h * T);
            d = R(1.0) - c2 * z2 / (sp * sp);
            p = vmax(p - r / d, P.p_floor);
        }
    }
    const R dd = vmax(e_lab + p, R(1e-30));
    return V4<R>{zx / dd, zy / dd, zz / dd, p};
}

// Forms of a lattice (the FORM parameter of the kernels): the bag model in
// plain FP32; mixed = FP64 primitive recovery where the Lorentz factor
// exceeds 3; perturbation = mixed, with E stored as E - e_bg; gamma = the
// gamma-law equation of state in plain arithmetic; thermal = the thermal
// potential's plasma in plain arithmetic (its EOS depends on phi).
constexpr int kPlain = 0, kMixed = 1, kPert = 2, kGamma = 3, kThermal = 4;

// `phi` is the cell's field value; only the thermal form's EOS reads it.
template <typename R, bool FAST, int MODE>
BUBBLE_DEV V4<R> recover(const V4<R> &u, const LatticeParams<R> &P, R phi = R(0)) {
    if constexpr (MODE == kThermal) {
        return prim_from_cons_thermal<R, FAST>(u, phi, P);
    } else if constexpr (MODE == kGamma) {
        return prim_from_cons_gamma<R, FAST>(u, P);
    } else if constexpr (MODE == kPert) {
        V4<R> q = prim_from_cons_pert<R, FAST>(u, P);
        if constexpr (sizeof(R) == 4) {
            const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
            if (v2 > R(8.0) / R(9.0)) q = prim_from_cons_pert_f64<FAST>(u, P);
        }
        return q;
    } else {
        V4<R> q = prim_from_cons<R, FAST>(u, P);
        if constexpr (MODE == kMixed) {
            const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
            if (v2 > R(8.0) / R(9.0)) q = prim_from_cons_f64<FAST>(u, P);
        }
        return q;
    }
}

// ---------------------------------------------------------------------------
//  sanitise (shaders/step.wgsl:61-72)
// ---------------------------------------------------------------------------
template <typename R>
BUBBLE_DEV V4<R> sanitise(const V4<R> &q, R p_floor, R vmax2) {
    const R p = vmax(q.w, p_floor);
    R vx = q.x, vy = q.y, vz = q.z;
    const R v2 = vx * vx + vy * vy + vz * vz;
    if (v2 > vmax2) {
        const R s = sqrt(vmax2 / vmax(v2, R(1e-30)));
        vx = vx * s;
        vy = vy * s;
        vz = vz * s;
    }
    return V4<R>{vx, vy, vz, p};
}

// sanitise(recover(u)) of one staged cell.  The fast bag and perturbation
// forms reuse the |v|^2 of the Lorentz-factor test for the clamp (the same
// values) and round explicitly, so the chunk prologue and the z-march give
// the same bits.
template <typename R, bool FAST, int MODE>
BUBBLE_DEV V4<R> recover_sanitised(const V4<R> &u, const LatticeParams<R> &P, R phi, R vmax2) {
    if constexpr (FAST && sizeof(R) == 4 && (MODE == kPlain || MODE == kMixed || MODE == kPert)) {
        V4<R> q = MODE == kPert ? prim_from_cons_pert<R, FAST>(u, P) : prim_from_cons<R, FAST>(u, P);
        R v2 = dot3_rn(q.x, q.y, q.z);
        if constexpr (MODE == kMixed || MODE == kPert) {
            if (v2 > R(8.0) / R(9.0)) {
                q = MODE == kPert ? prim_from_cons_pert_f64<true>(u, P) : prim_from_cons_f64<true>(u, P);
                v2 = dot3_rn(q.x, q.y, q.z);
            }
        }
        q.w = vmax(q.w, P.p_floor);
        if (v2 > vmax2) {
            const R s = __fsqrt_rn(__fdiv_rn(vmax2, vmax(v2, R(1e-30))));
            q.x = __fmul_rn(q.x, s);
            q.y = __fmul_rn(q.y, s);
            q.z = __fmul_rn(q.z, s);
        }
        return q;
    } else {
        return sanitise(recover<R, FAST, MODE>(u, P, phi), P.p_floor, vmax2);
    }
}

template <typename R>
BUBBLE_DEV V4<R> v4_sub(const V4<R> &a, const V4<R> &b) {
    return V4<R>{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w};
}

// limit_slope4 (shaders/common.wgsl:129-136).
template <typename R, bool FAST = false>
BUBBLE_DEV V4<R> limit_slope4(const V4<R> &dm, const V4<R> &dp) {
    return V4<R>{limit_slope<R, FAST>(dm.x, dp.x), limit_slope<R, FAST>(dm.y, dp.y),
                 limit_slope<R, FAST>(dm.z, dp.z), limit_slope<R, FAST>(dm.w, dp.w)};
}

// q + 0.5 s and q - 0.5 s (shaders/step.wgsl:135-144).
template <typename R>
BUBBLE_DEV V4<R> half_step(const V4<R> &q, const V4<R> &s, R sign) {
    // sign is +1 or -1; multiplying by it is exact, so this equals q +- 0.5 s.
    return V4<R>{q.x + sign * (R(0.5) * s.x), q.y + sign * (R(0.5) * s.y),
                 q.z + sign * (R(0.5) * s.z), q.w + sign * (R(0.5) * s.w)};
}

// The two sanitised face states of a cell along one axis from its
// neighbours qm, qp: lo = q - s/2 (face i-1/2), hi = q + s/2 (face i+1/2),
// s the MC-limited slope (shaders/step.wgsl:125-144).  The fast states floor
// the pressure only; their velocity clamp happens in face_side<FAST>.
template <typename R, bool FAST>
BUBBLE_DEV void face_states(const V4<R> &qm, const V4<R> &q, const V4<R> &qp, R p_floor, R vmax2, V4<R> &lo,
                            V4<R> &hi) {
    if constexpr (FAST && sizeof(R) == 4) {
        const float2 qa = lo2(q), qb = hi2(q);
        const float2 dma = p_sub(qa, lo2(qm)), dmb = p_sub(qb, hi2(qm));
        const float2 dpa = p_sub(lo2(qp), qa), dpb = p_sub(hi2(qp), qb);
        const float2 ha = p_mul(p_add(dma, dpa), bc2(0.5f)), hb = p_mul(p_add(dmb, dpb), bc2(0.5f));
        const float2 pa = p_mul(dma, dpa), pb = p_mul(dmb, dpb);
        const float2 ma = p_mul(make_float2(fminf(fabsf(dma.x), fabsf(dpa.x)), fminf(fabsf(dma.y), fabsf(dpa.y))),
                                bc2(2.0f));
        const float2 mb = p_mul(make_float2(fminf(fabsf(dmb.x), fabsf(dpb.x)), fminf(fabsf(dmb.y), fabsf(dpb.y))),
                                bc2(2.0f));
        const float2 sa = make_float2(pa.x > 0.0f ? copysignf(fminf(fabsf(ha.x), ma.x), dma.x) : 0.0f,
                                      pa.y > 0.0f ? copysignf(fminf(fabsf(ha.y), ma.y), dma.y) : 0.0f);
        const float2 sb = make_float2(pb.x > 0.0f ? copysignf(fminf(fabsf(hb.x), mb.x), dmb.x) : 0.0f,
                                      pb.y > 0.0f ? copysignf(fminf(fabsf(hb.y), mb.y), dmb.y) : 0.0f);
        // pressure floor only: face_side<FAST> applies the velocity clamp
        lo = v4of(p_fma(sa, bc2(-0.5f), qa), p_fma(sb, bc2(-0.5f), qb));
        hi = v4of(p_fma(sa, bc2(0.5f), qa), p_fma(sb, bc2(0.5f), qb));
        lo.w = vmax(lo.w, p_floor);
        hi.w = vmax(hi.w, p_floor);
    } else {
        const V4<R> s = limit_slope4<R, FAST>(v4_sub(q, qm), v4_sub(qp, q));
        lo = sanitise(half_step(q, s, R(-1)), p_floor, vmax2);
        hi = sanitise(half_step(q, s, R(1)), p_floor, vmax2);
    }
}

// ---------------------------------------------------------------------------
//  HLL face flux (shaders/step.wgsl:74-90 with eos.wgsl:129-176)
// ---------------------------------------------------------------------------
template <int AXIS, typename R>
BUBBLE_DEV R comp(const V4<R> &q) {
    if constexpr (AXIS == 0) return q.x;
    else if constexpr (AXIS == 1) return q.y;
    else return q.z;
}

// Per-side quantities of the HLL solver for one sanitised face state.
template <typename R>
struct FaceSide {
    V4<R> u;     // eos_cons_from_prim
    V4<R> f;     // eos_flux along the axis
    R lm, lp;    // eos_wave_speeds
};

// PERT: q.w is p - p_bg, the energy component of u is E - e_bg = w v^2 + 3 (p - p_bg)
// (w = 4p W^2, e_bg = 3 p_bg), and the momentum flux carries p - p_bg: the
// constant p_bg would cancel in every flux difference.
// GAMMA (FORM kGamma): w = p / c2 + p + e0 and the general wave speeds
// with c_s^2 = c2; E = w W^2 - p and the fluxes as for the bag model.
// THERMAL (FORM kThermal): w = e(T, phi) + p with T = eos_temperature(p, phi)
// and c_s^2(T, phi), phi the field value of the state's own cell.
template <int AXIS, typename R, bool FAST, int FORM = kPlain>
BUBBLE_DEV FaceSide<R> face_side(const V4<R> &q, R zmax2, const LatticeParams<R> &P, R phi = R(0)) {
    constexpr bool PERT = FORM == kPert;
    FaceSide<R> s;
    R vx = q.x, vy = q.y, vz = q.z;
    const R p = q.w;
    // The fast forms round explicitly wherever the compiler could contract
    // differently at the chunk prologue's and the z-march's call sites.
    R v2raw;
    if constexpr (FAST && sizeof(R) == 4) v2raw = dot3_rn(vx, vy, vz);
    else v2raw = vx * vx + vy * vy + vz * vz;
    if constexpr (FAST) {
        // The velocity half of sanitise (shaders/step.wgsl:61-72): the fast
        // face states floor only the pressure and leave the velocity clamp to
        // this point, where |v|^2 is needed anyway (same values, one |v|^2
        // per face state instead of two).
        if (v2raw > zmax2) {
            const R sc = sqrt(zmax2 / vmax(v2raw, R(1e-30)));
            vx = vx * sc;
            vy = vy * sc;
            vz = vz * sc;
            v2raw = dot3_rn(vx, vy, vz);
        }
    }
    const R v2 = vmin(v2raw, zmax2);
    const R vd = AXIS == 0 ? vx : (AXIS == 1 ? vy : vz);
    if constexpr (FORM == kGamma || FORM == kThermal) {
        R cs2, enth;
        if constexpr (FORM == kThermal) {
            const R T = thermal_temperature<R, FAST>(p, phi, P);
            enth = thermal_energy(T, phi, P) + p;
            cs2 = thermal_cs2<R, FAST>(T, phi, P);
        } else {
            enth = gamma_enthalpy(p, P);
            cs2 = P.eos_c2;
        }
        R w, den_inv;
        if constexpr (FAST) {
            w = enth * rcp_approx(R(1.0) - v2);
            den_inv = rcp_approx(R(1.0) - v2 * cs2);
        } else {
            w = enth / (R(1.0) - v2);
        }
        s.u = V4<R>{w - p, w * vx, w * vy, w * vz};
        const R cs = sqrt(cs2);
        const R rad = vmax((R(1.0) - v2) * (R(1.0) - vd * vd - cs2 * (v2 - vd * vd)), R(0.0));
        if constexpr (FAST) {
            const R a = vd * (R(1.0) - cs2) * den_inv;
            const R b = cs * sqrt_approx(rad) * den_inv;
            s.lm = a - b;
            s.lp = a + b;
        } else {
            const R denom = R(1.0) - v2 * cs2;
            const R a = vd * (R(1.0) - cs2) / denom;
            const R b = cs * sqrt(rad) / denom;
            s.lm = a - b;
            s.lp = a + b;
        }
        s.f = V4<R>{(s.u.x + p) * vd, s.u.y * vd, s.u.z * vd, s.u.w * vd};
        if constexpr (AXIS == 0) s.f.y = s.f.y + p;
        if constexpr (AXIS == 1) s.f.z = s.f.z + p;
        if constexpr (AXIS == 2) s.f.w = s.f.w + p;
        return s;
    }
    const R pf = PERT ? P.p_bg + p : p;  // the full pressure
    const R cs2 = R(1.0) / R(3.0);  // eos_sound_speed2 (eos.wgsl:50-53)
    if constexpr (FAST) {
        // 1 - vd^2 - cs2 (v^2 - vd^2) = 1 - (2/3) vd^2 - v^2/3 for cs2 = 1/3;
        // E + p = w W^2, so the energy flux is w vd.
        const R om = R(1.0) - v2;
        const R w = (R(4.0) * pf) * rcp_approx(om);
        {
            const float2 uzw = p_mul(bc2(w), make_float2(vy, vz));
            s.u = V4<R>{PERT ? __fmaf_rn(w, v2, __fmul_rn(R(3.0), p)) : w - p, w * vx, uzw.x, uzw.y};
        }
        const R inv_den = rcp_approx(__fmaf_rn(-v2, cs2, R(1.0)));
        const R tt = __fmaf_rn(-cs2, v2, __fmaf_rn(-(R(2.0) / R(3.0)), __fmul_rn(vd, vd), R(1.0)));
        const R rad = vmax(om * tt, R(0.0));
        const R cs = R(0.57735026918962576451);
        const R a = vd * ((R(2.0) / R(3.0)) * inv_den);
        const R b = cs * sqrt_approx(rad) * inv_den;
        s.lm = a - b;
        s.lp = a + b;
        s.f = v4of(p_mul(make_float2(w, s.u.y), bc2(vd)), p_mul(hi2(s.u), bc2(vd)));
        if constexpr (AXIS == 0) s.f.y = s.f.y + p;
        if constexpr (AXIS == 1) s.f.z = s.f.z + p;
        if constexpr (AXIS == 2) s.f.w = s.f.w + p;
        return s;
    } else {
        const R w = R(4.0) * pf / (R(1.0) - v2);
        s.u = V4<R>{PERT ? w * v2 + R(3.0) * p : w - p, w * vx, w * vy, w * vz};
        const R cs = sqrt(cs2);
        const R denom = R(1.0) - v2 * cs2;
        const R rad = vmax((R(1.0) - v2) * (R(1.0) - vd * vd - cs2 * (v2 - vd * vd)), R(0.0));
        const R a = vd * (R(1.0) - cs2) / denom;
        const R b = cs * sqrt(rad) / denom;
        s.lm = a - b;
        s.lp = a + b;
        // energy flux (E + p) v_d = w v_d; the reference's order for the plain form
        s.f = V4<R>{PERT ? w * vd : (s.u.x + p) * vd, s.u.y * vd, s.u.z * vd, s.u.w * vd};
    }
    if constexpr (AXIS == 0) s.f.y = s.f.y + p;
    if constexpr (AXIS == 1) s.f.z = s.f.z + p;
    if constexpr (AXIS == 2) s.f.w = s.f.w + p;
    return s;
}

// hll_flux(q_l, phi_l, q_r, phi_r, axis).  The phi arguments reach only the
// EOS functions; the forms whose EOS ignores phi pass 0.
template <int AXIS, typename R, bool FAST, int FORM = kPlain>
BUBBLE_DEV V4<R> hll_flux(const V4<R> &ql, const V4<R> &qr, R zmax2, const LatticeParams<R> &P, R phi_l = R(0),
                          R phi_r = R(0)) {
    const FaceSide<R> L = face_side<AXIS, R, FAST, FORM>(ql, zmax2, P, phi_l);
    const FaceSide<R> Rt = face_side<AXIS, R, FAST, FORM>(qr, zmax2, P, phi_r);
    const R s_min = vmin(vmin(L.lm, Rt.lm), R(0.0));
    const R s_max = vmax(vmax(L.lp, Rt.lp), R(0.0));
    const R den = vmax(s_max - s_min, R(1e-12));
    const R smm = s_min * s_max;
    if constexpr (FAST) {
        const R inv = rcp_approx(den);
        float2 a = p_mul(bc2(smm), p_sub(lo2(Rt.u), lo2(L.u)));
        float2 b = p_mul(bc2(smm), p_sub(hi2(Rt.u), hi2(L.u)));
        a = p_fma(bc2(-s_min), lo2(Rt.f), p_fma(bc2(s_max), lo2(L.f), a));
        b = p_fma(bc2(-s_min), hi2(Rt.f), p_fma(bc2(s_max), hi2(L.f), b));
        return v4of(p_mul(a, bc2(inv)), p_mul(b, bc2(inv)));
    } else {
        return V4<R>{(s_max * L.f.x - s_min * Rt.f.x + smm * (Rt.u.x - L.u.x)) / den,
                     (s_max * L.f.y - s_min * Rt.f.y + smm * (Rt.u.y - L.u.y)) / den,
                     (s_max * L.f.z - s_min * Rt.f.z + smm * (Rt.u.z - L.u.z)) / den,
                     (s_max * L.f.w - s_min * Rt.f.w + smm * (Rt.u.w - L.u.w)) / den};
    }
}

// ---------------------------------------------------------------------------
//  SSP-RK3 stage combine a0 U^n + a1 U1 (shaders/step.wgsl:170-173)
// ---------------------------------------------------------------------------
// In binary32 fl(1/3) + fl(2/3) = 1 + 2^-25, so the reference's form is that
// much too large before rounding on the third stage; over evolving cells the
// rounding is unbiased and the mean keeps the excess: a systematic energy
// drift of about 3e-8 per step that the FP64 scheme does not have (measured:
// 3.2e-5 of excess drift over 1300 steps at 128^3, 7e-5 over 2900 at 256^3).  The
// fast arithmetic evaluates U^n + a1 (U1 - U^n), whose weights sum to 1
// exactly; the strict arithmetic keeps the reference's expression, for bit
// parity with the oracle.
template <typename R, bool FAST>
BUBBLE_DEV R rk_combine(R a0, R a1, R un, R u1) {
    if constexpr (FAST) return un + a1 * (u1 - un);
    else return a0 * un + a1 * u1;
}

// ---------------------------------------------------------------------------
//  Deterministic tanh for the nucleation profile
// ---------------------------------------------------------------------------
// tanh(x) = expm1(2|x|) / (expm1(2|x|) + 2) with the sign of x, expm1 from a
// Taylor series near zero and otherwise from Cody-Waite range reduction by
// ln 2 (split into the classic high/low parts) and a Taylor polynomial for
// exp(r), |r| <= ln2/2, scaled by an exact power of two.  Evaluated in FP64
// with plain IEEE operations only, so a CPU and a GPU build without FMA
// contraction return identical bits; the FP32 result is the FP64 value
// rounded once.  Relative error of the FP64 value is below 1e-15.
BUBBLE_HD double pow2_int(int k) {
    // k in [0, 1023]
    const unsigned long long bits = (unsigned long long)(k + 1023) << 52;
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)bits);
#else
    double d;
    __builtin_memcpy(&d, &bits, sizeof(d));
    return d;
#endif
}

BUBBLE_HD double det_expm1_nonneg(double y) {
    if (y < 0.5) {
        double r = 1.0;
        for (int k = 18; k >= 2; --k) r = 1.0 + y * r / (double)k;
        return y * r;
    }
    const double inv_ln2 = 1.44269504088896338700e+00;
    const double ln2_hi = 6.93147180369123816490e-01;
    const double ln2_lo = 1.90821492927058770002e-10;
    const double kf = floor(y * inv_ln2 + 0.5);
    const double r = (y - kf * ln2_hi) - kf * ln2_lo;
    double e = 1.0;
    for (int k = 16; k >= 1; --k) e = 1.0 + r * e / (double)k;
    return e * pow2_int((int)kf) - 1.0;
}

BUBBLE_HD double det_tanh(double x) {
    const double ax = fabs(x);
    double t;
    if (ax > 22.0) {
        t = 1.0;
    } else {
        const double em = det_expm1_nonneg(2.0 * ax);
        t = em / (em + 2.0);
    }
    return x < 0.0 ? -t : t;
}

// Cut-off beyond which the profile is exactly zero: det_tanh rounds to 1.
template <typename R>
struct TanhCut;
template <>
struct TanhCut<float> {
    static constexpr float value = 9.5f;
};
template <>
struct TanhCut<double> {
    static constexpr double value = 22.0;
};

// Deterministic FP32 tanh of the FP32 nucleation profile:
// tanh|x| = m / (m + 2) with m = expm1(2|x|); expm1(y) from its Taylor series
// to y^8/8! for y < ln2/2, else by Cody-Waite reduction y = k ln2 + r (ln2 split
// so that k ln2_hi is exact) as 2^k expm1(r) + (2^k - 1).  Only IEEE +, -, *,
// / rounded to nearest (explicit on the device, so no FMA contraction whatever
// the flags) and exact operations (rint, ldexp, copysign): the CPU oracle gets
// the same bits.  Beyond |x| = 9.5 it returns +-1 exactly, which is what a
// correctly rounded tanhf returns there (1 - tanh(9.5) < 2^-25).  Error below
// 4 ulp against libm (tested).
BUBBLE_HD float f32_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
BUBBLE_HD float f32_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
BUBBLE_HD float f32_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
BUBBLE_HD float expm1_taylor_f32(float y) {
    float t = 2.48015873e-05f;  // 1/8!
    t = f32_add(1.98412698e-04f, f32_mul(y, t));
    t = f32_add(1.38888889e-03f, f32_mul(y, t));
    t = f32_add(8.33333333e-03f, f32_mul(y, t));
    t = f32_add(4.16666667e-02f, f32_mul(y, t));
    t = f32_add(1.66666667e-01f, f32_mul(y, t));
    t = f32_add(0.5f, f32_mul(y, t));
    t = f32_add(1.0f, f32_mul(y, t));
    return f32_mul(y, t);
}
BUBBLE_HD float det_tanh_f32(float x) {
    const float a = fabsf(x);
    if (a > 9.5f) return copysignf(1.0f, x);
    const float y = f32_add(a, a);
    float m;
    if (y < 0.346573590f) {
        m = expm1_taylor_f32(y);
    } else {
        const float k = rintf(f32_mul(y, 1.44269504f));
        const float r = f32_add(f32_add(y, -f32_mul(k, 0.693145752f)), -f32_mul(k, 1.42860677e-06f));
        const float p2 = ldexpf(1.0f, (int)k);
        m = f32_add(f32_mul(p2, expm1_taylor_f32(r)), f32_add(p2, -1.0f));
    }
    return copysignf(f32_div(m, f32_add(m, 2.0f)), x);
}

template <typename R>
BUBBLE_HD R det_tanh_r(R x) {
    if constexpr (sizeof(R) == 4) {
        return det_tanh_f32(x);
    } else {
        if (x > TanhCut<R>::value) return R(1);
        if (x < -TanhCut<R>::value) return R(-1);
        return det_tanh(x);
    }
}

// min_image (shaders/nucleate.wgsl:51-57).
template <typename R>
BUBBLE_DEV R min_image(R d, R n) {
    R r = d;
    if (r > R(0.5) * n) r = r - n;
    if (r < R(-0.5) * n) r = r + n;
    return r;
}

}  // namespace dev
}  // namespace bubble
