// Parameter blocks shared by the host driver and the CUDA kernels.
//
// LatticeParams mirrors the `SimParams` uniform (shaders/common.wgsl:25-58,
// host values src/gpu/sim.rs:613-644) minus the fields no kernel on this path
// reads (time, vis_gain, padding).  It is templated on the arithmetic type so
// the FP64 kernels get double constants (each widened exactly from the f32
// value the host derives, so both precisions solve the same problem).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define BUBBLE_HD __host__ __device__ __forceinline__
#else
#define BUBBLE_HD inline
#endif

namespace bubble {

template <typename R>
struct alignas(4 * sizeof(R)) V4 {
    R x, y, z, w;
};
template <typename R>
struct alignas(2 * sizeof(R)) V2 {
    R x, y;
};

template <typename R>
struct LatticeParams {
    int32_t nx, ny, nz, _pad;
    R dx, inv_dx, eta, lambda;
    R phi_b, m2, delta, wall_width;
    R p_floor, e_floor, z_max, e_ref;
    // Perturbation form: the background subtracted from the stored energy
    // (e_bg = e_ref) and from the pressure (p_bg = e_bg / 3); both 0, and the
    // floors unshifted, for the other forms.
    R e_bg, p_bg;
    // Gamma-law equation of state: c_s^2 = Gamma - 1 and the offset e0 of
    // e = p / (Gamma - 1) + e0; both 0 for the bag model.
    R eos_c2, eos_e0;
    // Thermal potential V(phi) + gamma/2 (T^2 - T_ref^2) phi^2 - A/3 (T - T_ref) phi^3:
    // th_k = a/3, th_g = gamma, th_h = A/3, th_a = A, th_lo = sqrt(3 gamma / (4 a))
    // (the physical branch is T >= th_lo |phi|), th_i2a = 1/(2a), the radiation
    // constant a and T_ref; all 0 for the other equations of state.
    R th_k, th_g, th_h, th_a, th_lo, th_i2a, a_rad, t_ref;
};

// One SSP-RK3 stage: U_out = a0 U^n + a1 (U_in + dt L(U_in))
// (shaders/common.wgsl:60-68, src/gpu/sim.rs:133-135, 650-656).
template <typename R>
struct StageArgs {
    const V2<R> *field_n;
    const V4<R> *fluid_n;
    const V2<R> *field_in;
    const V4<R> *fluid_in;
    V2<R> *field_out;
    V4<R> *fluid_out;
    R a0, a1, dt;
    int32_t stage;  // 0, 1, 2; stage 0 has a0 == 0 and never reads U^n
    // Bounded waits of the stage kernel give up after 2^wait_shift SM cycles.
    // Test hook (bubble_ext_test_expire_stage_wait): when test_tx != 0, every
    // CTA staging planes through TMA arms its first plane's mbarrier for
    // test_tx bytes and issues no copy for it, so that wait expires.
    uint32_t test_tx = 0;
    int32_t wait_shift = 31;
};

// Result of the diagnostics reduction (shaders/reduce.wgsl:32-38), with FP64
// sums.
struct DiagResult {
    double sums[4];       // e_total, broken, kinetic, E
    uint32_t max_v_bits;  // bits of max |v| (non-negative f32)
    uint32_t nonfinite;   // count of blocks that saw a non-finite term
    uint64_t cells;
};

// Tile shape of the fused stage kernel.
struct TileShape {
    int32_t tx, ty, lz;  // x, y tile (cells) and z chunk (planes)
    int32_t form = 0;    // BUBBLE_STAGE_FORM_* of 16 x 16 FP32 launches
};

// The stage kernel's tiles are 16 x 16 (FP32 default: the least perimeter,
// so the least halo work, for 256 column threads) or 32 x ty (ty = 8, 4):
// the tile height selects the width.
constexpr int tile_x_for(int ty) { return ty == 16 ? 16 : 32; }

// Cost model of one stage launch of the 16 x 16 FP32 column kernel, in plane
// times of a CTA that shares its SM with one other.  The register form holds
// two CTAs per SM, the shared form three, each then 1.4x slower per plane;
// the busiest SM (ceil(CTAs / SMs) CTAs) runs them in rounds, a last round
// of one CTA at 0.65x and of two (shared form) at 0.8x of the full round's
// plane time; a chunk costs its planes plus 2 for its warm-up.  Fitted to
// about 150 measured (form, chunk) pairs from 32^3 to 512^3: the cheapest
// pick (chunks of 4 planes or more) is the fastest measured or within 0.6 %
// of it at every size.
inline double column_stage_cost(uint32_t nx, uint32_t ny, uint32_t nz, int lz, bool shared, int sms) {
    if (lz < 1) lz = 1;
    if (sms < 1) sms = 1;
    const long tiles = (long)((nx + 15) / 16) * (long)((ny + 15) / 16);
    const long chunks = ((long)nz + lz - 1) / lz;
    const long lz_eff = ((long)nz + chunks - 1) / chunks;
    const long k = shared ? 3 : 2;
    const double p = shared ? 1.4 : 1.0;
    const long m = (tiles * chunks + sms - 1) / sms;
    const long rounds = (m + k - 1) / k;
    const long last = m - (rounds - 1) * k;
    const double p_last = last == k ? p : (last == 1 ? 0.65 * p : 0.8 * p);
    return ((double)(rounds - 1) * p + p_last) * (double)(lz_eff + 2);
}

}  // namespace bubble
