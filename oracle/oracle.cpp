// ORACLE -- test infrastructure only.
//
// A CPU restatement of the reference's lattice time step, used by the tests
// and by bench.py's CPU baseline as the checker.  Nothing in the product
// (the CUDA library) links, loads or calls this file.
//
// It follows the reference shaders function by function, in their
// evaluation order, templated on the arithmetic type (float restates the
// reference's f32 shaders; double is the FP64 restatement):
//   wrap1, cell_index            shaders/common.wgsl:80-95
//   minmod3, limit_slope(4)      shaders/common.wgsl:114-136
//   potential, dpotential        shaders/potential.wgsl:38-47
//   eos_*                        shaders/eos.wgsl:50-176
//   sanitise, hll_flux, main     shaders/step.wgsl:63-174
//   primitives main              shaders/primitives.wgsl:16-23
//   init main                    shaders/init.wgsl:18-26
//   nucleate main, min_image     shaders/nucleate.wgsl:51-85
//   cell_contribution, reduce    shaders/reduce.wgsl:49-140 (sums in FP64)
//   vis main                     shaders/vis.wgsl:30-55 (binary16 round to nearest even)
//   MIXED form's FP64 recovery   shaders/eos.wgsl:94-123 in FP64 where the
//                                FP32 v^2 > 8/9 (docs/PRECISION.md:150-152)
//   fs_main and helpers          shaders/volume.wgsl:80-381, with the
//                                sampler of src/gpu/render.rs:206-218
//                                (trilinear, clamp to edge) in software
// Built with -ffp-contract=off so every operation is one IEEE rounding.
// WGSL's tanh has implementation-defined accuracy; the oracle uses the
// Cody-Waite / Taylor tanh described at oracle_tanh (accurate to a few
// units in 1e-16), which the CUDA library evaluates with the same
// operations, so nucleated fields compare bit for bit.  Its FP64 relative
// error is below 1e-15 (tests/test_oracle_pins.py).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// SimParams (shaders/common.wgsl:25-58), 96 bytes in the f32 instance.
template <typename R>
struct SimParams {
    uint32_t nx, ny, nz, _pad_u0;
    R dx, inv_dx, dt, eta;
    R lambda, eps, phi_b, m2;
    R delta, a_rad, wall_width, p_floor;
    R e_floor, z_max, e_ref, t_ref;
    R time, vis_gain, _pad0, _pad1;
};
static_assert(sizeof(SimParams<float>) == 96, "SimParams is 96 bytes");

// StageParams (shaders/common.wgsl:63-68).
template <typename R>
struct StageParams {
    R a0, a1, dt_stage, _pad;
};

template <typename R>
struct vec4 {
    R x, y, z, w;
};
template <typename R>
struct vec3 {
    R x, y, z;
};

template <typename R>
inline R wmax(R a, R b) {
    return std::fmax(a, b);
}
template <typename R>
inline R wmin(R a, R b) {
    return std::fmin(a, b);
}
// WGSL sign(): 1, 0 or -1.
template <typename R>
inline R wsign(R e) {
    return e > R(0) ? R(1) : (e < R(0) ? R(-1) : R(0));
}

// ---------------------------------------------------------------------------
//  common.wgsl
// ---------------------------------------------------------------------------
inline int wrap1(int i, int n) {
    int r = i;
    if (r < 0) r += n;
    if (r < 0) r += n;
    if (r >= n) r -= n;
    if (r >= n) r -= n;
    return r;
}

template <typename R>
inline size_t cell_index(const SimParams<R> &P, int x, int y, int z) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
    const int wx = wrap1(x, nx), wy = wrap1(y, ny), wz = wrap1(z, nz);
    return ((size_t)wz * (size_t)ny + (size_t)wy) * (size_t)nx + (size_t)wx;
}

template <typename R>
inline R minmod3(R a, R b, R c) {
    const R sa = wsign(a);
    if (sa != wsign(b) || sa != wsign(c)) return R(0.0);
    return sa * wmin(std::fabs(a), wmin(std::fabs(b), std::fabs(c)));
}

template <typename R>
inline R limit_slope(R dm, R dp) {
    return minmod3(R(0.5) * (dm + dp), R(2.0) * dm, R(2.0) * dp);
}

template <typename R>
inline vec4<R> limit_slope4(vec4<R> dm, vec4<R> dp) {
    return {limit_slope(dm.x, dp.x), limit_slope(dm.y, dp.y), limit_slope(dm.z, dp.z),
            limit_slope(dm.w, dp.w)};
}

// ---------------------------------------------------------------------------
//  potential.wgsl
// ---------------------------------------------------------------------------
template <typename R>
inline R potential(const SimParams<R> &P, R phi) {
    const R p2 = phi * phi;
    return R(0.5) * P.m2 * p2 - P.delta * p2 * phi / R(3.0) + R(0.25) * P.lambda * p2 * p2;
}
template <typename R>
inline R dpotential(const SimParams<R> &P, R phi) {
    return phi * (P.m2 - P.delta * phi + P.lambda * phi * phi);
}

// ---------------------------------------------------------------------------
//  eos.wgsl
// ---------------------------------------------------------------------------
template <typename R>
inline R eos_sound_speed2(R, R) {
    return R(1.0) / R(3.0);
}
template <typename R>
inline R eos_enthalpy_from_pressure(R p, R) {
    return R(4.0) * p;
}
template <typename R>
inline R eos_pressure_from_conserved(const SimParams<R> &P, R e_lab, R z2, R) {
    const R disc = wmax(R(4.0) * e_lab * e_lab - R(3.0) * z2, R(0.0));
    const R p = (e_lab * e_lab - z2) / (e_lab + std::sqrt(disc));
    return wmax(p, P.p_floor);
}
template <typename R>
inline R length3(R x, R y, R z) {
    return std::sqrt(x * x + y * y + z * z);
}
template <typename R>
inline vec4<R> eos_regularise(const SimParams<R> &P, vec4<R> u) {
    const R e_lab = wmax(u.x, P.e_floor);
    R zx = u.y, zy = u.z, zz = u.w;
    const R zlen = length3(zx, zy, zz);
    const R zcap = P.z_max * e_lab;
    if (zlen > zcap) {
        const R s = zcap / wmax(zlen, R(1e-30));
        zx = zx * s;
        zy = zy * s;
        zz = zz * s;
    }
    return {e_lab, zx, zy, zz};
}
// Perturbation form (PERT): u.x holds E - e_bg and the primitive's w
// p - p_bg, with e_bg = e_ref and p_bg = e_ref / 3, and P carries the floors
// shifted by the backgrounds.  p = (E^2 - Z^2) / (E + s) equals
// E/3 - Z^2 / (s + 2E) (s = sqrt(4E^2 - 3Z^2)), so
// p - p_bg = (E - e_bg)/3 - Z^2 / (s + 2E): the backgrounds cancel exactly.
template <typename R>
inline vec4<R> eos_prim_from_cons_pert(const SimParams<R> &P, vec4<R> u) {
    const R e_bg = P.e_ref, p_bg = P.e_ref / R(3.0);
    const R de = wmax(u.x, P.e_floor);
    const R e_lab = e_bg + de;
    R zx = u.y, zy = u.z, zz = u.w;
    const R zlen = length3(zx, zy, zz);
    const R zcap = P.z_max * e_lab;
    if (zlen > zcap) {
        const R sc = zcap / wmax(zlen, R(1e-30));
        zx = zx * sc;
        zy = zy * sc;
        zz = zz * sc;
    }
    const R z2 = zx * zx + zy * zy + zz * zz;
    const R sq = std::sqrt(wmax(R(4.0) * e_lab * e_lab - R(3.0) * z2, R(0.0)));
    R dp = de / R(3.0) - z2 / (sq + R(2.0) * e_lab);
    dp = wmax(dp, P.p_floor);
    const R d = wmax(e_lab + p_bg + dp, R(1e-30));
    return {zx / d, zy / d, zz / d, dp};
}

// Equation-of-state constants outside the reference's SimParams, set by
// oracle_set_eos: the gamma law's c2 = Gamma - 1 and e0
// (e = p / c2 + e0, docs/EOS.md:86-118) and the degrees-of-freedom ratio of
// the phase-dependent radiation constant (docs/EOS.md:58-84).
float g_eos_c2 = 0.0f, g_eos_e0 = 0.0f, g_eos_dof = 1.0f;

// Gamma-law inversion: f(p) = p - c2 (E - Z^2 / (E + p) - e0) = 0 by a fixed
// eight Newton steps from c2 (E - e0), floored at p_floor after each.
template <typename R>
inline vec4<R> eos_prim_from_cons_gamma(const SimParams<R> &P, vec4<R> u_raw) {
    const vec4<R> u = eos_regularise(P, u_raw);
    const R e_lab = u.x;
    const R z2 = u.y * u.y + u.z * u.z + u.w * u.w;
    const R c2 = R(g_eos_c2), e0 = R(g_eos_e0);
    R p = wmax(c2 * (e_lab - e0), P.p_floor);
    for (int it = 0; it < 8; ++it) {
        const R sp = e_lab + p;
        const R r = p - c2 * (e_lab - z2 / sp - e0);
        const R d = R(1.0) - c2 * z2 / (sp * sp);
        p = wmax(p - r / d, P.p_floor);
    }
    const R d = wmax(e_lab + p, R(1e-30));
    return {u.y / d, u.z / d, u.w / d, p};
}

// Thermal potential (docs/EOS.md:120-150): V(phi, T) = V(phi)
// + gamma/2 (T^2 - T_ref^2) phi^2 - A/3 (T - T_ref) phi^3, the field keeping
// V(phi, 0) and the plasma dV = gamma/2 T^2 phi^2 - A/3 T phi^3:
// p = a/3 T^4 - dV, e = a T^4 - gamma/2 T^2 phi^2, c_s^2 = (dp/dT)/(de/dT).
// Constants as the library's host rounds them (oracle_set_thermal):
// k = a/3, gamma, h = A/3, A, lo = sqrt(3 gamma / (4a)), i2a = 1/(2a).
float g_th_k = 0.0f, g_th_g = 0.0f, g_th_h = 0.0f, g_th_a = 0.0f, g_th_lo = 0.0f, g_th_i2a = 0.0f;

template <typename R>
inline R thermal_energy(const SimParams<R> &P, R T, R phi) {
    const R t2 = T * T;
    return P.a_rad * (t2 * t2) - (R(0.5) * R(g_th_g)) * (t2 * (phi * phi));
}
// c_s^2 held in [1e-4, 1]
template <typename R>
inline R thermal_cs2(const SimParams<R> &P, R T, R phi) {
    const R t2 = T * T, f2 = phi * phi;
    const R dp = T * (R(4.0) * R(g_th_k) * t2 - R(g_th_g) * f2) + R(g_th_h) * (f2 * phi);
    const R de = wmax(T * (R(4.0) * P.a_rad * t2 - R(g_th_g) * f2), R(1e-30));
    return wmin(wmax(dp / de, R(1e-4)), R(1.0));
}
// eos_temperature(p, phi): eight Newton steps on p(T, phi) = p from the
// phi = 0 root, each held to [max(lo |phi|, T/2), 2T].
template <typename R>
inline R thermal_temperature(const SimParams<R> &P, R p, R phi) {
    const R k = R(g_th_k), gm = R(g_th_g), hc = R(g_th_h);
    const R pp = wmax(p, P.p_floor);
    const R lo = R(g_th_lo) * std::fabs(phi);
    const R f2 = phi * phi, h = hc * (f2 * phi);
    R T = wmax(std::sqrt(std::sqrt(pp / k)), lo);
    for (int it = 0; it < 8; ++it) {
        const R t2 = T * T;
        const R g = k * (t2 * t2) - (R(0.5) * gm) * (t2 * f2) + hc * (T * (f2 * phi)) - pp;
        const R d = wmax(T * (R(4.0) * k * t2 - gm * f2) + h, R(1e-30));
        const R tn = T - g / d;
        T = wmin(wmax(tn, wmax(lo, R(0.5) * T)), R(2.0) * T);
    }
    return T;
}
template <typename R>
inline R thermal_dpotential(const SimParams<R> &P, R phi, R T) {
    return dpotential(P, phi) +
           phi * (R(g_th_g) * (T * T - P.t_ref * P.t_ref) - R(g_th_a) * ((T - P.t_ref) * phi));
}
template <typename R>
inline R thermal_exchange(R phi, R T) {
    return phi * (R(g_th_g) * (T * T) - R(g_th_a) * (T * phi));
}
template <typename R>
inline R thermal_potential0(const SimParams<R> &P, R phi) {
    const R f2 = phi * phi;
    return potential(P, phi) + f2 * (R(g_th_h) * (P.t_ref * phi) - (R(0.5) * R(g_th_g)) * (P.t_ref * P.t_ref));
}
// Inversion: f(p) = p - p(T(e), phi), e = E - Z^2 / (E + p), T^2 the root of
// e(T) = e on the physical branch; eight Newton steps floored at p_floor.
template <typename R>
inline vec4<R> eos_prim_from_cons_thermal(const SimParams<R> &P, vec4<R> u_raw, R phi) {
    const vec4<R> u = eos_regularise(P, u_raw);
    const R e_lab = u.x;
    const R z2 = u.y * u.y + u.z * u.z + u.w * u.w;
    const R k = R(g_th_k), gm = R(g_th_g), i2a = R(g_th_i2a);
    const R f2 = phi * phi;
    const R g = (R(0.5) * gm) * f2;
    const R h = R(g_th_h) * (f2 * phi);
    const R a4 = R(4.0) * P.a_rad;
    R X = (g + std::sqrt(g * g + a4 * e_lab)) * i2a;
    R p = wmax(k * (X * X) - g * X + h * std::sqrt(X), P.p_floor);
    for (int it = 0; it < 8; ++it) {
        const R sp = e_lab + p;
        const R e = e_lab - z2 / sp;
        X = (g + std::sqrt(g * g + a4 * e)) * i2a;
        const R T = std::sqrt(X);
        const R dp = T * (R(4.0) * k * X - gm * f2) + h;
        const R de = wmax(T * (a4 * X - gm * f2), R(1e-30));
        const R c2 = wmin(wmax(dp / de, R(1e-4)), R(1.0));
        const R r = p - (k * (X * X) - g * X + h * T);
        const R d = R(1.0) - c2 * z2 / (sp * sp);
        p = wmax(p - r / d, P.p_floor);
    }
    const R d = wmax(e_lab + p, R(1e-30));
    return {u.y / d, u.z / d, u.w / d, p};
}

template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false>
inline vec4<R> eos_prim_from_cons(const SimParams<R> &P, vec4<R> u_raw, R phi) {
    if (THERMAL) return eos_prim_from_cons_thermal(P, u_raw, phi);
    if (GAMMA) return eos_prim_from_cons_gamma(P, u_raw);
    if (PERT) return eos_prim_from_cons_pert(P, u_raw);
    const vec4<R> u = eos_regularise(P, u_raw);
    const R e_lab = u.x;
    const R p = eos_pressure_from_conserved(P, e_lab, u.y * u.y + u.z * u.z + u.w * u.w, phi);
    const R s = e_lab + p;
    const R d = wmax(s, R(1e-30));
    return {u.y / d, u.z / d, u.w / d, p};
}
// PERT: the energy component is E - e_bg = w W^2 v^2 + 3 (p - p_bg); `w_out`
// returns w W^2 for the energy flux w W^2 v_d.
template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false>
inline vec4<R> eos_cons_from_prim(const SimParams<R> &P, vec4<R> q, R phi, R *w_out = nullptr) {
    const R p = q.w;
    const R v2 = wmin(q.x * q.x + q.y * q.y + q.z * q.z, P.z_max * P.z_max);
    const R pf = PERT ? P.e_ref / R(3.0) + p : p;
    // gamma law: w = e + p = p / c2 + p + e0; thermal: e(T(p, phi), phi) + p
    R enth;
    if (THERMAL) enth = thermal_energy(P, thermal_temperature(P, p, phi), phi) + p;
    else enth = GAMMA ? p / R(g_eos_c2) + p + R(g_eos_e0) : eos_enthalpy_from_pressure(pf, phi);
    const R w_gam2 = enth / (R(1.0) - v2);
    if (w_out) *w_out = w_gam2;
    if (PERT) return {w_gam2 * v2 + R(3.0) * p, w_gam2 * q.x, w_gam2 * q.y, w_gam2 * q.z};
    return {w_gam2 - p, w_gam2 * q.x, w_gam2 * q.y, w_gam2 * q.z};
}
template <typename R>
inline R axis_comp(vec4<R> q, int axis) {
    return axis == 0 ? q.x : (axis == 1 ? q.y : q.z);
}
// PERT: the energy flux is w W^2 v_d (passed as w), the momentum flux carries
// p - p_bg (the constant p_bg cancels in every flux difference).
template <typename R, bool PERT = false>
inline vec4<R> eos_flux(vec4<R> q, vec4<R> u, int axis, R w = R(0)) {
    const R p = q.w;
    const R vd = axis_comp(q, axis);
    vec4<R> f{PERT ? w * vd : (u.x + p) * vd, u.y * vd, u.z * vd, u.w * vd};
    if (axis == 0) f.y = f.y + p;
    if (axis == 1) f.z = f.z + p;
    if (axis == 2) f.w = f.w + p;
    return f;
}
template <typename R, bool GAMMA = false, bool THERMAL = false>
inline void eos_wave_speeds(const SimParams<R> &P, vec4<R> q, R phi, int axis, R &lm, R &lp) {
    const R v2 = wmin(q.x * q.x + q.y * q.y + q.z * q.z, P.z_max * P.z_max);
    const R vd = axis_comp(q, axis);
    const R cs2 = THERMAL ? thermal_cs2(P, thermal_temperature(P, q.w, phi), phi)
                          : (GAMMA ? R(g_eos_c2) : eos_sound_speed2(q.w, phi));
    const R cs = std::sqrt(cs2);
    const R denom = R(1.0) - v2 * cs2;
    const R rad = wmax((R(1.0) - v2) * (R(1.0) - vd * vd - cs2 * (v2 - vd * vd)), R(0.0));
    const R a = vd * (R(1.0) - cs2) / denom;
    const R b = cs * std::sqrt(rad) / denom;
    lm = a - b;
    lp = a + b;
}

// ---------------------------------------------------------------------------
//  step.wgsl
// ---------------------------------------------------------------------------
template <typename R>
inline vec4<R> sanitise(const SimParams<R> &P, vec4<R> q) {
    const R p = wmax(q.w, P.p_floor);
    R vx = q.x, vy = q.y, vz = q.z;
    const R v2 = vx * vx + vy * vy + vz * vz;
    const R vmax2 = P.z_max * P.z_max;
    if (v2 > vmax2) {
        const R s = std::sqrt(vmax2 / wmax(v2, R(1e-30)));
        vx = vx * s;
        vy = vy * s;
        vz = vz * s;
    }
    return {vx, vy, vz, p};
}

template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false>
inline vec4<R> hll_flux(const SimParams<R> &P, vec4<R> q_l, R phi_l, vec4<R> q_r, R phi_r, int axis) {
    R w_l, w_r;
    const vec4<R> u_l = eos_cons_from_prim<R, PERT, GAMMA, THERMAL>(P, q_l, phi_l, &w_l);
    const vec4<R> u_r = eos_cons_from_prim<R, PERT, GAMMA, THERMAL>(P, q_r, phi_r, &w_r);
    const vec4<R> f_l = eos_flux<R, PERT>(q_l, u_l, axis, w_l);
    const vec4<R> f_r = eos_flux<R, PERT>(q_r, u_r, axis, w_r);
    R lml, lpl, lmr, lpr;
    eos_wave_speeds<R, GAMMA, THERMAL>(P, q_l, phi_l, axis, lml, lpl);
    eos_wave_speeds<R, GAMMA, THERMAL>(P, q_r, phi_r, axis, lmr, lpr);
    const R s_min = wmin(wmin(lml, lmr), R(0.0));
    const R s_max = wmax(wmax(lpl, lpr), R(0.0));
    const R den = wmax(s_max - s_min, R(1e-12));
    const R k = s_min * s_max;
    return {(s_max * f_l.x - s_min * f_r.x + k * (u_r.x - u_l.x)) / den,
            (s_max * f_l.y - s_min * f_r.y + k * (u_r.y - u_l.y)) / den,
            (s_max * f_l.z - s_min * f_r.z + k * (u_r.z - u_l.z)) / den,
            (s_max * f_l.w - s_min * f_r.w + k * (u_r.w - u_l.w)) / den};
}

template <typename R>
inline vec4<R> add(vec4<R> a, vec4<R> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w};
}
template <typename R>
inline vec4<R> sub(vec4<R> a, vec4<R> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w};
}
template <typename R>
inline vec4<R> scale(R s, vec4<R> a) {
    return {s * a.x, s * a.y, s * a.z, s * a.w};
}

template <typename R>
inline vec4<R> ld4(const R *a, size_t i) {
    return {a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]};
}

// step.wgsl main for one cell.
template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false>
void step_cell(const SimParams<R> &P, const StageParams<R> &S, const R *field_n, const R *fluid_n,
               const R *field_in, const R *fluid_in, const R *prim, R *field_out, R *fluid_out,
               int cx, int cy, int cz) {
    const size_t i0 = cell_index(P, cx, cy, cz);
    const R phi0 = field_in[2 * i0];
    const R pi0 = field_in[2 * i0 + 1];
    const vec4<R> q0 = sanitise(P, ld4(prim, i0));
    R lap_sum = R(0.0);
    R grad[3] = {R(0.0), R(0.0), R(0.0)};
    vec4<R> flux_div{R(0.0), R(0.0), R(0.0), R(0.0)};
    for (int axis = 0; axis < 3; ++axis) {
        const int e1[3] = {axis == 0, axis == 1, axis == 2};
        const size_t im1 = cell_index(P, cx - e1[0], cy - e1[1], cz - e1[2]);
        const size_t ip1 = cell_index(P, cx + e1[0], cy + e1[1], cz + e1[2]);
        const size_t im2 = cell_index(P, cx - 2 * e1[0], cy - 2 * e1[1], cz - 2 * e1[2]);
        const size_t ip2 = cell_index(P, cx + 2 * e1[0], cy + 2 * e1[1], cz + 2 * e1[2]);
        const R phi_m = field_in[2 * im1];
        const R phi_p = field_in[2 * ip1];
        lap_sum = lap_sum + (phi_m + phi_p - R(2.0) * phi0);
        grad[axis] = R(0.5) * (phi_p - phi_m) * P.inv_dx;
        const vec4<R> qm2 = sanitise(P, ld4(prim, im2));
        const vec4<R> qm1 = sanitise(P, ld4(prim, im1));
        const vec4<R> qp1 = sanitise(P, ld4(prim, ip1));
        const vec4<R> qp2 = sanitise(P, ld4(prim, ip2));
        const vec4<R> slope_m1 = limit_slope4(sub(qm1, qm2), sub(q0, qm1));
        const vec4<R> slope_0 = limit_slope4(sub(q0, qm1), sub(qp1, q0));
        const vec4<R> slope_p1 = limit_slope4(sub(qp1, q0), sub(qp2, qp1));
        const vec4<R> f_minus = hll_flux<R, PERT, GAMMA, THERMAL>(P, sanitise(P, add(qm1, scale(R(0.5), slope_m1))), phi_m,
                                         sanitise(P, sub(q0, scale(R(0.5), slope_0))), phi0, axis);
        const vec4<R> f_plus = hll_flux<R, PERT, GAMMA, THERMAL>(P, sanitise(P, add(q0, scale(R(0.5), slope_0))), phi0,
                                        sanitise(P, sub(qp1, scale(R(0.5), slope_p1))), phi_p, axis);
        flux_div = add(flux_div, scale(P.inv_dx, sub(f_plus, f_minus)));
    }
    const R laplacian = lap_sum * P.inv_dx * P.inv_dx;
    const R vv = q0.x * q0.x + q0.y * q0.y + q0.z * q0.z;
    const R gam = R(1.0) / std::sqrt(wmax(R(1.0) - vv, R(1e-12)));
    const R dphi_proper = gam * (pi0 + (q0.x * grad[0] + q0.y * grad[1] + q0.z * grad[2]));
    const R drag = P.eta * dphi_proper;
    const R d_phi = pi0;
    // thermal potential: dV/dphi at the cell's temperature eos_temperature(q0.w,
    // phi0) (docs/EOS.md:133-135), and its plasma part exchanged like the drag
    R dpot = dpotential(P, phi0), src = drag;
    if (THERMAL) {
        const R T0 = thermal_temperature(P, q0.w, phi0);
        dpot = thermal_dpotential(P, phi0, T0);
        src = drag + thermal_exchange(phi0, T0);
    }
    const R d_pi = laplacian - dpot - drag;
    vec4<R> d_fluid{-flux_div.x, -flux_div.y, -flux_div.z, -flux_div.w};
    d_fluid.x = d_fluid.x + src * pi0;
    d_fluid.y = d_fluid.y - src * grad[0];
    d_fluid.z = d_fluid.z - src * grad[1];
    d_fluid.w = d_fluid.w - src * grad[2];
    const R fu_x = phi0 + S.dt_stage * d_phi;
    const R fu_y = pi0 + S.dt_stage * d_pi;
    const vec4<R> uin = ld4(fluid_in, i0);
    const vec4<R> uu = add(uin, scale(S.dt_stage, d_fluid));
    field_out[2 * i0] = S.a0 * field_n[2 * i0] + S.a1 * fu_x;
    field_out[2 * i0 + 1] = S.a0 * field_n[2 * i0 + 1] + S.a1 * fu_y;
    const vec4<R> un = ld4(fluid_n, i0);
    fluid_out[4 * i0] = S.a0 * un.x + S.a1 * uu.x;
    fluid_out[4 * i0 + 1] = S.a0 * un.y + S.a1 * uu.y;
    fluid_out[4 * i0 + 2] = S.a0 * un.z + S.a1 * uu.z;
    fluid_out[4 * i0 + 3] = S.a0 * un.w + S.a1 * uu.w;
}

// ---------------------------------------------------------------------------
//  tanh for the nucleation profile
// ---------------------------------------------------------------------------
// tanh(x) = sign(x) * m / (m + 2) with m = expm1(2|x|).  expm1(y) for
// y < 1/2 from its Taylor series (terms to y^18/18!, nested);
// otherwise exp(y) - 1 with exp(y) = 2^k exp(r), k = floor(y/ln2 + 1/2),
// r = (y - k ln2_hi) - k ln2_lo (Cody & Waite, "Software Manual for the
// Elementary Functions", 1980; the ln 2 split of fdlibm), exp(r) from its
// Taylor series to r^16/16!.  Saturates to +-1 for |x| > 22 (FP64) and
// |x| > 12 (FP32 argument), where the rounded result is exactly +-1.
inline double pow2i(int k) {
    const uint64_t bits = (uint64_t)(k + 1023) << 52;
    double d;
    std::memcpy(&d, &bits, sizeof(d));
    return d;
}
inline double oracle_expm1_nonneg(double y) {
    if (y < 0.5) {
        double r = 1.0;
        for (int k = 18; k >= 2; --k) r = 1.0 + y * r / (double)k;
        return y * r;
    }
    const double kf = std::floor(y * 1.44269504088896338700e+00 + 0.5);
    const double r = (y - kf * 6.93147180369123816490e-01) - kf * 1.90821492927058770002e-10;
    double e = 1.0;
    for (int k = 16; k >= 1; --k) e = 1.0 + r * e / (double)k;
    return e * pow2i((int)kf) - 1.0;
}
inline double oracle_tanh(double x) {
    const double ax = std::fabs(x);
    double t = 1.0;
    if (!(ax > 22.0)) {
        const double m = oracle_expm1_nonneg(2.0 * ax);
        t = m / (m + 2.0);
    }
    return x < 0.0 ? -t : t;
}
// FP32 tanh for the FP32 profile: tanh|x| = m / (m + 2), m = expm1(2|x|),
// expm1 from its Taylor series to y^8/8! below ln2/2, else by Cody-Waite
// reduction y = k ln2_hi + k ln2_lo + r and 2^k expm1(r) + (2^k - 1); +-1
// beyond |x| = 9.5 (where tanhf rounds to 1).  Single-precision IEEE
// operations in a fixed order (-ffp-contract=off), as the CUDA library
// evaluates them.
inline float oracle_expm1_f32(float y) {
    float t = 2.48015873e-05f;
    t = 1.98412698e-04f + y * t;
    t = 1.38888889e-03f + y * t;
    t = 8.33333333e-03f + y * t;
    t = 4.16666667e-02f + y * t;
    t = 1.66666667e-01f + y * t;
    t = 0.5f + y * t;
    t = 1.0f + y * t;
    return y * t;
}
inline float oracle_tanh_r(float x) {
    const float a = std::fabs(x);
    if (a > 9.5f) return std::copysign(1.0f, x);
    const float y = a + a;
    float m;
    if (y < 0.346573590f) {
        m = oracle_expm1_f32(y);
    } else {
        const float k = std::rint(y * 1.44269504f);
        const float r = (y + -(k * 0.693145752f)) + -(k * 1.42860677e-06f);
        const float p2 = std::ldexp(1.0f, (int)k);
        m = p2 * oracle_expm1_f32(r) + (p2 + -1.0f);
    }
    return std::copysign(m / (m + 2.0f), x);
}
inline double oracle_tanh_r(double x) { return oracle_tanh(x); }

template <typename R>
inline R min_image(R d, R n) {
    R r = d;
    if (r > R(0.5) * n) r = r - n;
    if (r < R(-0.5) * n) r = r + n;
    return r;
}

template <typename R>
void nucleate_all(const SimParams<R> &P, const float *bubbles, uint32_t count, R *field) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z) {
        for (int y = 0; y < ny; ++y) {
            for (int x = 0; x < nx; ++x) {
                const size_t i = ((size_t)z * ny + y) * nx + x;
                const R px = R(x), py = R(y), pz = R(z);
                const R n_x = R(P.nx), n_y = R(P.ny), n_z = R(P.nz);
                R phi = field[2 * i];
                for (uint32_t b = 0; b < count; ++b) {
                    const R cx = R(bubbles[4 * b]), cy = R(bubbles[4 * b + 1]);
                    const R cz = R(bubbles[4 * b + 2]), r0 = R(bubbles[4 * b + 3]);
                    const R dx = min_image(px - cx, n_x);
                    const R dy = min_image(py - cy, n_y);
                    const R dz = min_image(pz - cz, n_z);
                    const R r = length3(dx, dy, dz) * P.dx;
                    const R profile =
                        R(0.5) * P.phi_b * (R(1.0) - oracle_tanh_r((r - r0 * P.dx) / P.wall_width));
                    phi = wmax(phi, profile);
                }
                field[2 * i] = phi;
            }
        }
    }
}

template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false>
void step_all(const SimParams<R> &P, const StageParams<R> &S, const R *field_n, const R *fluid_n,
              const R *field_in, const R *fluid_in, const R *prim, R *field_out, R *fluid_out) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                step_cell<R, PERT, GAMMA, THERMAL>(P, S, field_n, fluid_n, field_in, fluid_in, prim, field_out,
                                                   fluid_out, x, y, z);
}

// ---------------------------------------------------------------------------
//  MIXED precision form: FP64 recovery where the Lorentz factor exceeds 3
// ---------------------------------------------------------------------------
// The FP32 recovery is redone in FP64 from the same FP32 conserved state
// wherever the FP32 result has v^2 > 8/9 (gamma > 3), where E^2 - Z^2
// cancels and FP32 loses the pressure; the reference's precision plan puts
// FP64 at exactly this inversion (docs/PRECISION.md:150-152).  The FP64 steps
// are eos_regularise and eos_pressure_from_conserved (shaders/eos.wgsl:
// 94-123) on the FP32 inputs and constants widened exactly, the result rounded
// once to FP32.  PERT: the perturbation form's inversion (as
// eos_prim_from_cons_pert) with p_bg the FP32 value of e_ref / 3 widened.
template <bool PERT>
inline vec4<float> prim_from_cons_f64(const SimParams<float> &P, vec4<float> u) {
    const double e_bg = PERT ? (double)P.e_ref : 0.0;
    const double p_bg = PERT ? (double)(P.e_ref / 3.0f) : 0.0;
    const double de = wmax((double)u.x, (double)P.e_floor);
    const double e_lab = PERT ? e_bg + de : de;
    double zx = u.y, zy = u.z, zz = u.w;
    const double zlen = length3(zx, zy, zz);
    const double zcap = (double)P.z_max * e_lab;
    if (zlen > zcap) {
        const double s = zcap / wmax(zlen, 1e-30);
        zx = zx * s;
        zy = zy * s;
        zz = zz * s;
    }
    const double z2 = zx * zx + zy * zy + zz * zz;
    double p;
    if (PERT) {
        const double sq = std::sqrt(wmax(4.0 * e_lab * e_lab - 3.0 * z2, 0.0));
        p = de / 3.0 - z2 / (sq + 2.0 * e_lab);
    } else {
        const double disc = wmax(4.0 * e_lab * e_lab - 3.0 * z2, 0.0);
        p = (e_lab * e_lab - z2) / (e_lab + std::sqrt(disc));
    }
    p = wmax(p, (double)P.p_floor);
    const double d = PERT ? wmax(e_lab + p_bg + p, 1e-30) : wmax(e_lab + p, 1e-30);
    return {(float)(zx / d), (float)(zy / d), (float)(zz / d), (float)p};
}

template <typename R, bool PERT = false, bool GAMMA = false, bool THERMAL = false, bool MIXED = false>
void primitives_all(const SimParams<R> &P, const R *field, const R *fluid, R *prim) {
    const size_t n = (size_t)P.nx * P.ny * P.nz;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        vec4<R> q = eos_prim_from_cons<R, PERT, GAMMA, THERMAL>(P, ld4(fluid, (size_t)i), field[2 * i]);
        if constexpr (MIXED && sizeof(R) == 4) {
            const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
            if (v2 > R(8.0) / R(9.0)) q = prim_from_cons_f64<PERT>(P, ld4(fluid, (size_t)i));
        }
        prim[4 * i] = q.x;
        prim[4 * i + 1] = q.y;
        prim[4 * i + 2] = q.z;
        prim[4 * i + 3] = q.w;
    }
}

template <typename R>
void init_all(const SimParams<R> &P, R *field, R *fluid) {
    const size_t n = (size_t)P.nx * P.ny * P.nz;
    for (size_t i = 0; i < n; ++i) {
        field[2 * i] = R(0.0);
        field[2 * i + 1] = R(0.0);
        fluid[4 * i] = P.e_ref;
        fluid[4 * i + 1] = R(0.0);
        fluid[4 * i + 2] = R(0.0);
        fluid[4 * i + 3] = R(0.0);
    }
}

// cell_contribution (reduce.wgsl:56-79) per cell in R; sums in FP64, one
// partial per z-plane, planes folded in order.
// PERT: e_total and e_lab miss e_bg per cell (the caller adds N e_bg in FP64);
// the kinetic term adds e_bg + p_bg back.
template <typename R, bool PERT = false, bool THERMAL = false>
void reduce_all(const SimParams<R> &P, const R *field, const R *fluid, const R *prim, double sums[4],
                R *max_v) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
    std::vector<double> part((size_t)nz * 4, 0.0);
    std::vector<R> vmax((size_t)nz, R(0.0));
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        R vm = R(0.0);
        for (int y = 0; y < ny; ++y) {
            for (int x = 0; x < nx; ++x) {
                const size_t i = ((size_t)z * ny + y) * nx + x;
                const R phi = field[2 * i];
                const R pi = field[2 * i + 1];
                R grad2 = R(0.0);
                for (int axis = 0; axis < 3; ++axis) {
                    const int e[3] = {axis == 0, axis == 1, axis == 2};
                    const R d = R(0.5) *
                                (field[2 * cell_index(P, x + e[0], y + e[1], z + e[2])] -
                                 field[2 * cell_index(P, x - e[0], y - e[1], z - e[2])]) *
                                P.inv_dx;
                    grad2 = grad2 + d * d;
                }
                const R e_lab = wmax(fluid[4 * i], P.e_floor);
                const vec4<R> q = ld4(prim, i);
                const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
                // thermal potential: the field holds V(phi, 0), E the rest
                const R pot = THERMAL ? thermal_potential0(P, phi) : potential(P, phi);
                const R e_total = R(0.5) * pi * pi + R(0.5) * grad2 + pot + e_lab;
                const R broken = phi > R(0.5) * P.phi_b ? R(1.0) : R(0.0);
                const R kinetic = PERT ? ((e_lab + q.w) + (P.e_ref + P.e_ref / R(3.0))) * v2 : (e_lab + q.w) * v2;
                a0 += (double)e_total;
                a1 += (double)broken;
                a2 += (double)kinetic;
                a3 += (double)e_lab;
                vm = wmax(vm, length3(q.x, q.y, q.z));
            }
        }
        part[4 * z] = a0;
        part[4 * z + 1] = a1;
        part[4 * z + 2] = a2;
        part[4 * z + 3] = a3;
        vmax[z] = vm;
    }
    for (int k = 0; k < 4; ++k) sums[k] = 0.0;
    R vm = R(0.0);
    for (int z = 0; z < nz; ++z) {
        for (int k = 0; k < 4; ++k) sums[k] += part[4 * z + k];
        vm = wmax(vm, vmax[z]);
    }
    *max_v = vm;
}


// ---------------------------------------------------------------------------
//  vis.wgsl and volume.wgsl (the headless screenshot path)
// ---------------------------------------------------------------------------
// IEEE binary32 -> binary16, round to nearest even (the rgba16float store).
inline uint16_t f32_to_f16(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // >= 65520 rounds to infinity
    if (ax < 0x38800000u) {                                    // below 2^-14: subnormal or zero
        const float v = std::fabs(f) * 16777216.0f;            // exact: scaled by 2^24
        return (uint16_t)(sign | (uint32_t)std::nearbyint(v));
    }
    const uint32_t mant = ax & 0x7fffffu;
    const uint32_t e = (ax >> 23) - 127u + 15u;
    uint32_t h = (e << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
    return (uint16_t)(sign | h);
}

inline float f16_to_f32(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    float v;
    if (e == 0) v = std::ldexp((float)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 0x400u), (int)e - 25);
    uint32_t b;
    std::memcpy(&b, &v, 4);
    b |= sign;
    std::memcpy(&v, &b, 4);
    return v;
}

// vis main (shaders/vis.wgsl:30-55) over a primitives buffer from
// primitives_all; out = nx*ny*nz half4 texels.
template <typename R, bool PERT = false, bool THERMAL = false>
void vis_all(const SimParams<R> &P, const R *field, const R *fluid, const R *prim, uint16_t *out) {
    const int64_t n = (int64_t)P.nx * P.ny * P.nz;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const R phi = field[2 * i];
        const R vx = prim[4 * i], vy = prim[4 * i + 1], vz = prim[4 * i + 2], q_w = prim[4 * i + 3];
        const R p_bg = P.e_ref / R(3.0);
        const R p = PERT ? p_bg + q_w : q_w;
        const R e_lab = PERT ? P.e_ref + wmax(fluid[4 * i], P.e_floor) : wmax(fluid[4 * i], P.e_floor);
        const R vv = vx * vx + vy * vy + vz * vz;
        const R speed = std::sqrt(vv);
        const R pt = PERT ? p_bg + wmax(q_w, P.p_floor) : wmax(p, P.p_floor);
        R a = P.a_rad;
        if (g_eos_dof != 1.0f) {  // the phase-dependent radiation constant
            const R h = wmin(wmax(phi / P.phi_b, R(0.0)), R(1.0));
            const R smooth = h * h * (R(3.0) - R(2.0) * h);
            a = P.a_rad * (R(1.0) + (R(g_eos_dof) - R(1.0)) * smooth);
        }
        const R x = R(3.0) * pt / a;  // eos_temperature (shaders/eos.wgsl:65-69)
        const R temp = THERMAL ? thermal_temperature(P, pt, phi) : std::sqrt(std::sqrt(x));
        const R kinetic = (e_lab + p) * vv;
        out[4 * i + 0] = f32_to_f16((float)(phi / P.phi_b));
        out[4 * i + 1] = f32_to_f16((float)speed);
        out[4 * i + 2] = f32_to_f16((float)(temp / P.t_ref - R(1.0)));
        out[4 * i + 3] = f32_to_f16((float)(kinetic / P.e_ref));
    }
}

// The ViewUniform of shaders/volume.wgsl:22-31 as 44 floats.
struct View {
    float m[16];
    float cam[4], box[4], grid[4], r0[4], r1[4], r2[4], r3[4];
};
static_assert(sizeof(View) == 176, "ViewUniform is 176 bytes");

struct Vol {
    const uint16_t *tex;
    int nx, ny, nz;
    int quant;  // filter-weight fraction: 0 exact, 1 nearest 1/256, 2 truncated 1/256
};

using f3v = vec3<float>;
inline f3v v3(float x, float y, float z) { return f3v{x, y, z}; }
inline f3v vadd(f3v a, f3v b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline f3v vsub(f3v a, f3v b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline f3v vmul(f3v a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float vdot(f3v a, f3v b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline f3v vnorm(f3v a) {
    const float l = std::sqrt(vdot(a, a));
    return v3(a.x / l, a.y / l, a.z / l);
}
inline float wclamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float wmix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline f3v wmix3(f3v a, f3v b, float t) { return v3(wmix(a.x, b.x, t), wmix(a.y, b.y, t), wmix(a.z, b.z, t)); }
inline float wfract(float x) { return x - std::floor(x); }

// Colour maps, shaders/volume.wgsl:37-78.
const float kViridis[11][3] = {{0.267f, 0.005f, 0.329f}, {0.283f, 0.141f, 0.458f}, {0.254f, 0.265f, 0.530f},
                               {0.207f, 0.372f, 0.553f}, {0.164f, 0.471f, 0.558f}, {0.128f, 0.567f, 0.551f},
                               {0.135f, 0.659f, 0.518f}, {0.267f, 0.749f, 0.441f}, {0.478f, 0.821f, 0.318f},
                               {0.741f, 0.873f, 0.150f}, {0.993f, 0.906f, 0.144f}};
const float kInferno[11][3] = {{0.001f, 0.000f, 0.014f}, {0.078f, 0.044f, 0.214f}, {0.225f, 0.036f, 0.388f},
                               {0.373f, 0.074f, 0.432f}, {0.522f, 0.128f, 0.420f}, {0.665f, 0.182f, 0.370f},
                               {0.798f, 0.280f, 0.270f}, {0.902f, 0.413f, 0.144f}, {0.969f, 0.579f, 0.032f},
                               {0.988f, 0.762f, 0.135f}, {0.988f, 0.998f, 0.645f}};
const float kSigned[11][3] = {{0.30f, 0.55f, 1.00f}, {0.22f, 0.42f, 0.85f}, {0.15f, 0.30f, 0.66f},
                              {0.09f, 0.19f, 0.45f}, {0.04f, 0.09f, 0.24f}, {0.02f, 0.02f, 0.03f},
                              {0.26f, 0.09f, 0.04f}, {0.48f, 0.17f, 0.06f}, {0.72f, 0.29f, 0.08f},
                              {0.92f, 0.48f, 0.14f}, {1.00f, 0.72f, 0.32f}};

// ramp (shaders/volume.wgsl:80-90)
inline f3v ramp(float t, int which) {
    const float x = wclamp(t, 0.0f, 1.0f) * 10.0f;
    const int i0 = (int)std::floor(x);
    const int i1 = i0 + 1 < 10 ? i0 + 1 : 10;
    const float f = x - std::floor(x);
    const float(*tab)[3] = which == 0 ? kViridis : (which == 1 ? kInferno : kSigned);
    return wmix3(v3(tab[i0][0], tab[i0][1], tab[i0][2]), v3(tab[i1][0], tab[i1][1], tab[i1][2]), f);
}

// Trilinear filtering with clamp-to-edge addressing and normalised
// coordinates: texel space x = u n - 1/2, weights from the fraction.
inline void tex_sample(const Vol &T, float u, float v, float w, float out[4]) {
    const float c[3] = {u * (float)T.nx - 0.5f, v * (float)T.ny - 0.5f, w * (float)T.nz - 0.5f};
    const int n[3] = {T.nx, T.ny, T.nz};
    int i0[3], i1[3];
    float a[3];
    for (int k = 0; k < 3; ++k) {
        const float fl = std::floor(c[k]);
        float f = c[k] - fl;
        if (T.quant == 1) f = std::nearbyint(f * 256.0f) / 256.0f;
        else if (T.quant == 2) f = std::floor(f * 256.0f) / 256.0f;
        a[k] = f;
        const int b = (int)fl;
        i0[k] = b < 0 ? 0 : (b > n[k] - 1 ? n[k] - 1 : b);
        i1[k] = b + 1 < 0 ? 0 : (b + 1 > n[k] - 1 ? n[k] - 1 : b + 1);
    }
    for (int ch = 0; ch < 4; ++ch) out[ch] = 0.0f;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const float wgt = (dx ? a[0] : 1.0f - a[0]) * (dy ? a[1] : 1.0f - a[1]) * (dz ? a[2] : 1.0f - a[2]);
                const int x = dx ? i1[0] : i0[0], y = dy ? i1[1] : i0[1], z = dz ? i1[2] : i0[2];
                const uint16_t *t = T.tex + 4 * (((size_t)z * T.ny + y) * T.nx + x);
                for (int ch = 0; ch < 4; ++ch) out[ch] += wgt * f16_to_f32(t[ch]);
            }
}

// sample_state (shaders/volume.wgsl:115-121)
inline void sample_state(const View &V, const Vol &T, f3v p, float s[4]) {
    tex_sample(T, (p.x / V.box[0]) * 0.5f + 0.5f, (p.y / V.box[1]) * 0.5f + 0.5f, (p.z / V.box[2]) * 0.5f + 0.5f, s);
}

// fs_main (shaders/volume.wgsl:229-381) for the pixel centre (px, py).
inline f3v fs_main(const View &V, const Vol &T, float px, float py, float ndc_x, float ndc_y) {
    const f3v ro = v3(V.cam[0], V.cam[1], V.cam[2]);
    float far4[4];
    for (int r = 0; r < 4; ++r) far4[r] = V.m[r] * ndc_x + V.m[4 + r] * ndc_y + V.m[8 + r] * 1.0f + V.m[12 + r] * 1.0f;
    const f3v rd = vnorm(vsub(v3(far4[0] / far4[3], far4[1] / far4[3], far4[2] / far4[3]), ro));

    const float horizon = wclamp(rd.y * 0.5f + 0.5f, 0.0f, 1.0f);
    f3v color = vmul(wmix3(v3(0.015f, 0.017f, 0.028f), v3(0.045f, 0.055f, 0.085f), horizon), V.r3[2]);

    auto safe_inv = [](float x) {
        const float s = x < 0.0f ? -1.0f : 1.0f;
        return s / std::fmax(std::fabs(x), 1e-9f);
    };
    const f3v inv_rd = v3(safe_inv(rd.x), safe_inv(rd.y), safe_inv(rd.z));
    const f3v half = v3(V.box[0], V.box[1], V.box[2]);
    const f3v t0 = v3((-half.x - ro.x) * inv_rd.x, (-half.y - ro.y) * inv_rd.y, (-half.z - ro.z) * inv_rd.z);
    const f3v t1 = v3((half.x - ro.x) * inv_rd.x, (half.y - ro.y) * inv_rd.y, (half.z - ro.z) * inv_rd.z);
    const float tmin_x = std::fmin(t0.x, t1.x), tmin_y = std::fmin(t0.y, t1.y), tmin_z = std::fmin(t0.z, t1.z);
    const float tmax_x = std::fmax(t0.x, t1.x), tmax_y = std::fmax(t0.y, t1.y), tmax_z = std::fmax(t0.z, t1.z);
    float t_near = std::fmax(std::fmax(std::fmax(tmin_x, tmin_y), tmin_z), 0.0f);
    float t_far = std::fmin(std::fmin(tmax_x, tmax_y), tmax_z);
    if (t_near >= t_far) return color;

    const int clip_axis = (int)V.r1[1];
    if (clip_axis >= 0) {
        const float n_axis[3] = {clip_axis == 0 ? 1.0f : 0.0f, clip_axis == 1 ? 1.0f : 0.0f, clip_axis == 2 ? 1.0f : 0.0f};
        const float plane = V.r1[2] * V.box[clip_axis];
        const float denom = rd.x * n_axis[0] + rd.y * n_axis[1] + rd.z * n_axis[2];
        const float dist = plane - (ro.x * n_axis[0] + ro.y * n_axis[1] + ro.z * n_axis[2]);
        if (std::fabs(denom) < 1e-6f) {
            if (dist < 0.0f) return color;
        } else {
            const float t_plane = dist / denom;
            if (denom > 0.0f) t_far = std::fmin(t_far, t_plane);
            else t_near = std::fmax(t_near, t_plane);
            if (t_near >= t_far) return color;
        }
    }

    if (V.r3[1] > 0.5f) {
        const float w = 0.004f * V.box[3] * V.grid[0];
        float edge = 0.0f;
        for (int k = 0; k < 2; ++k) {
            const f3v p = vadd(ro, vmul(rd, k == 0 ? t_near : t_far));
            const f3v d = v3(half.x - std::fabs(p.x), half.y - std::fabs(p.y), half.z - std::fabs(p.z));
            const float median = std::fmax(std::fmin(d.x, d.y), std::fmin(std::fmax(d.x, d.y), d.z));
            const float st = wclamp((median - 0.0f) / (w - 0.0f), 0.0f, 1.0f);
            edge = std::fmax(edge, 1.0f - st * st * (3.0f - 2.0f * st));
        }
        color = vadd(color, vmul(v3(0.20f, 0.26f, 0.34f), edge));
    }

    const float cell = V.box[3];
    const float spc = std::fmax(V.r0[2], 0.25f);
    float ds = cell / spc;
    const float span = t_far - t_near;
    if (span / ds > 2048.0f) ds = span / 2048.0f;
    const int n_steps = std::min((int)std::ceil(span / ds), 2048);

    // hash12 (shaders/volume.wgsl:136-140) of the pixel centre + the frame offset
    const float hx = px + V.r3[0], hy = py + V.r3[0];
    f3v p3 = v3(wfract(hx * 0.1031f), wfract(hy * 0.1031f), wfract(hx * 0.1031f));
    const float dd = vdot(p3, v3(p3.y + 33.33f, p3.z + 33.33f, p3.x + 33.33f));
    p3 = v3(p3.x + dd, p3.y + dd, p3.z + dd);
    const float jitter = wfract((p3.x + p3.y) * p3.z);

    const float iso = V.r0[0], wall_opacity = V.r0[1], exposure = V.r0[3], absorption = V.r2[1];
    const bool show_iso = V.r2[2] > 0.5f, show_vol = V.r2[3] > 0.5f;
    f3v accum = v3(0.0f, 0.0f, 0.0f);
    float alpha = 0.0f;
    float t = t_near + jitter * ds;
    float s0[4];
    sample_state(V, T, vadd(ro, vmul(rd, t_near)), s0);
    float prev_phi = s0[0];
    float prev_t = t_near;
    const f3v l1 = vnorm(v3(0.55f, 0.72f, 0.42f));
    const f3v l2 = vnorm(v3(-0.5f, -0.2f, -0.7f));
    for (int i = 0; i < n_steps; ++i) {
        if (t > t_far || alpha > 0.995f) break;
        const f3v p = vadd(ro, vmul(rd, t));
        float s[4];
        sample_state(V, T, p, s);
        const float d_prev = prev_phi - iso;
        const float d_cur = s[0] - iso;
        if (show_iso && d_prev != 0.0f && d_prev * d_cur <= 0.0f) {
            const float denom = s[0] - prev_phi;
            const float frac = std::fabs(denom) > 1e-6f ? (iso - prev_phi) / denom : 0.5f;
            const float t_hit = wmix(prev_t, t, wclamp(frac, 0.0f, 1.0f));
            const f3v p_hit = vadd(ro, vmul(rd, t_hit));
            const float h = V.box[3];
            float a_[4], b_[4];
            float g[3];
            for (int k = 0; k < 3; ++k) {
                const f3v e = v3(k == 0 ? h : 0.0f, k == 1 ? h : 0.0f, k == 2 ? h : 0.0f);
                sample_state(V, T, vadd(p_hit, e), a_);
                sample_state(V, T, vsub(p_hit, e), b_);
                g[k] = a_[0] - b_[0];
            }
            const f3v grad = v3(g[0] / (2.0f * h), g[1] / (2.0f * h), g[2] / (2.0f * h));
            const f3v n = vnorm(vsub(vmul(grad, -1.0f), vmul(rd, 1e-6f)));
            float hs[4];
            sample_state(V, T, p_hit, hs);
            const float drive = wclamp(hs[1] * 4.0f, 0.0f, 1.0f);
            const f3v base = wmix3(v3(0.16f, 0.62f, 0.72f), v3(1.00f, 0.72f, 0.28f), drive);
            const f3v view = vmul(rd, -1.0f);
            const float diff = std::fmax(vdot(n, l1), 0.0f) + 0.35f * std::fmax(vdot(n, l2), 0.0f);
            const f3v hh = vnorm(vadd(vadd(l1, view), v3(0.0f, 1e-5f, 0.0f)));
            const float spec = std::pow(std::fmax(vdot(n, hh), 0.0f), 48.0f);
            const float fres = std::pow(1.0f - std::fabs(vdot(n, view)), 3.0f);
            const f3v shaded = vadd(vadd(vmul(base, 0.22f + 0.85f * diff), vmul(v3(1.0f, 1.0f, 1.0f), spec * 0.35f)),
                                    vmul(vmul(base, fres), 0.9f));
            const float a = wall_opacity;
            accum = vadd(accum, vmul(vmul(shaded, 1.0f - alpha), a));
            alpha = alpha + (1.0f - alpha) * a;
        }
        if (show_vol) {
            // map_field (shaders/volume.wgsl:152-185)
            const int mode = (int)V.r1[0];
            const float gain = V.r2[0];
            int rid = (int)V.r1[3];
            float mt, mi;
            if (mode == 0) {
                const float x = wclamp(s[0], 0.0f, 1.0f);
                mt = x;
                mi = x * gain;
            } else if (mode == 1) {
                const float x = wclamp(s[1] * gain, 0.0f, 1.0f);
                mt = x;
                mi = x;
            } else if (mode == 2) {
                const float x = wclamp(s[2] * gain, -1.0f, 1.0f);
                mt = 0.5f + 0.5f * x;
                mi = std::fabs(x);
                rid = 2;
            } else {
                const float x = wclamp(s[3] * gain, 0.0f, 1.0f);
                mt = x;
                mi = x;
            }
            if (mi > 1e-4f) {
                const float weight = mi * mi;
                const float a = 1.0f - std::exp(-absorption * weight * ds);
                const f3v emit = vmul(ramp(mt, rid), exposure);
                accum = vadd(accum, vmul(vmul(emit, 1.0f - alpha), a));
                alpha = alpha + (1.0f - alpha) * a;
            }
        }
        prev_phi = s[0];
        prev_t = t;
        t = t + ds;
    }
    return vadd(vmul(color, 1.0f - alpha), accum);
}

void render_all(const View &V, const Vol &T, int width, int height, uint8_t *out) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int py = 0; py < height; ++py)
        for (int px = 0; px < width; ++px) {
            const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
            const float ndc_x = fx / (float)width * 2.0f - 1.0f;
            const float ndc_y = 1.0f - fy / (float)height * 2.0f;
            f3v c = fs_main(V, T, fx, fy, ndc_x, ndc_y);
            c = v3(c.x / (1.0f + c.x), c.y / (1.0f + c.y), c.z / (1.0f + c.z));
            const float g = 1.0f / 2.2f;
            const float rgb[3] = {std::pow(std::fmax(c.x, 0.0f), g), std::pow(std::fmax(c.y, 0.0f), g),
                                  std::pow(std::fmax(c.z, 0.0f), g)};
            uint8_t *o = out + 4 * ((size_t)py * width + px);
            for (int k = 0; k < 3; ++k) o[k] = (uint8_t)std::nearbyint(wclamp(rgb[k], 0.0f, 1.0f) * 255.0f);
            o[3] = 255;
        }
}

}  // namespace

extern "C" {

int oracle_params_size_f32(void) { return (int)sizeof(SimParams<float>); }
int oracle_params_size_f64(void) { return (int)sizeof(SimParams<double>); }

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

#define ORACLE_API(T, sfx)                                                                          \
    void oracle_init_##sfx(const SimParams<T> *P, T *field, T *fluid) { init_all(*P, field, fluid); } \
    void oracle_nucleate_##sfx(const SimParams<T> *P, const float *bubbles, uint32_t count,         \
                               T *field) {                                                          \
        nucleate_all(*P, bubbles, count, field);                                                    \
    }                                                                                               \
    void oracle_primitives_##sfx(const SimParams<T> *P, const T *field, const T *fluid, T *prim) {  \
        primitives_all(*P, field, fluid, prim);                                                     \
    }                                                                                               \
    void oracle_step_##sfx(const SimParams<T> *P, const StageParams<T> *S, const T *field_n,        \
                           const T *fluid_n, const T *field_in, const T *fluid_in, const T *prim,   \
                           T *field_out, T *fluid_out) {                                            \
        step_all(*P, *S, field_n, fluid_n, field_in, fluid_in, prim, field_out, fluid_out);         \
    }                                                                                               \
    void oracle_reduce_##sfx(const SimParams<T> *P, const T *field, const T *fluid, const T *prim,  \
                             double *sums, T *max_v) {                                              \
        reduce_all(*P, field, fluid, prim, sums, max_v);                                            \
    }

ORACLE_API(float, f32)
ORACLE_API(double, f64)

// The perturbation form in FP32: the same kernels over E - e_ref, with the
// floors shifted by the backgrounds as the library's host shifts them.
static SimParams<float> pert_params(const SimParams<float> &P) {
    SimParams<float> Q = P;
    Q.e_floor = P.e_floor - P.e_ref;
    Q.p_floor = P.p_floor - P.e_ref / 3.0f;
    return Q;
}
void oracle_init_pert_f32(const SimParams<float> *P, float *field, float *fluid) {
    init_all(*P, field, fluid);
    const size_t n = (size_t)P->nx * P->ny * P->nz;
    for (size_t i = 0; i < n; ++i) fluid[4 * i] = 0.0f;
}
// The perturbation form is the MIXED form over E - e_ref: FP64 recovery
// where v^2 > 8/9.
void oracle_primitives_pert_f32(const SimParams<float> *P, const float *field, const float *fluid, float *prim) {
    primitives_all<float, true, false, false, true>(pert_params(*P), field, fluid, prim);
}
void oracle_step_pert_f32(const SimParams<float> *P, const StageParams<float> *S, const float *field_n,
                          const float *fluid_n, const float *field_in, const float *fluid_in, const float *prim,
                          float *field_out, float *fluid_out) {
    step_all<float, true>(pert_params(*P), *S, field_n, fluid_n, field_in, fluid_in, prim, field_out, fluid_out);
}
void oracle_reduce_pert_f32(const SimParams<float> *P, const float *field, const float *fluid, const float *prim,
                            double *sums, float *max_v) {
    reduce_all<float, true>(pert_params(*P), field, fluid, prim, sums, max_v);
}
void oracle_vis_pert_f32(const SimParams<float> *P, const float *field, const float *fluid, const float *prim,
                         uint16_t *out) {
    vis_all<float, true>(pert_params(*P), field, fluid, prim, out);
}

// The MIXED precision form: the FP32 kernels with the primitives pass
// recovering in FP64 where v^2 > 8/9 (step, reduce and vis read its output).
void oracle_primitives_mixed_f32(const SimParams<float> *P, const float *field, const float *fluid, float *prim) {
    primitives_all<float, false, false, false, true>(*P, field, fluid, prim);
}

void oracle_vis_f32(const SimParams<float> *P, const float *field, const float *fluid, const float *prim,
                    uint16_t *out) {
    vis_all(*P, field, fluid, prim, out);
}
void oracle_vis_f64(const SimParams<double> *P, const double *field, const double *fluid, const double *prim,
                    uint16_t *out) {
    vis_all(*P, field, fluid, prim, out);
}
// One frame of the volume renderer over half4 texels `tex` (nx*ny*nz).
void oracle_render(const float *view44, const uint16_t *tex, int nx, int ny, int nz, int width, int height,
                   int quant, uint8_t *out) {
    View V;
    std::memcpy(&V, view44, sizeof(View));
    const Vol T{tex, nx, ny, nz, quant};
    render_all(V, T, width, height, out);
}
uint16_t oracle_f32_to_f16(float x) { return f32_to_f16(x); }

// Equation of state of the following calls: c2 = Gamma - 1 and e0 of the
// gamma law (used by the *_gamma_f32 kernels), and the degrees-of-freedom
// ratio of the vis pack's temperature (1 = the bag model).
void oracle_set_eos(float c2, float e0, float dof) {
    g_eos_c2 = c2;
    g_eos_e0 = e0;
    g_eos_dof = dof;
}
void oracle_primitives_gamma_f32(const SimParams<float> *P, const float *field, const float *fluid, float *prim) {
    primitives_all<float, false, true>(*P, field, fluid, prim);
}
void oracle_step_gamma_f32(const SimParams<float> *P, const StageParams<float> *S, const float *field_n,
                           const float *fluid_n, const float *field_in, const float *fluid_in, const float *prim,
                           float *field_out, float *fluid_out) {
    step_all<float, false, true>(*P, *S, field_n, fluid_n, field_in, fluid_in, prim, field_out, fluid_out);
}

// Thermal potential constants of the following *_thermal_f32 calls.
void oracle_set_thermal(float k, float g, float h, float a, float lo, float i2a) {
    g_th_k = k;
    g_th_g = g;
    g_th_h = h;
    g_th_a = a;
    g_th_lo = lo;
    g_th_i2a = i2a;
}
void oracle_init_thermal_f32(const SimParams<float> *P, float *field, float *fluid) { init_all(*P, field, fluid); }
void oracle_primitives_thermal_f32(const SimParams<float> *P, const float *field, const float *fluid, float *prim) {
    primitives_all<float, false, false, true>(*P, field, fluid, prim);
}
void oracle_step_thermal_f32(const SimParams<float> *P, const StageParams<float> *S, const float *field_n,
                             const float *fluid_n, const float *field_in, const float *fluid_in, const float *prim,
                             float *field_out, float *fluid_out) {
    step_all<float, false, false, true>(*P, *S, field_n, fluid_n, field_in, fluid_in, prim, field_out, fluid_out);
}
void oracle_reduce_thermal_f32(const SimParams<float> *P, const float *field, const float *fluid,
                               const float *prim, double *sums, float *max_v) {
    reduce_all<float, false, true>(*P, field, fluid, prim, sums, max_v);
}
void oracle_vis_thermal_f32(const SimParams<float> *P, const float *field, const float *fluid, const float *prim,
                            uint16_t *out) {
    vis_all<float, false, true>(*P, field, fluid, prim, out);
}

double oracle_tanh_f64(double x) { return oracle_tanh(x); }
float oracle_tanh_f32(float x) { return oracle_tanh_r(x); }

}  // extern "C"
