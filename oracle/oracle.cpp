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
// Built with -ffp-contract=off so every operation is one IEEE rounding.
// WGSL's tanh has implementation-defined accuracy; the oracle uses the
// Cody-Waite / Taylor tanh described at oracle_tanh (accurate to a few
// units in 1e-16), which the CUDA library evaluates with the same
// operations, so nucleated fields compare bit for bit.  Its FP64 relative
// error is below 1e-15 (tests/test_oracle_pins.py).
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
template <typename R>
inline vec4<R> eos_prim_from_cons(const SimParams<R> &P, vec4<R> u_raw, R phi) {
    const vec4<R> u = eos_regularise(P, u_raw);
    const R e_lab = u.x;
    const R p = eos_pressure_from_conserved(P, e_lab, u.y * u.y + u.z * u.z + u.w * u.w, phi);
    const R s = e_lab + p;
    const R d = wmax(s, R(1e-30));
    return {u.y / d, u.z / d, u.w / d, p};
}
template <typename R>
inline vec4<R> eos_cons_from_prim(const SimParams<R> &P, vec4<R> q, R phi) {
    const R p = q.w;
    const R v2 = wmin(q.x * q.x + q.y * q.y + q.z * q.z, P.z_max * P.z_max);
    const R w_gam2 = eos_enthalpy_from_pressure(p, phi) / (R(1.0) - v2);
    return {w_gam2 - p, w_gam2 * q.x, w_gam2 * q.y, w_gam2 * q.z};
}
template <typename R>
inline R axis_comp(vec4<R> q, int axis) {
    return axis == 0 ? q.x : (axis == 1 ? q.y : q.z);
}
template <typename R>
inline vec4<R> eos_flux(vec4<R> q, vec4<R> u, int axis) {
    const R p = q.w;
    const R vd = axis_comp(q, axis);
    vec4<R> f{(u.x + p) * vd, u.y * vd, u.z * vd, u.w * vd};
    if (axis == 0) f.y = f.y + p;
    if (axis == 1) f.z = f.z + p;
    if (axis == 2) f.w = f.w + p;
    return f;
}
template <typename R>
inline void eos_wave_speeds(const SimParams<R> &P, vec4<R> q, R phi, int axis, R &lm, R &lp) {
    const R v2 = wmin(q.x * q.x + q.y * q.y + q.z * q.z, P.z_max * P.z_max);
    const R vd = axis_comp(q, axis);
    const R cs2 = eos_sound_speed2(q.w, phi);
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

template <typename R>
inline vec4<R> hll_flux(const SimParams<R> &P, vec4<R> q_l, R phi_l, vec4<R> q_r, R phi_r, int axis) {
    const vec4<R> u_l = eos_cons_from_prim(P, q_l, phi_l);
    const vec4<R> u_r = eos_cons_from_prim(P, q_r, phi_r);
    const vec4<R> f_l = eos_flux(q_l, u_l, axis);
    const vec4<R> f_r = eos_flux(q_r, u_r, axis);
    R lml, lpl, lmr, lpr;
    eos_wave_speeds(P, q_l, phi_l, axis, lml, lpl);
    eos_wave_speeds(P, q_r, phi_r, axis, lmr, lpr);
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
template <typename R>
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
        const vec4<R> f_minus = hll_flux(P, sanitise(P, add(qm1, scale(R(0.5), slope_m1))), phi_m,
                                         sanitise(P, sub(q0, scale(R(0.5), slope_0))), phi0, axis);
        const vec4<R> f_plus = hll_flux(P, sanitise(P, add(q0, scale(R(0.5), slope_0))), phi0,
                                        sanitise(P, sub(qp1, scale(R(0.5), slope_p1))), phi_p, axis);
        flux_div = add(flux_div, scale(P.inv_dx, sub(f_plus, f_minus)));
    }
    const R laplacian = lap_sum * P.inv_dx * P.inv_dx;
    const R vv = q0.x * q0.x + q0.y * q0.y + q0.z * q0.z;
    const R gam = R(1.0) / std::sqrt(wmax(R(1.0) - vv, R(1e-12)));
    const R dphi_proper = gam * (pi0 + (q0.x * grad[0] + q0.y * grad[1] + q0.z * grad[2]));
    const R drag = P.eta * dphi_proper;
    const R d_phi = pi0;
    const R d_pi = laplacian - dpotential(P, phi0) - drag;
    vec4<R> d_fluid{-flux_div.x, -flux_div.y, -flux_div.z, -flux_div.w};
    d_fluid.x = d_fluid.x + drag * pi0;
    d_fluid.y = d_fluid.y - drag * grad[0];
    d_fluid.z = d_fluid.z - drag * grad[1];
    d_fluid.w = d_fluid.w - drag * grad[2];
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
inline float oracle_tanh_r(float x) {
    if (x > 12.0f) return 1.0f;
    if (x < -12.0f) return -1.0f;
    return (float)oracle_tanh((double)x);
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

template <typename R>
void step_all(const SimParams<R> &P, const StageParams<R> &S, const R *field_n, const R *fluid_n,
              const R *field_in, const R *fluid_in, const R *prim, R *field_out, R *fluid_out) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                step_cell(P, S, field_n, fluid_n, field_in, fluid_in, prim, field_out, fluid_out, x, y, z);
}

template <typename R>
void primitives_all(const SimParams<R> &P, const R *field, const R *fluid, R *prim) {
    const size_t n = (size_t)P.nx * P.ny * P.nz;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        const vec4<R> q = eos_prim_from_cons(P, ld4(fluid, (size_t)i), field[2 * i]);
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
template <typename R>
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
                const R e_total = R(0.5) * pi * pi + R(0.5) * grad2 + potential(P, phi) + e_lab;
                const R broken = phi > R(0.5) * P.phi_b ? R(1.0) : R(0.0);
                const R kinetic = (e_lab + q.w) * v2;
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

double oracle_tanh_f64(double x) { return oracle_tanh(x); }
float oracle_tanh_f32(float x) { return oracle_tanh_r(x); }

}  // extern "C"
