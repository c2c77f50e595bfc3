// Host physics: see physics.h.
#include "physics.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace bubble {

namespace {

// f32::powi for the small exponents the model uses, as repeated squaring.
float powi(float x, int n) {
    float r = 1.0f;
    float a = x;
    while (true) {
        if (n & 1) r *= a;
        n >>= 1;
        if (n == 0) break;
        a *= a;
    }
    return r;
}

inline uint32_t rotr32(uint32_t x, uint32_t r) {
    r &= 31u;
    return r == 0 ? x : (x >> r) | (x << (32u - r));
}
inline uint64_t rotr64(uint64_t x, uint32_t r) {
    r &= 63u;
    return r == 0 ? x : (x >> r) | (x << (64u - r));
}

constexpr unsigned __int128 kMcgMultiplier =
    (static_cast<unsigned __int128>(0x2360ED051FC65DA4ULL) << 64) |
    static_cast<unsigned __int128>(0x4385DF649FCCF645ULL);

}  // namespace

const float kRK3[3][2] = {{0.0f, 1.0f}, {0.75f, 0.25f}, {1.0f / 3.0f, 2.0f / 3.0f}};

// ---------------------------------------------------------------------------
//  Pcg64Mcg
// ---------------------------------------------------------------------------
Pcg64Mcg Pcg64Mcg::seed_from_u64(uint64_t s) {
    // rand_core 0.9 SeedableRng::seed_from_u64: advance a PCG32 state and
    // emit its XSH-RR output as 4 little-endian bytes per chunk.
    uint8_t seed[16];
    for (int chunk = 0; chunk < 4; ++chunk) {
        s = s * 6364136223846793005ULL + 11634580027462260723ULL;
        const uint32_t xorshifted = static_cast<uint32_t>(((s >> 18) ^ s) >> 27);
        const uint32_t rot = static_cast<uint32_t>(s >> 59);
        const uint32_t x = rotr32(xorshifted, rot);
        for (int b = 0; b < 4; ++b) seed[chunk * 4 + b] = static_cast<uint8_t>(x >> (8 * b));
    }
    unsigned __int128 st = 0;
    for (int b = 15; b >= 0; --b) st = (st << 8) | seed[b];
    Pcg64Mcg g;
    g.state_ = st | 1;  // Mcg128Xsl64::new forces the low bit
    return g;
}

uint64_t Pcg64Mcg::next_u64() {
    state_ = state_ * kMcgMultiplier;
    const uint32_t rot = static_cast<uint32_t>(state_ >> 122);
    const uint64_t xsl = static_cast<uint64_t>(state_ >> 64) ^ static_cast<uint64_t>(state_);
    return rotr64(xsl, rot);
}

float Pcg64Mcg::next_f32() {
    const uint32_t v = next_u32() >> 8;
    return (1.0f / 16777216.0f) * static_cast<float>(v);
}

// ---------------------------------------------------------------------------
//  Model
// ---------------------------------------------------------------------------
bubble_model default_model() {
    bubble_model m;
    m.lambda = 0.5f;
    m.eps_ratio = 0.3f;
    m.alpha = 0.1f;
    m.eta = 0.3f;
    m.phi_b = 1.0f;
    m.dx = 1.0f;
    m.cfl = 0.2f;
    m.seed_kind = BUBBLE_SEED_CRITICAL;
    m.seed_value = 1.15f;  // SeedSize::DEFAULT_FACTOR
    return m;
}

std::string validate_model(const bubble_model &m) {
    // Order, comparisons and messages of Model::validate
    // (src/physics.rs:191-217); like the reference, a NaN passes every
    // check except the eps_ratio range test.
    if (!(m.eps_ratio >= 0.0f && m.eps_ratio < 1.0f) || m.eps_ratio <= 0.0f)
        return "eps_ratio must lie in (0, 1)";
    if (m.lambda <= 0.0f) return "lambda must be positive";
    if (m.alpha <= 0.0f) return "alpha must be positive";
    if (m.eta < 0.0f) return "eta must be non-negative";
    if (m.cfl <= 0.0f || m.cfl > 0.5f)
        return "cfl must lie in (0, 0.5]; see docs/NUMERICS.md";
    if (m.seed_kind == BUBBLE_SEED_CRITICAL) {
        if (m.seed_value <= 0.0f) return "seed factor must be positive";
    } else if (m.seed_kind == BUBBLE_SEED_CELLS) {
        if (m.seed_value <= 0.0f) return "seed radius must be positive";
    } else {
        return "seed_kind must be BUBBLE_SEED_CRITICAL or BUBBLE_SEED_CELLS";
    }
    return "";
}

Derived derive(const bubble_model &m) {
    Derived d;
    d.eps = m.eps_ratio * m.lambda * powi(m.phi_b, 4) / 12.0f;
    d.m2 = 0.5f * m.lambda * powi(m.phi_b, 2) - 6.0f * d.eps / powi(m.phi_b, 2);
    d.delta = 1.5f * m.lambda * m.phi_b - 6.0f * d.eps / powi(m.phi_b, 3);
    const float sqrt2 = 1.41421356237309504880f;  // std::f32::consts::SQRT_2
    d.wall_width = 2.0f * sqrt2 / (m.phi_b * std::sqrt(m.lambda));
    d.surface_tension = std::sqrt(m.lambda / 2.0f) * powi(m.phi_b, 3) / 6.0f;
    d.critical_radius = 2.0f * d.surface_tension / d.eps;
    d.e_ref = d.eps / m.alpha;
    d.t_ref = 1.0f;
    d.a_rad = d.e_ref / powi(d.t_ref, 4);
    d.dt = m.cfl * m.dx;
    const float seed = m.seed_kind == BUBBLE_SEED_CRITICAL
                           ? m.seed_value * d.critical_radius
                           : m.seed_value;
    d.seed_radius = std::max(seed, 0.25f * m.dx);
    d.critical_to_wall_ratio = 1.0f / m.eps_ratio;
    const float x = d.eps / (std::max(m.eta, 1e-6f) * d.surface_tension);
    d.estimated_wall_velocity = x / std::sqrt(1.0f + x * x);
    d.sound_speed = std::sqrt(1.0f / 3.0f);
    d.p_floor = 1e-7f * d.e_ref;
    d.e_floor = 1e-7f * d.e_ref;
    d.z_max = 0.9999f;
    return d;
}

SimParamsHost sim_params(const bubble_model &m, const uint32_t grid[3]) {
    const Derived d = derive(m);
    SimParamsHost p;
    p.nx = grid[0];
    p.ny = grid[1];
    p.nz = grid[2];
    p.dx = m.dx;
    p.inv_dx = 1.0f / m.dx;
    p.dt = d.dt;
    p.eta = m.eta;
    p.lambda = m.lambda;
    p.eps = d.eps;
    p.phi_b = m.phi_b;
    p.m2 = d.m2;
    p.delta = d.delta;
    p.a_rad = d.a_rad;
    p.wall_width = d.wall_width;
    p.p_floor = d.p_floor;
    p.e_floor = d.e_floor;
    p.z_max = d.z_max;
    p.e_ref = d.e_ref;
    p.t_ref = d.t_ref;
    return p;
}

// ---------------------------------------------------------------------------
//  Schedule
// ---------------------------------------------------------------------------
namespace {
float periodic_distance(const float a[3], const float b[3], const float n[3]) {
    float sum = 0.0f;
    for (int i = 0; i < 3; ++i) {
        float d = std::fabs(a[i] - b[i]);
        if (d > 0.5f * n[i]) d = n[i] - d;
        sum += d * d;
    }
    return std::sqrt(sum);
}
}  // namespace

std::vector<bubble_event> make_schedule(int mode, uint64_t count, float radius,
                                        const uint32_t grid[3], float duration,
                                        uint64_t seed) {
    Pcg64Mcg rng = Pcg64Mcg::seed_from_u64(seed);
    const float n[3] = {static_cast<float>(grid[0]), static_cast<float>(grid[1]),
                        static_cast<float>(grid[2])};
    const float min_sep = 2.5f * radius;
    std::vector<bubble_event> events;
    events.reserve(count);
    for (uint64_t k = 0; k < count; ++k) {
        float time = 0.0f;
        if (mode == BUBBLE_NUCLEATION_EXPONENTIAL) {
            const float growth = 4.0f;
            const float frac = (static_cast<float>(k) + 0.5f) / static_cast<float>(count);
            time = duration / growth * std::log(1.0f + frac * (std::exp(growth) - 1.0f));
        } else if (mode == BUBBLE_NUCLEATION_UNIFORM) {
            time = rng.next_f32() * duration;
        }
        bubble_event e;
        e.time = time;
        e.radius = radius;
        if (mode == BUBBLE_NUCLEATION_CENTRE) {
            for (int a = 0; a < 3; ++a) e.pos[a] = 0.5f * n[a];
        } else {
            float pos[3] = {0.0f, 0.0f, 0.0f};
            for (int attempt = 0; attempt < 64; ++attempt) {
                float cand[3];
                cand[0] = rng.next_f32() * n[0];
                cand[1] = rng.next_f32() * n[1];
                cand[2] = rng.next_f32() * n[2];
                bool ok = true;
                for (const auto &prev : events) {
                    if (!(periodic_distance(cand, prev.pos, n) > min_sep)) {
                        ok = false;
                        break;
                    }
                }
                std::memcpy(pos, cand, sizeof(pos));
                if (ok) break;
            }
            std::memcpy(e.pos, pos, sizeof(pos));
        }
        events.push_back(e);
    }
    std::stable_sort(events.begin(), events.end(),
                     [](const bubble_event &a, const bubble_event &b) { return a.time < b.time; });
    return events;
}

}  // namespace bubble

namespace bubble {

std::string validate_eos(const bubble_spec &spec) {
    switch (spec.eos) {
        case BUBBLE_EOS_BAG:
            return {};
        case BUBBLE_EOS_BAG_DOF:
            if (!(spec.eos_param[0] > 0.0f) || !std::isfinite(spec.eos_param[0]))
                return "the degrees-of-freedom ratio must be positive and finite";
            return {};
        case BUBBLE_EOS_GAMMA_LAW: {
            const float g = spec.eos_param[0], e0 = spec.eos_param[1];
            if (!(g > 1.0f && g <= 2.0f)) return "Gamma must lie in (1, 2] (a causal sound speed)";
            const float e_ref = derive(spec.model).e_ref;
            if (!(e0 >= 0.0f && e0 < 0.99f * e_ref))
                return "e0 must lie in [0, 0.99 e_ref) so the reference pressure is positive";
            if (spec.precision != BUBBLE_PRECISION_SINGLE)
                return "the gamma-law equation of state is built for BUBBLE_PRECISION_SINGLE";
            return {};
        }
        case BUBBLE_EOS_THERMAL: {
            // For T >= T_ref / sqrt(2) and |phi| <= phi_b: gamma <= a T_ref^2 /
            // (6 phi_b^2) keeps the thermal mass term below half the radiation
            // pressure (p >= a T^4 / 6 at A = 0) and the state on the branch
            // T >= sqrt(3 gamma / (4a)) |phi|; A <= a T_ref^3 / (sqrt(2) phi_b^3)
            // keeps p <= e (A phi^3 <= 2 a T^3), so |Z| <= E holds for every
            // physical state and the regularisation never alters one
            const float g = spec.eos_param[0], a_c = spec.eos_param[1];
            const Derived d = derive(spec.model);
            const float a = d.a_rad, t_ref = d.t_ref, pb = spec.model.phi_b;
            const float g_max = a * t_ref * t_ref / (6.0f * pb * pb);
            const float a_max = a * t_ref * t_ref * t_ref / (1.41421356f * pb * pb * pb);
            if (!(g >= 0.0f && g <= g_max)) return "gamma must lie in [0, a T_ref^2 / (6 phi_b^2)]";
            if (!(a_c >= 0.0f && a_c <= a_max)) return "A must lie in [0, a T_ref^3 / (sqrt(2) phi_b^3)]";
            if (spec.precision != BUBBLE_PRECISION_SINGLE)
                return "the thermal potential is built for BUBBLE_PRECISION_SINGLE";
            return {};
        }
        default:
            return "unknown equation of state";
    }
}

}  // namespace bubble
