// Host physics: parameter derivation, the nucleation schedule and its PRNG.
//
// Restates `impl Model` (src/physics.rs:85-218) and `make_schedule`
// (src/physics.rs:243-308) in single precision with the reference's
// evaluation order, so derived constants and seeding positions match the
// Rust host bit for bit where the same IEEE operations are performed.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bubble.h"

namespace bubble {

// Pcg64Mcg = Mcg128Xsl64 of rand_pcg 0.9: a 128-bit multiplicative
// congruential generator with the XSL-RR output function (O'Neill 2014),
// seeded through rand_core 0.9's `seed_from_u64` (a PCG32 stream filling
// the 16 seed bytes little-endian) and sampled as f32 by rand 0.9's
// StandardUniform: the top 24 bits of next_u32 scaled by 2^-24.
class Pcg64Mcg {
   public:
    static Pcg64Mcg seed_from_u64(uint64_t seed);
    uint64_t next_u64();
    uint32_t next_u32() { return static_cast<uint32_t>(next_u64()); }
    float next_f32();
    unsigned __int128 state() const { return state_; }

   private:
    unsigned __int128 state_ = 1;
};

// Derived model quantities (src/physics.rs:85-189).
struct Derived {
    float eps, m2, delta, wall_width, surface_tension, critical_radius;
    float e_ref, t_ref, a_rad, dt, seed_radius, critical_to_wall_ratio;
    float estimated_wall_velocity, sound_speed;
    float p_floor, e_floor, z_max;
};

bubble_model default_model();
// Returns "" when valid, else the reference's message.
std::string validate_model(const bubble_model &m);
Derived derive(const bubble_model &m);

std::vector<bubble_event> make_schedule(int mode, uint64_t count, float radius,
                                        const uint32_t grid[3], float duration,
                                        uint64_t seed);

// SimParams values used by every kernel (src/gpu/sim.rs:613-644).
struct SimParamsHost {
    uint32_t nx, ny, nz;
    float dx, inv_dx, dt, eta, lambda, eps, phi_b, m2, delta, a_rad,
        wall_width, p_floor, e_floor, z_max, e_ref, t_ref;
};
SimParamsHost sim_params(const bubble_model &m, const uint32_t grid[3]);

// Equation-of-state selection of a spec: the policy exists, its parameters
// are in range, and the arithmetic form supports it.  Empty string when valid.
std::string validate_eos(const bubble_spec &spec);

// RK3 (src/gpu/sim.rs:133-135).
extern const float kRK3[3][2];

// Sets the message returned by bubble_last_error() on this thread.
void set_last_error(const std::string &msg);

// stage_slots (src/gpu/sim.rs:1046-1051).
inline void stage_slots(uint32_t cur, uint32_t in[3], uint32_t out[3]) {
    const uint32_t a = cur % 3, b = (cur + 1) % 3, c = (cur + 2) % 3;
    in[0] = a; out[0] = b;
    in[1] = b; out[1] = c;
    in[2] = c; out[2] = b;
}

}  // namespace bubble
