/*
 * bubble.h -- C ABI of the GB300-native lattice time step of
 * bubble-simulation (AgenttiX/bubble-simulation).
 *
 * The reference drives its lattice through the Rust type `Simulation`
 * (src/gpu/sim.rs:180-1026), built from a `SimulationSpec`
 * (src/gpu/sim.rs:246-255) whose physics lives in `Model`
 * (src/physics.rs:44-218) and whose bubbles come from `make_schedule`
 * (src/physics.rs:248-296).  Every entry point below replaces one of those
 * methods; the comment on each names the reference symbol it stands in for.
 *
 * Conventions
 *   - Every fallible call returns an int status: 0 (BUBBLE_OK) or a negative
 *     BUBBLE_ERR_* code.  The message of the last failure on the calling
 *     thread is returned by bubble_last_error().
 *   - The library owns every device allocation behind a handle; callers pass
 *     only host pointers and sizes (and, optionally, a cudaStream_t as void*).
 *   - Lattice index is i = (z*ny + y)*nx + x (shaders/common.wgsl:17-23).
 *     `field` is (phi, pi) per cell, `fluid` is (E, Zx, Zy, Zz) per cell
 *     (src/gpu/sim.rs:7-21).
 *   - There is no CPU fallback: a call that needs the GPU fails with
 *     BUBBLE_ERR_CUDA when no device is present.
 */
#ifndef BUBBLE_GB300_H
#define BUBBLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/*  Status codes                                                            */
/* ------------------------------------------------------------------------ */
#define BUBBLE_OK 0
#define BUBBLE_ERR_INVALID (-1)   /* bad argument, model or lattice size      */
#define BUBBLE_ERR_CUDA (-2)      /* CUDA runtime error / no device           */
#define BUBBLE_ERR_MEMORY (-3)    /* allocation failed or admission refused   */
#define BUBBLE_ERR_NONFINITE (-4) /* diagnostics are not finite (blow-up)     */
#define BUBBLE_ERR_STATE (-5)     /* call not valid in the current state      */
#define BUBBLE_ERR_TIMEOUT (-6)   /* a bounded device wait gave up            */

/* Smallest lattice axis the two-cell stencil can address
 * (src/gpu/sim.rs:45-47). */
#define BUBBLE_MIN_GRID 8u
/* Largest axis accepted (src/gpu/sim.rs:49-51). */
#define BUBBLE_MAX_GRID 2048u
/* Largest lattice accepted: the stage kernels index cells in 32 bits (a
 * lattice this large holds 309 GB of FP32 state, more than one GB300's
 * HBM). */
#define BUBBLE_MAX_CELLS 4294967295ull
/* Bubbles stamped by one nucleation launch (src/gpu/sim.rs:40-41). */
#define BUBBLE_MAX_BATCH 1024u

/* ------------------------------------------------------------------------ */
/*  Physics model (src/physics.rs:23-83)                                    */
/* ------------------------------------------------------------------------ */
/* SeedSize (src/physics.rs:29-42). */
#define BUBBLE_SEED_CRITICAL 0 /* seed_value = multiple of R_c */
#define BUBBLE_SEED_CELLS 1    /* seed_value = radius in cells  */

typedef struct bubble_model {
    float lambda;     /* quartic coupling                                  */
    float eps_ratio;  /* eps / (lambda phi_b^4 / 12), in (0, 1)            */
    float alpha;      /* eps / e_ref                                       */
    float eta;        /* wall friction                                     */
    float phi_b;      /* broken-phase field value (1)                      */
    float dx;         /* lattice spacing (1)                               */
    float cfl;        /* dt = cfl * dx, in (0, 0.5]                        */
    int32_t seed_kind;  /* BUBBLE_SEED_*                                   */
    float seed_value;   /* factor or cells, per seed_kind                  */
} bubble_model;

/* Every derived quantity of `impl Model` (src/physics.rs:85-189), in f32
 * with the reference's evaluation order. */
typedef struct bubble_derived {
    float eps, m2, delta, wall_width, surface_tension, critical_radius;
    float e_ref, t_ref, a_rad, dt, seed_radius, critical_to_wall_ratio;
    float estimated_wall_velocity, sound_speed;
    /* SimParams floors (src/gpu/sim.rs:632-636) */
    float p_floor, e_floor, z_max;
} bubble_derived;

/* Model::default() (src/physics.rs:70-83). */
void bubble_model_default(bubble_model *out);
/* Model::validate (src/physics.rs:191-217).  BUBBLE_ERR_INVALID with the
 * reference's message on failure. */
int bubble_model_validate(const bubble_model *model);
/* Model::{eps, m2, delta, ...} (src/physics.rs:85-189). */
int bubble_model_derived(const bubble_model *model, bubble_derived *out);

/* ------------------------------------------------------------------------ */
/*  Nucleation schedule (src/physics.rs:224-308)                            */
/* ------------------------------------------------------------------------ */
#define BUBBLE_NUCLEATION_SIMULTANEOUS 0 /* NucleationMode::Simultaneous     */
#define BUBBLE_NUCLEATION_EXPONENTIAL 1  /* NucleationMode::Exponential      */
/* Two seeding modes the reference does not have, needed by the benchmark
 * workloads: every bubble at the box centre at t = 0, and nucleation times
 * drawn uniformly in [0, duration). */
#define BUBBLE_NUCLEATION_CENTRE 2
#define BUBBLE_NUCLEATION_UNIFORM 3

/* BubbleEvent (src/physics.rs:236-241). */
typedef struct bubble_event {
    float time;
    float pos[3];
    float radius;
} bubble_event;

/* make_schedule (src/physics.rs:248-296): Pcg64Mcg seeded from `seed`,
 * positions rng.random::<f32>() * n per axis with up to 64 attempts at
 * min separation 2.5 radius, then a stable sort by time.  Writes
 * min(count, capacity) events; *n_out = count.  */
int bubble_make_schedule(int32_t mode, uint64_t count, float radius,
                         const uint32_t grid[3], float duration, uint64_t seed,
                         bubble_event *out, uint64_t capacity,
                         uint64_t *n_out);

/* ------------------------------------------------------------------------ */
/*  Simulation spec (src/gpu/sim.rs:244-255)                                */
/* ------------------------------------------------------------------------ */
/* Precision (src/gpu/preprocess.rs Precision::{Single, Double}). */
#define BUBBLE_PRECISION_SINGLE 0 /* FP32 state, FP64 reductions           */
#define BUBBLE_PRECISION_MIXED 1  /* SINGLE + FP64 con2prim where gamma > 3 */
#define BUBBLE_PRECISION_DOUBLE 2 /* FP64 state and arithmetic throughout   */
/* MIXED with the fluid energy stored as E - e_ref and the pressure carried
 * as p - e_ref/3, so the weak-transition perturbation keeps its FP32 digits
 * (docs/PRECISION.md:117-124 of the reference, "evolve perturbations").
 * copy_state/load_state move the stored values: fluid.x is E - e_ref. */
#define BUBBLE_PRECISION_PERTURBATION 3
/* Arithmetic mode of the FP32 kernels. */
#define BUBBLE_MATH_FAST 0   /* FMA contraction, shared reciprocals        */
#define BUBBLE_MATH_STRICT 1 /* no contraction, IEEE div/sqrt, the WGSL
                                evaluation order: bit-identical with a
                                plain IEEE single-precision restatement   */

/* Equation of state.  The reference's swap point is the body of the ten
 * eos_* functions (docs/EOS.md:10-23); here each equation of state is a
 * compiled policy of the kernels, chosen per simulation. */
#define BUBBLE_EOS_BAG 0       /* e = 3p, closed-form inversion: the reference's   */
#define BUBBLE_EOS_BAG_DOF 1   /* bag with a(phi) = a_rad (1 + (r - 1) smoothstep(phi/phi_b)),
                                  r = eos_param[0]: only T changes (docs/EOS.md:58-84) */
#define BUBBLE_EOS_GAMMA_LAW 2 /* e = p/(Gamma - 1) + e0, c_s^2 = Gamma - 1, Newton
                                  inversion (docs/EOS.md:86-118); Gamma = eos_param[0]
                                  in (1, 2], e0 = eos_param[1] in [0, e_ref)          */
#define BUBBLE_EOS_THERMAL 3   /* temperature-dependent potential (docs/EOS.md:120-150):
                                  V(phi, T) = V(phi) + gamma/2 (T^2 - T_ref^2) phi^2
                                  - A/3 (T - T_ref) phi^3, the plasma carrying the
                                  T-dependent part, p = a T^4/3 - that part; gamma =
                                  eos_param[0] in [0, a T_ref^2 / (6 phi_b^2)], A =
                                  eos_param[1] in [0, a T_ref^3 / (sqrt(2) phi_b^3)]
                                  (p <= e); A = delta / T_ref would be the recipe's
                                  -A T phi^3 / 3 form; FP32 only                     */

typedef struct bubble_spec {
    bubble_model model;
    uint32_t grid[3];
    int32_t nucleation;        /* BUBBLE_NUCLEATION_*                     */
    uint64_t bubbles;          /* number of scheduled bubbles             */
    float nucleation_duration; /* time over which nucleation completes    */
    uint64_t seed;             /* schedule seed                           */
    int32_t precision;         /* BUBBLE_PRECISION_*                      */
    int32_t math;              /* BUBBLE_MATH_*                           */
    int32_t eos;               /* BUBBLE_EOS_*                            */
    float eos_param[2];        /* see BUBBLE_EOS_*                        */
} bubble_spec;

/* Config defaults (src/config.rs:197-297) as a SimulationSpec. */
void bubble_spec_default(bubble_spec *out);

/* Checks the spec's equation-of-state selection (policy, parameter ranges,
 * supported arithmetic); BUBBLE_ERR_INVALID with a message otherwise. */
int bubble_eos_validate(const bubble_spec *spec);

/* ------------------------------------------------------------------------ */
/*  Diagnostics (src/gpu/sim.rs:141-167, shaders/reduce.wgsl:15-79)          */
/* ------------------------------------------------------------------------ */
typedef struct bubble_diag {
    /* Diagnostics fields: sums / cell count. */
    float mean_energy;       /* 1/2 pi^2 + 1/2|grad phi|^2 + V(phi) + E  */
    float broken_fraction;   /* fraction of cells with phi > phi_b / 2    */
    float mean_kinetic;      /* (E + p) v^2                               */
    float mean_fluid_energy; /* E                                         */
    float max_velocity;      /* max |v|                                   */
    float kinetic_fraction;  /* Diagnostics::kinetic_fraction            */
    /* The same sums, accumulated in FP64. */
    double sum_energy, sum_broken, sum_kinetic, sum_fluid_energy;
    double mean_energy_f64, mean_kinetic_f64;
    uint64_t cells;
} bubble_diag;

/* ------------------------------------------------------------------------ */
/*  Host-side helpers with no device work                                   */
/* ------------------------------------------------------------------------ */
/* stage_slots (src/gpu/sim.rs:1046-1051): out = {in0,out0,in1,out1,in2,out2}. */
int bubble_stage_slots(uint32_t cur, uint32_t out[6]);
/* RK3 table (src/gpu/sim.rs:133-135): out = {a0,a1} x 3 stages. */
void bubble_rk3_coefficients(float out[6]);
/* Lattice::lattice_bytes (src/gpu/sim.rs:705-715), for this layout:
 * 3 RK slots x 24 B per cell; no primitive cache and no visualisation
 * texture are held, so this is 72 B per cell. */
uint64_t bubble_lattice_bytes(const uint32_t grid[3]);
/* Bytes per cell of bubble_lattice_bytes for a precision. */
uint64_t bubble_bytes_per_cell(int32_t precision);
/* Simulation::max_cubic_size (src/gpu/sim.rs:717-733): the largest cubic
 * side allowed by a per-buffer limit (bytes of one 16 B/cell fluid slot) and
 * an optional memory budget (bubble_lattice_bytes per cell), clamped to
 * [BUBBLE_MIN_GRID, BUBBLE_MAX_GRID] as there and, beyond the reference, to
 * 1625, the largest cube within BUBBLE_MAX_CELLS. */
int bubble_max_cubic_size(uint64_t max_buffer_bytes, uint64_t budget_bytes,
                          int32_t has_budget, uint32_t *side,
                          int32_t *limited_by_memory);

/* VramInfo (src/gpu/vram.rs:22-50). */
typedef struct bubble_vram_info {
    uint64_t capacity;
    uint64_t budget;  /* valid when has_budget */
    uint64_t used;    /* valid when has_budget */
    int32_t has_budget;
} bubble_vram_info;
/* vram::query (src/gpu/vram.rs:71-83), answered by cudaMemGetInfo:
 * capacity = total, budget = total, used = total - free. */
int bubble_vram_query(bubble_vram_info *out);
/* VramInfo::available (src/gpu/vram.rs:39-44). */
uint64_t bubble_vram_available(const bubble_vram_info *info);
/* vram::lattice_budget (src/gpu/vram.rs:52-69): 85 % of free + current. */
uint64_t bubble_lattice_budget(uint64_t available, uint64_t current_lattice);

/* ------------------------------------------------------------------------ */
/*  Simulation (src/gpu/sim.rs:180-1026)                                    */
/* ------------------------------------------------------------------------ */
typedef struct bubble_sim bubble_sim;

/* Simulation::new (src/gpu/sim.rs:258-607): validates the model and the
 * lattice, allocates three RK slots, builds the schedule and resets. */
int bubble_create(const bubble_spec *spec, bubble_sim **out);
/* Drop for Simulation: releases every device allocation. */
void bubble_destroy(bubble_sim *sim);
/* Launch on this CUDA stream (a cudaStream_t passed as void*; NULL selects
 * the library's own stream).  The reference records into a caller-owned
 * wgpu::CommandEncoder (src/gpu/sim.rs:829-834); this is its analogue. */
int bubble_set_stream(bubble_sim *sim, void *stream);
/* Simulation::reset (src/gpu/sim.rs:788-821).  With events != NULL the
 * schedule is replaced by the n given events. */
int bubble_reset(bubble_sim *sim, const bubble_event *events, uint64_t n);
/* Simulation::set_model (src/gpu/sim.rs:658-670).  An invalid model is not
 * applied (the reference ignores it silently) and BUBBLE_ERR_INVALID is
 * returned. */
int bubble_set_model(bubble_sim *sim, const bubble_model *model);
/* Simulation::resize (src/gpu/sim.rs:735-762): validates first, releases
 * the old lattice before allocating the new one, restarts the run. */
int bubble_resize(bubble_sim *sim, const uint32_t grid[3]);
/* Simulation::record_steps (src/gpu/sim.rs:827-841): nucleate the events
 * due at the current time (once), then n SSP-RK3 steps.  Asynchronous. */
int bubble_record_steps(bubble_sim *sim, uint32_t n_steps);
/* headless::advance's step loop (src/headless.rs:126-131): n times
 * record_steps(1), so due events are checked before every step. */
int bubble_advance(bubble_sim *sim, uint64_t n_steps);
/* record_diagnostics + poll (src/gpu/sim.rs:948-1010), synchronous: the
 * FP64 reduction of the current slot.  BUBBLE_ERR_NONFINITE when the energy
 * or max|v| is not finite (src/headless.rs:63-67); *out is still filled. */
int bubble_diagnostics(bubble_sim *sim, bubble_diag *out);
/* Simulation::nucleate_now (src/gpu/sim.rs:1012-1025): queue one bubble at
 * a random position drawn from a Pcg64Mcg seeded with rng_seed. */
int bubble_nucleate_now(bubble_sim *sim, uint64_t rng_seed);
/* Wait for all work queued on the simulation's stream. */
int bubble_synchronize(bubble_sim *sim);

/* Field accessors (src/gpu/sim.rs:180-199, 676-703). */
float bubble_time(const bubble_sim *sim);
uint64_t bubble_steps(const bubble_sim *sim);
uint64_t bubble_cell_count(const bubble_sim *sim);
uint64_t bubble_remaining_bubbles(const bubble_sim *sim);
uint64_t bubble_device_memory_bytes(const bubble_sim *sim);
int bubble_get_grid(const bubble_sim *sim, uint32_t grid[3]);
int bubble_get_model(const bubble_sim *sim, bubble_model *out);
int bubble_get_schedule(const bubble_sim *sim, bubble_event *out,
                        uint64_t capacity, uint64_t *n_out);

/* State transfer (no reference counterpart: the reference never reads the
 * lattice back; these serve checkpoint/resume and parity checks).
 * The current slot U^n, FP32 state: field = 2 floats/cell, fluid = 4. */
int bubble_copy_state(bubble_sim *sim, float *field, float *fluid);
int bubble_load_state(bubble_sim *sim, const float *field, const float *fluid);
/* FP64 state (BUBBLE_PRECISION_DOUBLE only). */
int bubble_copy_state_f64(bubble_sim *sim, double *field, double *fluid);
int bubble_load_state_f64(bubble_sim *sim, const double *field,
                          const double *fluid);

/* Version string of the library. */
const char *bubble_version(void);
/* Message of the last failed call on this thread ("" when none). */
const char *bubble_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_GB300_H */
