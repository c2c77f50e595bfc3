// extern "C" boundary: include/bubble.h.  Each entry point validates its
// arguments, forwards to the C++ driver and turns failures into a status
// code plus a thread-local message.
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>

#include "../../include/bubble.h"
#include "../../include/bubble_ext.h"
#include "physics.h"
#include "sim_handle.h"

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
int done(int code, const std::string &msg) {
    if (code != BUBBLE_OK) g_last_error = msg;
    return code;
}
#define NEED(ptr)                                                     \
    do {                                                              \
        if (!(ptr)) return fail(BUBBLE_ERR_INVALID, #ptr " is NULL"); \
    } while (0)
}  // namespace

namespace bubble {
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace bubble

extern "C" {

const char *bubble_version(void) { return "bubble-gb300 0.1.0"; }
const char *bubble_last_error(void) { return g_last_error.c_str(); }

void bubble_model_default(bubble_model *out) {
    if (out) *out = bubble::default_model();
}

int bubble_model_validate(const bubble_model *model) {
    NEED(model);
    const std::string msg = bubble::validate_model(*model);
    if (!msg.empty()) return fail(BUBBLE_ERR_INVALID, msg);
    return BUBBLE_OK;
}

int bubble_model_derived(const bubble_model *model, bubble_derived *out) {
    NEED(model);
    NEED(out);
    const bubble::Derived d = bubble::derive(*model);
    out->eps = d.eps;
    out->m2 = d.m2;
    out->delta = d.delta;
    out->wall_width = d.wall_width;
    out->surface_tension = d.surface_tension;
    out->critical_radius = d.critical_radius;
    out->e_ref = d.e_ref;
    out->t_ref = d.t_ref;
    out->a_rad = d.a_rad;
    out->dt = d.dt;
    out->seed_radius = d.seed_radius;
    out->critical_to_wall_ratio = d.critical_to_wall_ratio;
    out->estimated_wall_velocity = d.estimated_wall_velocity;
    out->sound_speed = d.sound_speed;
    out->p_floor = d.p_floor;
    out->e_floor = d.e_floor;
    out->z_max = d.z_max;
    return BUBBLE_OK;
}

int bubble_make_schedule(int32_t mode, uint64_t count, float radius, const uint32_t grid[3],
                         float duration, uint64_t seed, bubble_event *out, uint64_t capacity,
                         uint64_t *n_out) {
    NEED(grid);
    if (mode < BUBBLE_NUCLEATION_SIMULTANEOUS || mode > BUBBLE_NUCLEATION_UNIFORM)
        return fail(BUBBLE_ERR_INVALID, "unknown nucleation mode");
    const auto ev = bubble::make_schedule(mode, count, radius, grid, duration, seed);
    if (n_out) *n_out = ev.size();
    if (out) {
        const uint64_t m = ev.size() < capacity ? ev.size() : capacity;
        std::memcpy(out, ev.data(), m * sizeof(bubble_event));
    }
    return BUBBLE_OK;
}

void bubble_spec_default(bubble_spec *out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->model = bubble::default_model();
    out->grid[0] = out->grid[1] = out->grid[2] = 192;
    out->nucleation = BUBBLE_NUCLEATION_EXPONENTIAL;
    out->bubbles = 12;
    out->nucleation_duration = 60.0f;
    out->seed = 1;
    out->precision = BUBBLE_PRECISION_SINGLE;
    out->math = BUBBLE_MATH_FAST;
    out->eos = BUBBLE_EOS_BAG;
    out->eos_param[0] = 1.0f;
    out->eos_param[1] = 0.0f;
}

int bubble_eos_validate(const bubble_spec *spec) {
    NEED(spec);
    const std::string msg = bubble::validate_eos(*spec);
    if (!msg.empty()) return fail(BUBBLE_ERR_INVALID, msg);
    return BUBBLE_OK;
}

int bubble_stage_slots(uint32_t cur, uint32_t out[6]) {
    NEED(out);
    uint32_t in[3], o[3];
    bubble::stage_slots(cur, in, o);
    for (int s = 0; s < 3; ++s) {
        out[2 * s] = in[s];
        out[2 * s + 1] = o[s];
    }
    return BUBBLE_OK;
}

void bubble_rk3_coefficients(float out[6]) {
    if (!out) return;
    for (int s = 0; s < 3; ++s) {
        out[2 * s] = bubble::kRK3[s][0];
        out[2 * s + 1] = bubble::kRK3[s][1];
    }
}

uint64_t bubble_bytes_per_cell(int32_t precision) {
    return precision == BUBBLE_PRECISION_DOUBLE ? 3ull * (16 + 32) : 3ull * (8 + 16);
}

uint64_t bubble_lattice_bytes(const uint32_t grid[3]) {
    if (!grid) return 0;
    const uint64_t cells = (uint64_t)grid[0] * grid[1] * grid[2];
    return cells * bubble_bytes_per_cell(BUBBLE_PRECISION_SINGLE);
}

int bubble_max_cubic_size(uint64_t max_buffer_bytes, uint64_t budget_bytes, int32_t has_budget,
                          uint32_t *side, int32_t *limited_by_memory) {
    NEED(side);
    auto cbrt_side = [](uint64_t cells) { return (uint32_t)std::floor(std::cbrt((double)cells)); };
    const uint32_t by_buffer = cbrt_side(max_buffer_bytes / 16);
    const uint32_t by_budget =
        has_budget ? cbrt_side(budget_bytes / bubble_bytes_per_cell(BUBBLE_PRECISION_SINGLE)) : 0xffffffffu;
    uint32_t s = by_buffer < by_budget ? by_buffer : by_budget;
    if (s < BUBBLE_MIN_GRID) s = BUBBLE_MIN_GRID;
    if (s > BUBBLE_MAX_GRID) s = BUBBLE_MAX_GRID;
    // and the largest cube the stage kernels' 32-bit cell index covers
    while ((uint64_t)s * s * s > BUBBLE_MAX_CELLS) --s;
    *side = s;
    if (limited_by_memory) *limited_by_memory = by_budget < by_buffer ? 1 : 0;
    return BUBBLE_OK;
}

int bubble_vram_query(bubble_vram_info *out) {
    NEED(out);
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(BUBBLE_ERR_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
    }
    out->capacity = total_b;
    out->budget = total_b;
    out->used = total_b - free_b;
    out->has_budget = 1;
    return BUBBLE_OK;
}

uint64_t bubble_vram_available(const bubble_vram_info *info) {
    if (!info) return 0;
    if (info->has_budget) return info->budget > info->used ? info->budget - info->used : 0;
    return info->capacity;
}

uint64_t bubble_lattice_budget(uint64_t available, uint64_t current_lattice) {
    uint64_t sum = available + current_lattice;
    if (sum < available) sum = UINT64_MAX;  // saturating add
    return (uint64_t)((double)sum * 0.85);
}

// ---------------------------------------------------------------------------
//  Simulation
// ---------------------------------------------------------------------------
int bubble_create(const bubble_spec *spec, bubble_sim **out) {
    NEED(spec);
    NEED(out);
    *out = nullptr;
    std::string err;
    std::unique_ptr<bubble::Simulation> impl;
    const int rc = bubble::Simulation::create(*spec, impl, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    *out = new bubble_sim{std::move(impl)};
    return BUBBLE_OK;
}

void bubble_destroy(bubble_sim *sim) { delete sim; }

#define SIM_CALL(expr)                                                  \
    do {                                                                \
        if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL"); \
        std::string err;                                                \
        const int rc = (expr);                                          \
        return done(rc, err);                                           \
    } while (0)

int bubble_set_stream(bubble_sim *sim, void *stream) {
    SIM_CALL(sim->impl->set_stream(static_cast<cudaStream_t>(stream), err));
}
int bubble_reset(bubble_sim *sim, const bubble_event *events, uint64_t n) {
    SIM_CALL(sim->impl->reset(events, n, err));
}
int bubble_set_model(bubble_sim *sim, const bubble_model *model) {
    NEED(model);
    SIM_CALL(sim->impl->set_model(*model, err));
}
int bubble_resize(bubble_sim *sim, const uint32_t grid[3]) {
    NEED(grid);
    SIM_CALL(sim->impl->resize(grid, err));
}
int bubble_record_steps(bubble_sim *sim, uint32_t n_steps) {
    SIM_CALL(sim->impl->record_steps(n_steps, err));
}
int bubble_advance(bubble_sim *sim, uint64_t n_steps) { SIM_CALL(sim->impl->advance(n_steps, err)); }
int bubble_diagnostics(bubble_sim *sim, bubble_diag *out) {
    NEED(out);
    SIM_CALL(sim->impl->diagnostics(out, err));
}
int bubble_nucleate_now(bubble_sim *sim, uint64_t rng_seed) {
    SIM_CALL(sim->impl->nucleate_now(rng_seed, err));
}
int bubble_synchronize(bubble_sim *sim) { SIM_CALL(sim->impl->synchronize(err)); }

float bubble_time(const bubble_sim *sim) { return sim && sim->impl ? sim->impl->time() : 0.0f; }
uint64_t bubble_steps(const bubble_sim *sim) { return sim && sim->impl ? sim->impl->steps() : 0; }
uint64_t bubble_cell_count(const bubble_sim *sim) {
    return sim && sim->impl ? sim->impl->cell_count() : 0;
}
uint64_t bubble_remaining_bubbles(const bubble_sim *sim) {
    return sim && sim->impl ? sim->impl->remaining_bubbles() : 0;
}
uint64_t bubble_device_memory_bytes(const bubble_sim *sim) {
    return sim && sim->impl ? sim->impl->device_memory_bytes() : 0;
}
int bubble_get_grid(const bubble_sim *sim, uint32_t grid[3]) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    NEED(grid);
    std::memcpy(grid, sim->impl->grid(), 3 * sizeof(uint32_t));
    return BUBBLE_OK;
}
int bubble_get_model(const bubble_sim *sim, bubble_model *out) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    NEED(out);
    *out = sim->impl->model();
    return BUBBLE_OK;
}
int bubble_get_schedule(const bubble_sim *sim, bubble_event *out, uint64_t capacity, uint64_t *n_out) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    const auto &s = sim->impl->schedule();
    if (n_out) *n_out = s.size();
    if (out) {
        const uint64_t m = s.size() < capacity ? s.size() : capacity;
        std::memcpy(out, s.data(), m * sizeof(bubble_event));
    }
    return BUBBLE_OK;
}

int bubble_copy_state(bubble_sim *sim, float *field, float *fluid) {
    SIM_CALL(sim->impl->copy_state(field, fluid, false, err));
}
int bubble_load_state(bubble_sim *sim, const float *field, const float *fluid) {
    SIM_CALL(sim->impl->load_state(field, fluid, false, err));
}
int bubble_copy_state_f64(bubble_sim *sim, double *field, double *fluid) {
    SIM_CALL(sim->impl->copy_state(field, fluid, true, err));
}
int bubble_load_state_f64(bubble_sim *sim, const double *field, const double *fluid) {
    SIM_CALL(sim->impl->load_state(field, fluid, true, err));
}

// ---------------------------------------------------------------------------
//  Extensions (include/bubble_ext.h)
// ---------------------------------------------------------------------------
int bubble_ext_set_path(bubble_sim *sim, int32_t path) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    if (path != BUBBLE_PATH_FUSED && path != BUBBLE_PATH_REFERENCE)
        return fail(BUBBLE_ERR_INVALID, "unknown kernel path");
    sim->impl->set_path(static_cast<bubble::KernelPath>(path));
    return BUBBLE_OK;
}
int bubble_ext_test_expire_stage_wait(bubble_sim *sim, uint32_t extra_bytes, int32_t wait_shift) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    if (extra_bytes < 1 || extra_bytes > 65536) return fail(BUBBLE_ERR_INVALID, "extra_bytes must be 1..65536");
    if (wait_shift < 10 || wait_shift > 31) return fail(BUBBLE_ERR_INVALID, "wait_shift must be 10..31");
    sim->impl->arm_wait_expiry(extra_bytes, wait_shift);
    return BUBBLE_OK;
}
int bubble_ext_set_tile(bubble_sim *sim, int32_t ty, int32_t lz) {
    SIM_CALL(sim->impl->set_tile(bubble::TileShape{bubble::tile_x_for(ty), ty, lz}, err));
}
int bubble_ext_set_stage_form(bubble_sim *sim, int32_t form) {
    SIM_CALL(sim->impl->set_stage_form(form, err));
}
int bubble_ext_get_tile(const bubble_sim *sim, int32_t *ty, int32_t *lz) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    const bubble::TileShape t = sim->impl->tile();
    if (ty) *ty = t.ty;
    if (lz) *lz = t.lz;
    return BUBBLE_OK;
}
int bubble_ext_device_state(bubble_sim *sim, void **field, void **fluid) {
    if (!sim || !sim->impl) return fail(BUBBLE_ERR_INVALID, "sim is NULL");
    sim->impl->device_state(field, fluid);
    return BUBBLE_OK;
}
void *bubble_ext_stream(bubble_sim *sim) {
    return sim && sim->impl ? static_cast<void *>(sim->impl->stream()) : nullptr;
}
uint64_t bubble_ext_launches(const bubble_sim *sim) {
    return sim && sim->impl ? sim->impl->launches() : 0;
}
void bubble_ext_inject_allocation_failure(void) { bubble::inject_allocation_failure(); }

}  // extern "C"
