// The simulation driver: see simulation.h.
#include "simulation.h"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "../../include/bubble_ext.h"
#include "launch.h"

namespace bubble {

namespace {

std::atomic<int> g_fail_next_alloc{0};

#define BUBBLE_CUDA(call, what)                                                   \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string(what) + ": " + cudaGetErrorString(e_);              \
            return BUBBLE_ERR_CUDA;                                               \
        }                                                                         \
    } while (0)

cudaError_t device_alloc(void **p, size_t bytes) {
    if (g_fail_next_alloc.exchange(0) != 0) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

std::string check_grid(const uint32_t grid[3]) {
    for (int a = 0; a < 3; ++a) {
        if (grid[a] < BUBBLE_MIN_GRID)
            return "grid axis " + std::to_string(a) + " is " + std::to_string(grid[a]) +
                   "; the 5-point stencil needs at least " + std::to_string(BUBBLE_MIN_GRID) +
                   " cells";
        if (grid[a] > BUBBLE_MAX_GRID)
            return "grid axis " + std::to_string(a) + " is " + std::to_string(grid[a]) +
                   "; the largest supported axis is " + std::to_string(BUBBLE_MAX_GRID);
    }
    const uint64_t cells = (uint64_t)grid[0] * grid[1] * grid[2];
    if (cells > BUBBLE_MAX_CELLS)
        return "lattice of " + std::to_string(cells) + " cells; the stage kernels index at most " +
               std::to_string(BUBBLE_MAX_CELLS) + " cells";
    return "";
}

}  // namespace

void inject_allocation_failure() { g_fail_next_alloc.store(1); }

int default_chunk(const uint32_t grid[3], int ty, bool fp32) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (fp32 && ty == 16) {
        // the cheapest (chunk, form) of the cost model; ties go to longer
        // chunks (fewer warm-up planes)
        double best = 1e300;
        int best_lz = (int)grid[2];
        const int max_chunks = ((int)grid[2] + 3) / 4;  // chunks of >= 4 planes
        for (int chunks = 1; chunks <= max_chunks; ++chunks) {
            const int lz = ((int)grid[2] + chunks - 1) / chunks;
            const double c = std::min(column_stage_cost(grid[0], grid[1], grid[2], lz, false, sms),
                                      column_stage_cost(grid[0], grid[1], grid[2], lz, true, sms));
            if (c < best * (1.0 - 1e-9)) {
                best = c;
                best_lz = lz;
            }
        }
        return best_lz;
    }
    const long tx = tile_x_for(ty);
    const long tiles = (long)((grid[0] + tx - 1) / tx) * (long)((grid[1] + ty - 1) / ty);
    // Other tiles and FP64, two regimes (measured with 32 x 8 tiles, ms per
    // step, 8 bubbles):
    //  * lattices too small to fill the GPU with 16-plane chunks are latency
    //    bound: one wave of two CTAs per SM with chunks of >= 8 planes
    //    (48^3: lz 8 0.062, 16 0.105, 48 0.277; 64^3: 8 0.062, 16 0.105,
    //    32 0.194; 96^3: 12 0.116, 16 0.146, 32 0.197);
    //  * larger lattices: aim at >= 24 CTAs per SM over the launch (about a
    //    dozen waves, so the tail wave is short) with chunks of >= 32 planes
    //    so each chunk's prologue stays a small share of its work (128^3: 32
    //    0.281, 16 0.293; 192^3: 48 0.776, 32 0.785, 16 0.816; 256^3: 32
    //    1.750, 16 1.798; 512^3: 128 13.07, 64 13.20, 256 13.45).
    const long resident = 2L * sms;
    long lz;
    if (tiles * (((long)grid[2] + 15) / 16) < resident) {
        // as many chunks as fit in one wave (rounding up would spill a few
        // CTAs into a second one)
        const long chunks = std::max(1L, resident / tiles);
        lz = ((long)grid[2] + chunks - 1) / chunks;
        if (lz < 8) lz = 8;
    } else {
        const long want = (long)sms * 24;
        long chunks = (want + tiles - 1) / tiles;
        if (chunks < 1) chunks = 1;
        lz = ((long)grid[2] + chunks - 1) / chunks;
        if (lz < 32) lz = 32;
    }
    if (lz > (long)grid[2]) lz = grid[2];
    return (int)lz;
}

int Simulation::create(const bubble_spec &spec, std::unique_ptr<Simulation> &out, std::string &err) {
    const std::string msg = validate_model(spec.model);
    if (!msg.empty()) {
        err = msg;
        return BUBBLE_ERR_INVALID;
    }
    const std::string gmsg = check_grid(spec.grid);
    if (!gmsg.empty()) {
        err = gmsg;
        return BUBBLE_ERR_INVALID;
    }
    if (spec.precision < BUBBLE_PRECISION_SINGLE || spec.precision > BUBBLE_PRECISION_PERTURBATION) {
        err = "unknown precision";
        return BUBBLE_ERR_INVALID;
    }
    if (spec.math != BUBBLE_MATH_FAST && spec.math != BUBBLE_MATH_STRICT) {
        err = "unknown math mode";
        return BUBBLE_ERR_INVALID;
    }
    if (spec.nucleation < BUBBLE_NUCLEATION_SIMULTANEOUS || spec.nucleation > BUBBLE_NUCLEATION_UNIFORM) {
        err = "unknown nucleation mode";
        return BUBBLE_ERR_INVALID;
    }
    {
        const std::string emsg = validate_eos(spec);
        if (!emsg.empty()) {
            err = emsg;
            return BUBBLE_ERR_INVALID;
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        err = "no CUDA device is available (this library has no CPU path)";
        return BUBBLE_ERR_CUDA;
    }
    std::unique_ptr<Simulation> sim(new Simulation());
    sim->spec_ = spec;
    std::memcpy(sim->grid_, spec.grid, sizeof(sim->grid_));
    sim->n_cells_ = (uint64_t)spec.grid[0] * spec.grid[1] * spec.grid[2];
    sim->tile_.ty = 16;
    sim->tile_.tx = tile_x_for(sim->tile_.ty);
    sim->tile_.lz = default_chunk(sim->grid_, sim->tile_.ty, !sim->is_f64());
    BUBBLE_CUDA(cudaStreamCreateWithFlags(&sim->stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    sim->own_stream_ = true;
    int rc = sim->allocate(err);
    if (rc != BUBBLE_OK) return rc;
    const Derived d = derive(spec.model);
    sim->schedule_ = make_schedule(spec.nucleation, spec.bubbles, d.seed_radius, spec.grid,
                                   spec.nucleation_duration, spec.seed);
    rc = sim->reset(nullptr, 0, err);
    if (rc != BUBBLE_OK) return rc;
    out = std::move(sim);
    return BUBBLE_OK;
}

Simulation::~Simulation() {
    release();
    if (h_result_) cudaFreeHost(h_result_);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

void Simulation::release() {
    release_vis();
    if (state_) cudaFree(state_);
    if (prim_) cudaFree(prim_);
    if (scratch_) cudaFree(scratch_);
    state_ = prim_ = scratch_ = nullptr;
    for (int k = 0; k < 3; ++k) field_[k] = fluid_[k] = nullptr;
    partials_ = nullptr;
    ticket_ = nullptr;
    d_result_ = nullptr;
    d_status_ = nullptr;
    tma_ok_ = false;
    device_bytes_ = 0;
}

int Simulation::allocate(std::string &err) {
    const uint64_t lattice = bubble_lattice_bytes(grid_) * (is_f64() ? 2 : 1);
    // Admission against free device memory, with the reference's 85 % rule
    // (src/gpu/vram.rs:52-69): refuse before allocating rather than risk
    // an out-of-memory failure half-way.
    size_t free_b = 0, total_b = 0;
    BUBBLE_CUDA(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    if ((double)lattice > 0.85 * (double)free_b) {
        err = "a " + std::to_string(grid_[0]) + "x" + std::to_string(grid_[1]) + "x" +
              std::to_string(grid_[2]) + " lattice needs " + std::to_string(lattice) +
              " bytes, above 85% of the " + std::to_string(free_b) + " bytes free";
        return BUBBLE_ERR_MEMORY;
    }
    const size_t fb = (size_t)n_cells_ * elem_field();
    const size_t ub = (size_t)n_cells_ * elem_fluid();
    auto round_up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t slot = round_up(fb) + round_up(ub);
    cudaError_t e = device_alloc(&state_, 3 * slot);
    if (e != cudaSuccess) {
        cudaGetLastError();
        state_ = nullptr;
        err = std::string("device allocation of the lattice failed: ") + cudaGetErrorString(e);
        return BUBBLE_ERR_MEMORY;
    }
    for (int k = 0; k < 3; ++k) {
        field_[k] = static_cast<char *>(state_) + k * slot;
        fluid_[k] = static_cast<char *>(state_) + k * slot + round_up(fb);
    }
    const size_t pb = round_up(launch::diag_partials_bytes());
    const size_t scratch = pb + 256 + round_up(sizeof(DiagResult)) + 256;
    e = device_alloc(&scratch_, scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release();
        err = std::string("device allocation of the reduction scratch failed: ") + cudaGetErrorString(e);
        return BUBBLE_ERR_MEMORY;
    }
    partials_ = scratch_;
    ticket_ = reinterpret_cast<unsigned int *>(static_cast<char *>(scratch_) + pb);
    d_result_ = reinterpret_cast<DiagResult *>(static_cast<char *>(scratch_) + pb + 256);
    d_status_ = reinterpret_cast<int *>(static_cast<char *>(scratch_) + pb + 256 + round_up(sizeof(DiagResult)));
    BUBBLE_CUDA(cudaMemsetAsync(scratch_, 0, scratch, stream_), "cudaMemset");
    tma_ok_ = true;
    for (int k = 0; k < 3; ++k)
        tma_ok_ = tma_ok_ && encode_stage_maps(&maps_[k], field_[k], fluid_[k], (int)grid_[0], (int)grid_[1],
                                               (int)grid_[2], tile_.tx, tile_.ty, is_f64() ? 8 : 4);
    if (!h_result_) BUBBLE_CUDA(cudaMallocHost(reinterpret_cast<void **>(&h_result_), sizeof(DiagResult)), "cudaMallocHost");
    device_bytes_ = 3 * slot + scratch;
    return BUBBLE_OK;
}

LatticeParams<float> lattice_params_f32(const bubble_spec &spec) {
    const SimParamsHost h = sim_params(spec.model, spec.grid);
    LatticeParams<float> p{};
    p.nx = (int)h.nx;
    p.ny = (int)h.ny;
    p.nz = (int)h.nz;
    p.dx = h.dx;
    p.inv_dx = h.inv_dx;
    p.eta = h.eta;
    p.lambda = h.lambda;
    p.phi_b = h.phi_b;
    p.m2 = h.m2;
    p.delta = h.delta;
    p.wall_width = h.wall_width;
    p.p_floor = h.p_floor;
    p.e_floor = h.e_floor;
    p.z_max = h.z_max;
    p.e_ref = h.e_ref;
    if (spec.eos == BUBBLE_EOS_GAMMA_LAW) {
        p.eos_c2 = spec.eos_param[0] - 1.0f;
        p.eos_e0 = spec.eos_param[1];
    }
    if (spec.eos == BUBBLE_EOS_THERMAL) {
        const float g = spec.eos_param[0], a = spec.eos_param[1];
        p.th_k = h.a_rad / 3.0f;
        p.th_g = g;
        p.th_h = a / 3.0f;
        p.th_a = a;
        p.th_lo = std::sqrt(3.0f * g / (4.0f * h.a_rad));
        p.th_i2a = 1.0f / (2.0f * h.a_rad);
        p.a_rad = h.a_rad;
        p.t_ref = h.t_ref;
    }
    if (spec.precision == BUBBLE_PRECISION_PERTURBATION) {
        // the stored energy is E - e_bg and the primitive pressure p - p_bg;
        // the floors move with them
        p.e_bg = h.e_ref;
        p.p_bg = h.e_ref / 3.0f;
        p.e_floor = h.e_floor - p.e_bg;
        p.p_floor = h.p_floor - p.p_bg;
    }
    return p;
}

int arith_mode(const bubble_spec &spec) {
    if (spec.eos == BUBBLE_EOS_GAMMA_LAW) return 3;
    if (spec.eos == BUBBLE_EOS_THERMAL) return 4;
    switch (spec.precision) {
        case BUBBLE_PRECISION_MIXED: return 1;
        case BUBBLE_PRECISION_PERTURBATION: return 2;
        default: return 0;
    }
}

LatticeParams<double> lattice_params_f64(const bubble_spec &spec) {
    const LatticeParams<float> f = lattice_params_f32(spec);
    LatticeParams<double> p{};
    p.nx = f.nx;
    p.ny = f.ny;
    p.nz = f.nz;
    p.dx = f.dx;
    p.inv_dx = f.inv_dx;
    p.eta = f.eta;
    p.lambda = f.lambda;
    p.phi_b = f.phi_b;
    p.m2 = f.m2;
    p.delta = f.delta;
    p.wall_width = f.wall_width;
    p.p_floor = f.p_floor;
    p.e_floor = f.e_floor;
    p.z_max = f.z_max;
    p.e_ref = f.e_ref;
    return p;
}

LatticeParams<float> Simulation::params_f32() const { return lattice_params_f32(spec_); }
LatticeParams<double> Simulation::params_f64() const { return lattice_params_f64(spec_); }
int Simulation::arith_mode() const { return bubble::arith_mode(spec_); }

int Simulation::launch_init(std::string &err) {
    cudaError_t e;
    if (is_f64())
        e = launch::init_f64((V2<double> *)field_[cur_], (V4<double> *)fluid_[cur_], n_cells_,
                             (double)params_f32().e_ref, stream_);
    else
        e = launch::init_f32((V2<float> *)field_[cur_], (V4<float> *)fluid_[cur_], n_cells_,
                             params_f32().e_ref - params_f32().e_bg, stream_);
    ++launches_;
    BUBBLE_CUDA(e, "init kernel");
    return BUBBLE_OK;
}

int Simulation::reset(const bubble_event *events, uint64_t n, std::string &err) {
    time_ = 0.0f;
    steps_ = 0;
    cur_ = 0;
    next_event_ = 0;
    if (events) schedule_.assign(events, events + n);
    return launch_init(err);
}

int Simulation::set_model(const bubble_model &m, std::string &err) {
    const std::string msg = validate_model(m);
    if (!msg.empty()) {
        err = msg;
        return BUBBLE_ERR_INVALID;
    }
    bubble_spec next = spec_;
    next.model = m;
    const std::string emsg = validate_eos(next);  // e0 is bounded by the new e_ref
    if (!emsg.empty()) {
        err = emsg;
        return BUBBLE_ERR_INVALID;
    }
    spec_.model = m;
    return BUBBLE_OK;
}

int Simulation::resize(const uint32_t grid[3], std::string &err) {
    // Validate before releasing anything (src/gpu/sim.rs:749-752).
    const std::string gmsg = check_grid(grid);
    if (!gmsg.empty()) {
        err = gmsg;
        return BUBBLE_ERR_INVALID;
    }
    // Let in-flight work finish, release, then allocate the new lattice, so
    // peak memory is max(old, new) (src/gpu/sim.rs:735-762).
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    release();
    std::memcpy(grid_, grid, sizeof(grid_));
    spec_.grid[0] = grid[0];
    spec_.grid[1] = grid[1];
    spec_.grid[2] = grid[2];
    n_cells_ = (uint64_t)grid[0] * grid[1] * grid[2];
    tile_.lz = default_chunk(grid_, tile_.ty, !is_f64());
    int rc = allocate(err);
    if (rc != BUBBLE_OK) return rc;
    const Derived d = derive(spec_.model);
    schedule_ = make_schedule(spec_.nucleation, spec_.bubbles, d.seed_radius, grid_,
                              spec_.nucleation_duration, spec_.seed);
    return reset(nullptr, 0, err);
}

int Simulation::set_tile(TileShape t, std::string &err) {
    const bool strict = !is_f64() && spec_.math == BUBBLE_MATH_STRICT;
    const bool other = spec_.precision == BUBBLE_PRECISION_PERTURBATION || spec_.eos == BUBBLE_EOS_GAMMA_LAW ||
                       spec_.eos == BUBBLE_EOS_THERMAL;
    // Compiled shapes: FP64 16 x 16 and 32 x 4; FP32 16 x 16 in every form and
    // arithmetic; 32 x 8 for the plain and MIXED forms; 32 x 4 for those in
    // the fast arithmetic.
    bool ok = t.tx == tile_x_for(t.ty) && launch::stage_shape_supported(is_f64(), t.ty) && t.lz >= 1;
    if (!is_f64() && other && t.ty != 16) ok = false;
    if (strict && t.ty == 4) ok = false;
    if (!ok) {
        err = "unsupported tile shape";
        return BUBBLE_ERR_INVALID;
    }
    if (t.ty != tile_.ty) {
        BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        tma_ok_ = true;
        for (int k = 0; k < 3; ++k)
            tma_ok_ = tma_ok_ && encode_stage_maps(&maps_[k], field_[k], fluid_[k], (int)grid_[0], (int)grid_[1],
                                                   (int)grid_[2], t.tx, t.ty, is_f64() ? 8 : 4);
    }
    t.form = tile_.form;
    tile_ = t;
    return BUBBLE_OK;
}

int Simulation::set_stage_form(int form, std::string &err) {
    if (form != BUBBLE_STAGE_FORM_AUTO && form != BUBBLE_STAGE_FORM_REGISTERS && form != BUBBLE_STAGE_FORM_SHARED) {
        err = "unknown stage form";
        return BUBBLE_ERR_INVALID;
    }
    tile_.form = form;
    return BUBBLE_OK;
}

// A stage kernel whose bounded wait expired sets bit 0 of the status word;
// it is read and cleared here after the stream has drained.
int Simulation::check_status(std::string &err) {
    int st = 0;
    BUBBLE_CUDA(cudaMemcpyAsync(&st, d_status_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "status readback");
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (st != 0) {
        BUBBLE_CUDA(cudaMemsetAsync(d_status_, 0, sizeof(int), stream_), "cudaMemset");
        err = "a stage kernel gave up waiting for its staged data (status " + std::to_string(st) + ")";
        return BUBBLE_ERR_TIMEOUT;
    }
    return BUBBLE_OK;
}

int Simulation::set_stream(cudaStream_t s, std::string &err) {
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
    if (s) {
        stream_ = s;
        own_stream_ = false;
    } else {
        BUBBLE_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        own_stream_ = true;
    }
    return BUBBLE_OK;
}

// record_nucleation (src/gpu/sim.rs:843-879): one batch of at most 1024 due
// events (time <= the current time) per call; any further due events go out
// with the next call, as in the reference.
int Simulation::record_nucleation(std::string &err) {
    V4<float> batch[BUBBLE_MAX_BATCH];
    int count = 0;
    while (next_event_ < schedule_.size() && schedule_[next_event_].time <= time_ &&
           count < (int)BUBBLE_MAX_BATCH) {
        const bubble_event &e = schedule_[next_event_];
        batch[count++] = V4<float>{e.pos[0], e.pos[1], e.pos[2], e.radius};
        ++next_event_;
    }
    if (count == 0) return BUBBLE_OK;
    cudaError_t e;
    if (is_f64())
        e = launch::nucleate_f64((V2<double> *)field_[cur_], batch, count, params_f64(), stream_);
    else
        e = launch::nucleate_f32((V2<float> *)field_[cur_], batch, count, params_f32(), stream_);
    launches_ += (count + 127) / 128;
    BUBBLE_CUDA(e, "nucleate kernel");
    nucleated_this_frame_ = true;
    return BUBBLE_OK;
}

int Simulation::stage_launch(int stage, uint32_t in_slot, uint32_t out_slot, std::string &err) {
    const uint64_t n = n_cells_;
    cudaError_t e = cudaSuccess;
    const int mode = arith_mode();
    if (mode != 0 && path_ == KernelPath::Reference) {
        err = "the MIXED and perturbation forms and the gamma-law and thermal equations of state run on the "
              "default (fused) kernel path only";
        return BUBBLE_ERR_INVALID;
    }
    if (is_f64()) {
        StageArgs<double> A;
        A.field_n = (const V2<double> *)field_[cur_];
        A.fluid_n = (const V4<double> *)fluid_[cur_];
        A.field_in = (const V2<double> *)field_[in_slot];
        A.fluid_in = (const V4<double> *)fluid_[in_slot];
        A.field_out = (V2<double> *)field_[out_slot];
        A.fluid_out = (V4<double> *)fluid_[out_slot];
        const double rk[3][2] = {{0.0, 1.0}, {0.75, 0.25}, {1.0 / 3.0, 2.0 / 3.0}};
        A.a0 = rk[stage][0];
        A.a1 = rk[stage][1];
        A.dt = (double)derive(spec_.model).dt;
        A.stage = stage;
        A.test_tx = test_tx_;
        A.wait_shift = test_tx_ ? test_shift_ : 31;
        const LatticeParams<double> P = params_f64();
        if (path_ == KernelPath::Reference) {
            e = launch::prim_f64(A.fluid_in, (V4<double> *)prim_, n, P, stream_);
            if (e == cudaSuccess) e = launch::stage_ref_f64(A, (const V4<double> *)prim_, P, stream_);
            launches_ += 2;
        } else {
            e = launch::stage_f64(A, P, tile_, maps_[in_slot], tma_ok_ ? 1 : 0, d_status_, stream_);
            launches_ += 1;
        }
    } else {
        StageArgs<float> A;
        A.field_n = (const V2<float> *)field_[cur_];
        A.fluid_n = (const V4<float> *)fluid_[cur_];
        A.field_in = (const V2<float> *)field_[in_slot];
        A.fluid_in = (const V4<float> *)fluid_[in_slot];
        A.field_out = (V2<float> *)field_[out_slot];
        A.fluid_out = (V4<float> *)fluid_[out_slot];
        A.a0 = kRK3[stage][0];
        A.a1 = kRK3[stage][1];
        A.dt = derive(spec_.model).dt;
        A.stage = stage;
        A.test_tx = test_tx_;
        A.wait_shift = test_tx_ ? test_shift_ : 31;
        const LatticeParams<float> P = params_f32();
        if (path_ == KernelPath::Reference) {
            e = launch::prim_f32(A.fluid_in, (V4<float> *)prim_, n, P, stream_);
            if (e == cudaSuccess) e = launch::stage_ref_f32(A, (const V4<float> *)prim_, P, stream_);
            launches_ += 2;
        } else {
            const int tma = tma_ok_ ? 1 : 0;
            if (spec_.math == BUBBLE_MATH_STRICT)
                e = launch::stage_f32_strict(A, P, tile_, mode, maps_[in_slot], tma, d_status_, stream_);
            else
                e = launch::stage_f32_fast(A, P, tile_, mode, maps_[in_slot], tma, d_status_, stream_);
            launches_ += 1;
        }
    }
    test_tx_ = 0;  // the test hook arms one launch
    BUBBLE_CUDA(e, "stage kernel");
    return BUBBLE_OK;
}

// record_step (src/gpu/sim.rs:881-916).
int Simulation::record_step(std::string &err) {
    if (path_ == KernelPath::Reference && !prim_) {
        cudaError_t e = device_alloc(&prim_, (size_t)n_cells_ * elem_fluid());
        if (e != cudaSuccess) {
            cudaGetLastError();
            prim_ = nullptr;
            err = std::string("device allocation of the primitive cache failed: ") + cudaGetErrorString(e);
            return BUBBLE_ERR_MEMORY;
        }
        device_bytes_ += (size_t)n_cells_ * elem_fluid();
    }
    uint32_t in[3], out[3];
    stage_slots(cur_, in, out);
    for (int s = 0; s < 3; ++s) {
        const int rc = stage_launch(s, in[s], out[s], err);
        if (rc != BUBBLE_OK) return rc;
    }
    cur_ = (cur_ + 1) % 3;
    time_ += derive(spec_.model).dt;
    ++steps_;
    return BUBBLE_OK;
}

// record_steps (src/gpu/sim.rs:827-841).
int Simulation::record_steps(uint32_t n, std::string &err) {
    nucleated_this_frame_ = false;
    int rc = record_nucleation(err);
    if (rc != BUBBLE_OK) return rc;
    for (uint32_t k = 0; k < n; ++k) {
        rc = record_step(err);
        if (rc != BUBBLE_OK) return rc;
    }
    return BUBBLE_OK;
}

// headless::advance's loop (src/headless.rs:126-131).
int Simulation::advance(uint64_t n, std::string &err) {
    for (uint64_t k = 0; k < n; ++k) {
        const int rc = record_steps(1, err);
        if (rc != BUBBLE_OK) return rc;
    }
    return BUBBLE_OK;
}

int Simulation::diagnostics(bubble_diag *out, std::string &err) {
    cudaError_t e;
    if (is_f64()) {
        e = launch::diag_f64((const V2<double> *)field_[cur_], (const V4<double> *)fluid_[cur_],
                             params_f64(), partials_, ticket_, d_result_, stream_);
    } else {
        e = launch::diag_f32((const V2<float> *)field_[cur_], (const V4<float> *)fluid_[cur_],
                             params_f32(), arith_mode(), partials_,
                             ticket_, d_result_, stream_);
    }
    ++launches_;
    BUBBLE_CUDA(e, "diagnostics kernel");
    BUBBLE_CUDA(cudaMemcpyAsync(h_result_, d_result_, sizeof(DiagResult), cudaMemcpyDeviceToHost, stream_),
                "diagnostics readback");
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    {
        const int rc = check_status(err);
        if (rc != BUBBLE_OK) return rc;
    }
    DiagResult r = *h_result_;
    if (spec_.precision == BUBBLE_PRECISION_PERTURBATION) {
        // the kernel summed E - e_bg: add the background in FP64
        const double bg = (double)params_f32().e_bg * (double)n_cells_;
        r.sums[0] += bg;
        r.sums[3] += bg;
    }
    // Diagnostics (src/gpu/sim.rs:991-1010): sums / cells.
    const float inv_n = 1.0f / (float)n_cells_;
    bubble_diag d{};
    d.sum_energy = r.sums[0];
    d.sum_broken = r.sums[1];
    d.sum_kinetic = r.sums[2];
    d.sum_fluid_energy = r.sums[3];
    d.mean_energy = (float)r.sums[0] * inv_n;
    d.broken_fraction = (float)r.sums[1] * inv_n;
    d.mean_kinetic = (float)r.sums[2] * inv_n;
    d.mean_fluid_energy = (float)r.sums[3] * inv_n;
    float vmaxv;
    std::memcpy(&vmaxv, &r.max_v_bits, sizeof(vmaxv));
    d.max_velocity = vmaxv;
    d.kinetic_fraction = std::fabs(d.mean_energy) < 1e-20f ? 0.0f : d.mean_kinetic / d.mean_energy;
    d.mean_energy_f64 = r.sums[0] / (double)n_cells_;
    d.mean_kinetic_f64 = r.sums[2] / (double)n_cells_;
    d.cells = n_cells_;
    *out = d;
    if (r.nonfinite || !std::isfinite(d.mean_energy) || !std::isfinite(d.max_velocity)) {
        err = "the solution blew up at step " + std::to_string(steps_) +
              " (non-finite diagnostics); reduce --cfl or --alpha";
        return BUBBLE_ERR_NONFINITE;
    }
    return BUBBLE_OK;
}

int Simulation::nucleate_now(uint64_t rng_seed, std::string &err) {
    (void)err;
    Pcg64Mcg rng = Pcg64Mcg::seed_from_u64(rng_seed);
    bubble_event e;
    e.time = time_;
    e.pos[0] = rng.next_f32() * (float)grid_[0];
    e.pos[1] = rng.next_f32() * (float)grid_[1];
    e.pos[2] = rng.next_f32() * (float)grid_[2];
    e.radius = derive(spec_.model).seed_radius;
    schedule_.insert(schedule_.begin() + (std::ptrdiff_t)next_event_, e);
    return BUBBLE_OK;
}

int Simulation::synchronize(std::string &err) {
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    {
        const int rc = check_status(err);
        if (rc != BUBBLE_OK) return rc;
    }
    return BUBBLE_OK;
}

int Simulation::copy_state(void *field, void *fluid, bool f64, std::string &err) {
    if (f64 != is_f64()) {
        err = f64 ? "the simulation holds FP32 state" : "the simulation holds FP64 state";
        return BUBBLE_ERR_INVALID;
    }
    if (field)
        BUBBLE_CUDA(cudaMemcpyAsync(field, field_[cur_], n_cells_ * elem_field(), cudaMemcpyDeviceToHost, stream_),
                    "state readback");
    if (fluid)
        BUBBLE_CUDA(cudaMemcpyAsync(fluid, fluid_[cur_], n_cells_ * elem_fluid(), cudaMemcpyDeviceToHost, stream_),
                    "state readback");
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return BUBBLE_OK;
}

int Simulation::load_state(const void *field, const void *fluid, bool f64, std::string &err) {
    if (f64 != is_f64()) {
        err = f64 ? "the simulation holds FP32 state" : "the simulation holds FP64 state";
        return BUBBLE_ERR_INVALID;
    }
    if (field)
        BUBBLE_CUDA(cudaMemcpyAsync(field_[cur_], field, n_cells_ * elem_field(), cudaMemcpyHostToDevice, stream_),
                    "state upload");
    if (fluid)
        BUBBLE_CUDA(cudaMemcpyAsync(fluid_[cur_], fluid, n_cells_ * elem_fluid(), cudaMemcpyHostToDevice, stream_),
                    "state upload");
    BUBBLE_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return BUBBLE_OK;
}

void Simulation::device_state(void **field, void **fluid) const {
    if (field) *field = field_[cur_];
    if (fluid) *fluid = fluid_[cur_];
}

}  // namespace bubble
