// The simulation driver: device state, slot rotation, nucleation batching,
// stage launches and the diagnostics readback.
//
// Restates the host side of `Simulation` (src/gpu/sim.rs:180-1026) for CUDA:
// three RK slots of (field, fluid), `cur` rotating through `stage_slots`, the
// schedule consumed by `time <= sim.time` in batches, f32 time accumulation,
// and a synchronous FP64 diagnostics reduction.  There is no primitive cache
// (primitives are recovered inside the stage kernel) and no visualisation
// texture, so a lattice holds 72 B per cell in FP32.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bubble.h"
#include "../../include/bubble_render.h"
#include "params.h"
#include "physics.h"
#include "tma.h"

namespace bubble {

// Which stage kernels to run.
enum class KernelPath : int {
    Fused = 0,      // one fused launch per RK stage with async staging (default)
    Reference = 1,  // primitives pass + stage pass per RK stage, as in the reference
};

class Simulation {
   public:
    // Simulation::new.  Returns BUBBLE_OK or an error code with `err` set.
    static int create(const bubble_spec &spec, std::unique_ptr<Simulation> &out, std::string &err);
    ~Simulation();

    int reset(const bubble_event *events, uint64_t n, std::string &err);
    int set_model(const bubble_model &m, std::string &err);
    int resize(const uint32_t grid[3], std::string &err);
    int record_steps(uint32_t n, std::string &err);
    int advance(uint64_t n, std::string &err);
    int diagnostics(bubble_diag *out, std::string &err);
    int nucleate_now(uint64_t rng_seed, std::string &err);
    int synchronize(std::string &err);
    int set_stream(cudaStream_t s, std::string &err);

    int copy_state(void *field, void *fluid, bool f64, std::string &err);
    int load_state(const void *field, const void *fluid, bool f64, std::string &err);
    // Device pointers of the current slot (for zero-copy inspection).
    void device_state(void **field, void **fluid) const;

    void set_path(KernelPath p) { path_ = p; }
    // Test hook: the next stage launch arms, in every CTA that stages planes
    // through TMA, its first plane's mbarrier for `tx` bytes with no copy
    // issued, and bounds the stage kernel's waits by 2^shift SM cycles, so
    // those waits expire and the next check reports BUBBLE_ERR_TIMEOUT.
    void arm_wait_expiry(uint32_t tx, int shift) {
        test_tx_ = tx;
        test_shift_ = shift;
    }
    KernelPath path() const { return path_; }
    int set_tile(TileShape t, std::string &err);  // keeps the stage form
    // BUBBLE_STAGE_FORM_* of FP32 16 x 16 launches
    int set_stage_form(int form, std::string &err);
    TileShape tile() const { return tile_; }

    float time() const { return time_; }
    uint64_t steps() const { return steps_; }
    uint64_t cell_count() const { return n_cells_; }
    uint64_t remaining_bubbles() const {
        return schedule_.size() > next_event_ ? schedule_.size() - next_event_ : 0;
    }
    uint64_t device_memory_bytes() const { return device_bytes_; }
    const uint32_t *grid() const { return grid_; }
    const bubble_model &model() const { return spec_.model; }
    const bubble_spec &spec() const { return spec_; }
    const std::vector<bubble_event> &schedule() const { return schedule_; }
    bool nucleated_this_frame() const { return nucleated_this_frame_; }
    cudaStream_t stream() const { return stream_; }
    uint32_t current_slot() const { return cur_; }
    // Kernel launches issued since creation (init, nucleate, stage, diag).
    uint64_t launches() const { return launches_; }

    // Checkpoint and resume (checkpoint.cpp): the current slot's state, the
    // schedule and the clock, written to a file; `restore` reloads one into
    // this simulation (resizing it if the grid differs).
    int save_checkpoint(const std::string &path, std::string &err);
    int restore_checkpoint(const std::string &path, std::string &err);
    // Reads the spec stored in a checkpoint file without creating anything.
    static int checkpoint_spec(const std::string &path, bubble_spec &spec, std::string &err);

    // Visualisation (render_host.cpp): record_visualisation
    // (src/gpu/sim.rs:918-942) into a half4 CUDA array allocated on first
    // use, its readback, and one frame of the volume renderer.
    int visualise(std::string &err);
    int vis_copy(uint16_t *host_rgba16, std::string &err);
    int render(const bubble_view &view, uint32_t width, uint32_t height, uint8_t *host_rgba8,
               std::string &err);

   private:
    Simulation() = default;
    int allocate(std::string &err);
    void release();
    int launch_init(std::string &err);
    int record_nucleation(std::string &err);
    int record_step(std::string &err);
    int stage_launch(int stage, uint32_t in_slot, uint32_t out_slot, std::string &err);
    LatticeParams<float> params_f32() const;
    LatticeParams<double> params_f64() const;
    bool is_f64() const { return spec_.precision == BUBBLE_PRECISION_DOUBLE; }
    // 0 plain, 1 mixed, 2 perturbation form (the kernels' MODE parameter)
    int arith_mode() const;
    size_t elem_field() const { return is_f64() ? 16 : 8; }
    size_t elem_fluid() const { return is_f64() ? 32 : 16; }

    bubble_spec spec_{};
    uint32_t grid_[3] = {0, 0, 0};
    uint64_t n_cells_ = 0;
    float time_ = 0.0f;
    uint64_t steps_ = 0;
    uint32_t cur_ = 0;
    std::vector<bubble_event> schedule_;
    size_t next_event_ = 0;
    bool nucleated_this_frame_ = false;
    KernelPath path_ = KernelPath::Fused;
    uint32_t test_tx_ = 0;  // 0: the wait-expiry test hook is off
    int test_shift_ = 31;
    TileShape tile_{32, 8, 64};

    // device memory
    void *state_ = nullptr;     // 3 slots x (field, fluid)
    void *field_[3] = {nullptr, nullptr, nullptr};
    void *fluid_[3] = {nullptr, nullptr, nullptr};
    void *prim_ = nullptr;      // reference path only
    void *scratch_ = nullptr;   // diag partials | ticket | result | status
    void *partials_ = nullptr;
    unsigned int *ticket_ = nullptr;
    DiagResult *d_result_ = nullptr;
    int *d_status_ = nullptr;   // bit 0: a bounded wait in a stage kernel expired
    DiagResult *h_result_ = nullptr;  // pinned
    uint64_t device_bytes_ = 0;
    StageMaps maps_[3];         // TMA maps of each slot as a stage input
    bool tma_ok_ = false;
    int check_status(std::string &err);

    // visualisation texture (render_host.cpp); released with the lattice
    void release_vis();
    cudaArray_t vis_array_ = nullptr;
    cudaSurfaceObject_t vis_surf_ = 0;
    cudaTextureObject_t vis_tex_ = 0;
    uint64_t vis_bytes_ = 0;
    void *image_ = nullptr;  // device RGBA8 frame
    size_t image_bytes_ = 0;

    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;
    uint64_t launches_ = 0;
};

// Kernel constants of a lattice described by `spec` (its grid, model,
// precision form and equation of state), and the FORM parameter of the
// kernels (physics.cuh kPlain, kMixed, kPert, kGamma, kThermal).
LatticeParams<float> lattice_params_f32(const bubble_spec &spec);
LatticeParams<double> lattice_params_f64(const bubble_spec &spec);
int arith_mode(const bubble_spec &spec);

// Default z chunk of the fused kernel for a lattice.  FP32 16 x 16 tiles:
// the chunk whose cheaper form is cheapest under column_stage_cost (params.h);
// otherwise enough CTAs to fill the GPU while keeping each chunk's warm-up a
// small fraction of its work.
int default_chunk(const uint32_t grid[3], int ty, bool fp32);

// Test hook: make the next device allocation of this process fail.
void inject_allocation_failure();

}  // namespace bubble
