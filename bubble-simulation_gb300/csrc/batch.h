// Batched form: many independent lattices advanced together.
//
// Each lattice is a Simulation's worth of state (three RK slots, schedule,
// f32 time, slot rotation; src/gpu/sim.rs:180-1026) but stepping runs
// through one persistent cooperative launch for every active lattice
// (batch.cuh), captured in a CUDA graph and replayed.  Nucleation events are
// stamped between launches: a launch covers as many steps as every lattice
// can take before its next event is due, so each lattice sees its events
// before the same step as the plain per-lattice path.  Lattices can join
// and leave between launches (the serving loop's continuous batching);
// their indices stay stable.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/bubble.h"
#include "../../include/bubble_batch.h"
#include "batch_desc.h"
#include "params.h"
#include "physics.h"
#include "tma.h"

namespace bubble {

class Batch {
   public:
    // A batch of the given lattices (all FP32, one math mode).
    static int create(const bubble_spec *specs, uint32_t n, const bubble_batch_options *opt,
                      std::unique_ptr<Batch> &out, std::string &err);
    // An empty batch that lattices join later with add().
    static int create_empty(int math, const bubble_batch_options *opt, std::unique_ptr<Batch> &out,
                            std::string &err);
    ~Batch();

    // Adds a lattice (allocated and initialised; admission is the caller's).
    int add(const bubble_spec &spec, uint32_t *index, std::string &err);
    // Releases a lattice's device memory; its index is not reused.
    int remove(uint32_t k, std::string &err);

    // Advances every active lattice by `steps`.
    int advance(uint64_t steps, std::string &err);
    int diagnostics(uint32_t k, bubble_diag *out, std::string &err);
    int copy_state(uint32_t k, float *field, float *fluid, std::string &err);
    int load_state(uint32_t k, const float *field, const float *fluid, std::string &err);
    void info(bubble_batch_info *out) const;
    uint32_t size() const { return (uint32_t)lats_.size(); }
    uint32_t active_count() const;
    bool active(uint32_t k) const { return k < lats_.size() && lats_[k].state != nullptr; }
    float time(uint32_t k) const { return lats_[k].time; }
    uint64_t steps(uint32_t k) const { return lats_[k].steps; }
    cudaStream_t stream() const { return stream_; }

   private:
    struct Lat {
        bubble_spec spec{};
        uint32_t grid[3] = {0, 0, 0};
        uint64_t cells = 0;
        void *state = nullptr;  // null once removed
        void *field[3] = {nullptr, nullptr, nullptr};
        void *fluid[3] = {nullptr, nullptr, nullptr};
        StageMaps maps[3];
        bool tma_ok = false;
        LatticeParams<float> P{};
        float dt = 0.0f;
        float time = 0.0f;
        uint64_t steps = 0;
        uint32_t cur = 0;
        int lz = 16;
        // A lattice that fills the GPU by itself (two CTAs per SM with
        // 32-plane chunks) gains nothing from the shared launch: it runs
        // through the plain stage kernel with the plain path's chunk.
        bool solo = false;
        uint64_t bytes = 0;
        std::vector<bubble_event> schedule;
        size_t next_event = 0;
    };
    Batch() = default;
    int setup(int math, const bubble_batch_options *opt, std::string &err);
    int allocate(Lat &L, std::string &err);
    int nucleate_due(Lat &L, std::string &err);
    uint64_t steps_until_event(const Lat &L, uint64_t cap) const;
    int launch_chunk(uint64_t k, std::string &err);
    int launch_solo(Lat &L, uint64_t k, std::string &err);
    int autotune(std::string &err);
    void plan_items();
    int ensure_capacity(size_t n, std::string &err);
    int check_status(std::string &err);

   public:
    // z planes per work item of lattices that join later (0: 64).  A batch
    // with a chunk cap re-chunks on every membership change: among the cap
    // and shorter caps (48 .. 4 planes) it takes the one with the least cost
    // per round (the item-planes spread over the persistent grid plus the
    // longest item), so a round of a few lattices still spreads over the
    // GPU and a full one is not cut finer than it pays.
    void set_chunk_planes(int planes) {
        lz_cap_ = planes > 0 ? planes : 64;
        fill_ = true;
    }
    // Test hook: the next persistent launch runs its grid barrier with a
    // release count no arrival reaches and a 2^shift-cycle wait limit, so
    // every CTA's barrier wait expires and sets bit 1 of the status word.
    void arm_barrier_expiry(int shift) { test_barrier_shift_ = shift; }

   private:
    int test_barrier_shift_ = 0;  // 0: off

    std::vector<Lat> lats_;
    std::vector<uint32_t> item_order_;  // active lattices by decreasing size
    int math_ = BUBBLE_MATH_FAST;
    bool fast_ = true;
    int ty_ = 8;
    int lz_cap_ = 64;  // z chunk of lattices that join later
    bool fill_ = false;  // re-chunk under lz_cap_ to fill the grid
    int grid_ = 0;
    int max_grid_ = 0;
    int n_items_ = 0;
    bool use_graph_ = true;
    bool graph_ok_ = false;
    std::tuple<uint64_t, int, int, int> graph_key_{0, 0, 0, 0};  // steps, lattices, items, grid
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    size_t capacity_ = 0;            // descriptors the buffers hold
    BatchLattice *d_lat_ = nullptr;
    BatchLattice *h_lat_ = nullptr;  // pinned
    unsigned int *d_counters_ = nullptr;
    int *d_status_ = nullptr;
    void *d_scratch_ = nullptr;  // counters | status | diag partials | ticket | result
    DiagResult *h_result_ = nullptr;
    cudaStream_t stream_ = nullptr;
    uint64_t launches_ = 0;
    uint64_t device_bytes_ = 0;
    bool autotuned_ = false;
    bool dirty_ = true;  // membership changed since the last plan_items()
};

// Fastest z chunk of the fused stage kernel for one lattice size, measured
// on the device (cached per size, tile height and arithmetic mode).
int autotune_chunk(const uint32_t grid[3], int ty, bool fast, std::string &err);

}  // namespace bubble
