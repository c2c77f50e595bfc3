// Batched form: many independent lattices advanced together.
//
// Each lattice is a Simulation's worth of state (three RK slots, schedule,
// f32 time, slot rotation; src/gpu/sim.rs:180-1026) but stepping runs
// through one persistent cooperative launch for the whole batch
// (batch.cuh), captured in a CUDA graph and replayed.  Nucleation events are
// stamped between launches: a launch covers as many steps as every lattice
// can take before its next event is due, so each lattice sees its events
// before the same step as the plain per-lattice path.
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
    static int create(const bubble_spec *specs, uint32_t n, const bubble_batch_options *opt,
                      std::unique_ptr<Batch> &out, std::string &err);
    ~Batch();

    int advance(uint64_t steps, std::string &err);
    int diagnostics(uint32_t k, bubble_diag *out, std::string &err);
    int copy_state(uint32_t k, float *field, float *fluid, std::string &err);
    int load_state(uint32_t k, const float *field, const float *fluid, std::string &err);
    void info(bubble_batch_info *out) const;
    uint32_t size() const { return (uint32_t)lats_.size(); }
    float time(uint32_t k) const { return lats_[k].time; }
    uint64_t steps(uint32_t k) const { return lats_[k].steps; }
    uint64_t remaining_bubbles(uint32_t k) const {
        const auto &L = lats_[k];
        return L.schedule.size() > L.next_event ? L.schedule.size() - L.next_event : 0;
    }

   private:
    struct Lat {
        bubble_spec spec{};
        uint32_t grid[3] = {0, 0, 0};
        uint64_t cells = 0;
        void *state = nullptr;
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
        std::vector<bubble_event> schedule;
        size_t next_event = 0;
    };
    Batch() = default;
    int allocate(Lat &L, std::string &err);
    int nucleate_due(Lat &L, std::string &err);
    uint64_t steps_until_event(const Lat &L, uint64_t cap) const;
    int launch_chunk(uint64_t k, std::string &err);
    int autotune(std::string &err);
    void plan_items();
    int check_status(std::string &err);

    std::vector<Lat> lats_;      // user order
    std::vector<uint32_t> item_order_;  // lattices by decreasing size
    bool fast_ = true;
    int ty_ = 8;
    int grid_ = 0;
    int max_grid_ = 0;
    int n_items_ = 0;
    bool use_graph_ = true;
    bool graph_ok_ = false;
    uint64_t graph_steps_ = 0;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    BatchLattice *d_lat_ = nullptr;
    BatchLattice *h_lat_ = nullptr;  // pinned
    unsigned int *d_counters_ = nullptr;
    int *d_status_ = nullptr;
    void *d_scratch_ = nullptr;  // diag partials | ticket | result
    DiagResult *h_result_ = nullptr;
    cudaStream_t stream_ = nullptr;
    uint64_t launches_ = 0;
    uint64_t device_bytes_ = 0;
    bool autotuned_ = false;
};

// Fastest z chunk of the fused stage kernel for a lattice size, measured on
// the device (cached per size, tile height and arithmetic mode).
int autotune_chunk(const uint32_t grid[3], int ty, bool fast, std::string &err);

}  // namespace bubble
