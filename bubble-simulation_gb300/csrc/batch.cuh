// Batched form: many independent lattices of uneven size advanced by one
// persistent, cooperative launch.
//
// The launch runs `steps` SSP-RK3 steps of every lattice in the batch.  Each
// RK stage is a list of work items -- (lattice, column tile, z chunk), the
// unit of the fused stage kernel -- handed out dynamically from one atomic
// counter, largest lattices first; a grid-wide barrier separates the stages
// because a stage reads its neighbours' outputs of the previous one.  Every
// lattice keeps its own slot rotation (src/gpu/sim.rs:1046-1051).  The grid
// barrier's wait is bounded; on expiry bit 1 of *status is set and the CTA
// leaves, so the others expire in turn at their next barrier.
#pragma once

#include "batch_desc.h"
#include "stage_column.cuh"

namespace bubble {
namespace dev {

// Bounded grid barrier for a cooperative launch: the last of gridDim.x +
// `extra` arrivals releases it (extra is 0 except in the test hook
// bubble_ext_test_expire_batch_barrier, where no arrival is the last); a CTA
// waits at most 2^shift SM cycles.  Returns false on expiry.
BUBBLE_DEV bool grid_barrier(unsigned int *count, unsigned int *gen, int *status, unsigned int extra, int shift) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = gen;
        const unsigned int g = *vgen;
        // The next stage reads this stage's stores through TMA (the async
        // proxy): order generic-proxy writes before async-proxy reads.
        asm volatile("fence.proxy.async.global;" ::: "memory");
        __threadfence();
        const unsigned int arrived = atomicAdd(count, 1u) + 1u;
        int ok = 1;
        if (arrived == gridDim.x + extra) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == g) {
                if (clock64() - t0 > (1ll << shift)) {
                    ok = 0;
                    atomicOr(status, 2);
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        asm volatile("fence.proxy.async.global;" ::: "memory");
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// The batch's items run the shared form of the column kernel with 16 x 16
// tiles (three CTAs per SM: 43.6 against 42.1 solves/s on the 64-lattice
// mixed-size batch), the register form with 32 x 8 tiles.
template <int TY>
constexpr bool kBatchShared = TY == 16;

// sync: counters[0] = barrier count, counters[1] = barrier generation,
//       counters[2] = work counter (zeroed before the launch).
template <bool FAST, int TY>
__global__ void __launch_bounds__(ColumnLayout<float, TY, kBatchShared<TY>>::NT,
                                  ColumnLayout<float, TY, kBatchShared<TY>>::MIN_BLOCKS)
    batch_kernel(const BatchLattice *__restrict__ lat, int n_lat, int n_items, int steps,
                    unsigned int *counters, int *status, unsigned int barrier_extra, int barrier_shift) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int item_s;
    // the current item's stage arguments and lattice constants, read from
    // shared memory by the item body instead of held in registers
    __shared__ StageArgs<float> A_s;
    __shared__ LatticeParams<float> P_s;
    unsigned int round = 0;
    // Every CTA ends a round with one grab past the last item, so a round
    // consumes exactly n_items + gridDim.x grabs of the counter.
    const unsigned int per_round = (unsigned int)n_items + gridDim.x;
    for (int step = 0; step < steps; ++step) {
        for (int stage = 0; stage < 3; ++stage, ++round) {
            const unsigned int base = round * per_round;
            while (true) {
                __syncthreads();
                if (threadIdx.x == 0) item_s = (int)(atomicAdd(&counters[2], 1u) - base);
                __syncthreads();
                const int item = item_s;
                if (item >= n_items) break;
                // lattice of this item: largest item_begin <= item
                int lo = 0, hi = n_lat - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (lat[mid].item_begin <= item) lo = mid;
                    else hi = mid - 1;
                }
                const BatchLattice &B = lat[lo];
                const int local = item - B.item_begin;
                const int cur = (B.cur0 + step) % 3;
                const int a = cur, b = (cur + 1) % 3, c = (cur + 2) % 3;
                const int in_slot = stage == 0 ? a : (stage == 1 ? b : c);
                const int out_slot = stage == 1 ? c : b;
                // Thread 0 publishes the item's arguments: every thread has
                // left the previous item (the barriers above), and
                // column_item's opening barrier makes them visible.
                if (threadIdx.x == 0) {
                    StageArgs<float> A;
                    A.field_n = B.field[a];
                    A.fluid_n = B.fluid[a];
                    A.field_in = B.field[in_slot];
                    A.fluid_in = B.fluid[in_slot];
                    A.field_out = B.field[out_slot];
                    A.fluid_out = B.fluid[out_slot];
                    // the RK3 table (src/gpu/sim.rs:133-135) as selects, not an indexed array
                    A.a0 = stage == 0 ? 0.0f : (stage == 1 ? 0.75f : 1.0f / 3.0f);
                    A.a1 = stage == 0 ? 1.0f : (stage == 1 ? 0.25f : 2.0f / 3.0f);
                    A.dt = B.dt;
                    A.stage = stage;
                    A_s = A;
                    P_s = B.P;
                }
                if (!column_item<float, FAST, kPlain, TY, kBatchShared<TY>>(smem, A_s, P_s, B.lz, &B.maps[in_slot], B.tma_ok, status,
                                                      local % B.tiles_xy, local / B.tiles_xy)) {
                    // record where the stage's bounded wait gave up (status[8..12])
                    if (threadIdx.x == 0 && atomicCAS(&status[8], 0, 1) == 0) {
                        status[9] = item;
                        status[10] = lo;
                        status[11] = (int)round;
                        status[12] = local;
                    }
                    return;
                }
            }
            if (!grid_barrier(&counters[0], &counters[1], status, barrier_extra, barrier_shift)) return;
        }
    }
}

}  // namespace dev
}  // namespace bubble
