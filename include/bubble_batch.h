/*
 * bubble_batch.h -- batched form of the lattice time step: many independent
 * lattices of uneven size advanced together by one persistent, CUDA-graph
 * captured launch per chunk of steps.  No counterpart in the reference,
 * which advances one Simulation at a time (src/gpu/sim.rs:180-1026); each
 * lattice here follows that Simulation's semantics (schedule, f32 time, slot
 * rotation, nucleation before each step as in src/headless.rs:126-131).
 */
#ifndef BUBBLE_GB300_BATCH_H
#define BUBBLE_GB300_BATCH_H

#include <stdint.h>

#include "bubble.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bubble_batch bubble_batch;

typedef struct bubble_batch_options {
    int32_t tile_y;     /* 16 (16 x 16 tiles, default) or 8 (32 x 8, fast only) */
    int32_t autotune;   /* 1: time candidate z chunks per lattice size        */
    int32_t use_graph;  /* 1: capture the launch in a CUDA graph and replay   */
    int32_t max_grid;   /* 0: every co-resident CTA; else cap on the CTAs     */
} bubble_batch_options;

typedef struct bubble_batch_info {
    uint32_t lattices;
    uint32_t grid;        /* persistent CTAs                                    */
    uint32_t items;       /* work items per RK stage                            */
    int32_t tile_y;
    int32_t graph;        /* 1 when launches replay a captured CUDA graph       */
    int32_t autotuned;
    uint64_t cells;       /* total over the batch                               */
    uint64_t launches;    /* kernel launches so far (nucleation + persistent)   */
    uint64_t device_bytes;
} bubble_batch_info;

void bubble_batch_options_default(bubble_batch_options *out);
/* All specs must share precision SINGLE and one math mode.  Lattices keep
 * the order of `specs`. */
int bubble_batch_create(const bubble_spec *specs, uint32_t n, const bubble_batch_options *opt,
                        bubble_batch **out);
void bubble_batch_destroy(bubble_batch *batch);
/* Advance every lattice by n_steps (each step checks its due events first). */
int bubble_batch_advance(bubble_batch *batch, uint64_t n_steps);
int bubble_batch_diagnostics(bubble_batch *batch, uint32_t index, bubble_diag *out);
int bubble_batch_copy_state(bubble_batch *batch, uint32_t index, float *field, float *fluid);
int bubble_batch_load_state(bubble_batch *batch, uint32_t index, const float *field, const float *fluid);
int bubble_batch_info_get(const bubble_batch *batch, bubble_batch_info *out);
float bubble_batch_time(const bubble_batch *batch, uint32_t index);

/* Test hook of the persistent launch's bounded grid barrier: the next
 * launch of `batch` runs its barrier with a release count one above the
 * grid, so no arrival releases it, and a wait limit of 2^wait_shift SM
 * cycles (10..32); every CTA's wait expires, sets the status word and
 * returns, and the next bubble_batch_diagnostics reports BUBBLE_ERR_TIMEOUT.  Lattices that run solo (fill the GPU alone) do not use
 * the persistent launch. */
int bubble_ext_test_expire_batch_barrier(bubble_batch *batch, int32_t wait_shift);

/* Fastest z chunk of the fused stage kernel for a lattice size (autotuner,
 * cached per process). */
int bubble_autotune_chunk(const uint32_t grid[3], int32_t tile_y, int32_t math, int32_t *lz_out);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_GB300_BATCH_H */
