/*
 * bubble_server.h -- serving form: a request loop with continuous batching.
 * No counterpart in the reference, whose host advances one Simulation at a
 * time; each request here is one such simulation (a bubble_spec and a step
 * count), run with the semantics of headless::advance (src/headless.rs:
 * 120-150) and answered with its final diagnostics.
 *
 * Requests queue in arrival order.  A scheduling round (bubble_server_tick)
 * admits queued requests while their lattice fits in the configured
 * fraction of free device memory (the reference's VRAM clamp,
 * src/gpu/vram.rs:52-69) and the resident count allows, advances every
 * resident lattice by one chunk of steps in one persistent batched launch,
 * and retires the lattices that finished.  Requests that arrive while
 * others run join at the next round, so their work overlaps on the device.
 */
#ifndef BUBBLE_GB300_SERVER_H
#define BUBBLE_GB300_SERVER_H

#include <stdint.h>

#include "bubble.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bubble_server bubble_server;

typedef struct bubble_server_options {
    int32_t math;            /* BUBBLE_MATH_* of every request (default FAST)   */
    int32_t tile_y;          /* 16 (16 x 16 tiles, default) or 8 (fast only)     */
    uint32_t chunk_steps;    /* steps per scheduling round (default 50)         */
    uint32_t max_active;     /* resident lattices at most (default 64)          */
    float memory_fraction;   /* share of free device memory a new lattice may
                                take (default 0.85)                              */
    int32_t use_graph;       /* capture the batched launch in a CUDA graph      */
    uint64_t resident_cells; /* admit while the resident lattices hold fewer
                                cells than this (0: 24 M cells, about what keeps
                                every SM busy); a request larger than the budget
                                runs alone                                       */
    int32_t policy;          /* BUBBLE_SERVE_FIFO (default): arrival order, a
                                request that does not fit lets smaller later ones
                                backfill; BUBBLE_SERVE_SHORTEST: least work
                                (cells x steps) first                            */
    uint32_t chunk_planes;   /* z planes per work item of a lattice (0: 64);
                                columns are cut into equal chunks no longer
                                than this or a shorter cap (48 .. 4 planes)
                                that a cost model of the round rates cheaper
                                for the active lattices                          */
} bubble_server_options;

#define BUBBLE_SERVE_FIFO 0
#define BUBBLE_SERVE_SHORTEST 1

typedef struct bubble_server_result {
    uint64_t id;
    int32_t status;          /* BUBBLE_OK or the error of this request          */
    uint32_t grid[3];
    uint64_t steps;
    double submit_s;         /* seconds since the server started                */
    double admit_s;
    double done_s;
    bubble_diag diag;        /* diagnostics of the final state                  */
} bubble_server_result;

typedef struct bubble_server_stats {
    uint64_t submitted, admitted, completed, queued, active, rounds;
    double p50_latency_s, p99_latency_s, mean_latency_s;
    double solves_per_s;     /* completed / (last completion - first submission) */
    double cell_updates;     /* over completed requests                          */
} bubble_server_stats;

void bubble_server_options_default(bubble_server_options *out);
int bubble_server_create(const bubble_server_options *opt, bubble_server **out);
void bubble_server_destroy(bubble_server *server);
/* Queue a request: `spec` (precision SINGLE, the server's math mode) run for
 * `steps` steps.  Rejects invalid specs at once. */
int bubble_server_submit(bubble_server *server, const bubble_spec *spec, uint64_t steps, uint64_t *id);
/* One scheduling round.  *busy = 1 while requests are queued or resident. */
int bubble_server_tick(bubble_server *server, int32_t *busy);
int bubble_server_run_until_idle(bubble_server *server);
/* Completed results not yet returned, oldest first. */
int bubble_server_poll(bubble_server *server, bubble_server_result *out, uint64_t capacity, uint64_t *n_out);
int bubble_server_stats_get(const bubble_server *server, bubble_server_stats *out);
/* Seconds since the server started (the clock of submit_s / done_s). */
double bubble_server_now(const bubble_server *server);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_GB300_SERVER_H */
