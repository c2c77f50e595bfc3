/*
 * bubble_ext.h -- entry points of the GB300 library that have no
 * counterpart in the reference: kernel-path and tile selection (for the
 * cross-checks and the tile autotuner), device pointers of the current slot,
 * the stream, launch counts and a host-side fault-injection hook.
 */
#ifndef BUBBLE_GB300_EXT_H
#define BUBBLE_GB300_EXT_H

#include <stdint.h>

#include "bubble.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel path of the RK stages. */
#define BUBBLE_PATH_FUSED 0     /* one fused launch per stage (default)       */
#define BUBBLE_PATH_REFERENCE 1 /* primitives pass + stage pass per stage,
                                   the reference's own kernel structure (bag
                                   model, SINGLE and DOUBLE only)            */
int bubble_ext_set_path(bubble_sim *sim, int32_t path);

/* Tile of the fused kernel: y extent, which fixes the x extent (FP32: 16
 * for 16 x 16 tiles, the default, in every form; 8 for 32 x 8 in the plain
 * and MIXED forms; 4 for 32 x 4 in those forms with the fast arithmetic;
 * FP64: 16 (default) or 4 for 32 x 4) and z chunk (planes marched per CTA). */
int bubble_ext_set_tile(bubble_sim *sim, int32_t ty, int32_t lz);
int bubble_ext_get_tile(const bubble_sim *sim, int32_t *ty, int32_t *lz);

/* Form of the fused kernel for FP32 16 x 16 tiles; both forms give
 * identical bits.  REGISTERS keeps each column's z pipeline in registers
 * (two CTAs per SM); SHARED reads it back from shared memory (three CTAs
 * per SM, faster once a launch fills more than one wave); AUTO (default)
 * takes the form a cost model of the launch rates cheaper for the lattice
 * and chunk (the model also picks the default chunk).  Other tiles and FP64
 * always use REGISTERS. */
#define BUBBLE_STAGE_FORM_AUTO 0
#define BUBBLE_STAGE_FORM_REGISTERS 1
#define BUBBLE_STAGE_FORM_SHARED 2
int bubble_ext_set_stage_form(bubble_sim *sim, int32_t form);

/* Device pointers of the current slot U^n (valid until the next step). */
int bubble_ext_device_state(bubble_sim *sim, void **field, void **fluid);
/* The cudaStream_t the simulation launches on. */
void *bubble_ext_stream(bubble_sim *sim);
/* Number of kernel launches issued by this simulation so far. */
uint64_t bubble_ext_launches(const bubble_sim *sim);

/* Make the next device allocation of this process fail (host-side fault
 * injection for the failure-handling tests). */
void bubble_ext_inject_allocation_failure(void);

/* Test hook of the stage kernel's bounded waits (the device side of the
 * reference's failure path, src/headless.rs:63-67, which stops a run whose
 * diagnostics go bad).  The next stage launch of `sim` arms, in every CTA
 * that stages planes through TMA, its first plane's mbarrier for
 * `extra_bytes` (1..65536) bytes that no copy will deliver -- no copy is
 * issued for that plane -- and limits the kernel's waits to 2^wait_shift SM
 * cycles (10..31).  Those waits expire, the CTAs set the status word and
 * return with nothing in flight, and the next bubble_synchronize or
 * bubble_diagnostics returns BUBBLE_ERR_TIMEOUT; the context stays usable.
 * Lattices whose tiles all touch the periodic boundary (with the default
 * 16 x 16 tiles: x or y below 34 cells) have no TMA tile, and the hook then
 * changes nothing. */
int bubble_ext_test_expire_stage_wait(bubble_sim *sim, uint32_t extra_bytes, int32_t wait_shift);

/* Raw FP64 result of the diagnostics reduction: sums over cells of the
 * total energy density, broken-phase indicator, fluid kinetic energy
 * density and fluid energy E; the bits of max|v| (a non-negative float);
 * a non-zero `nonfinite` when any term or state value was not finite; the
 * cell count. */
typedef struct bubble_diag_raw {
    double sums[4];
    uint32_t max_v_bits;
    uint32_t nonfinite;
    uint64_t cells;
} bubble_diag_raw;

/* The diagnostics reduction of bubble_diagnostics for a caller that cannot
 * allocate device memory.  No counterpart in the reference, whose
 * reduction always runs on buffers the Simulation allocated itself.
 *
 * For engines that own all device memory through their own pool, real-time
 * loops that must not allocate mid-run, or hosts with a fixed memory
 * budget: the caller passes its own device buffers -- `field` (2 values per
 * cell) and `fluid` (4 per cell), float for the FP32 forms, double for
 * BUBBLE_PRECISION_DOUBLE, in the lattice order of this header -- the
 * lattice's `spec` (grid, model, precision form and equation of state, as
 * given to bubble_create; the schedule fields are not read) and a device
 * pointer `result` to one bubble_diag_raw.  The sums are those
 * bubble_diagnostics reports for the same state and spec (for the
 * perturbation form they include the background energy N e_ref).  The
 * launch goes on `stream` (a cudaStream_t, NULL for the default stream) and
 * is asynchronous.  The call allocates nothing: its scratch (1024 block
 * partials and a completion counter, 49,408 bytes) is a static device array
 * of the library, held on every GPU that loads the library until exit.
 * Any lattice with axes 8..2048 fits; other sizes, and specs that
 * bubble_create would refuse, are rejected with BUBBLE_ERR_INVALID.  The
 * first call on a device loads the module there: make it before any stream
 * capture.  All calls share the scratch: the counter is cleared on `stream`
 * before each launch, and calls that overlap on the GPU race. */
int bubble_diagnostics_noalloc(const void *field, const void *fluid, const bubble_spec *spec, void *result,
                               void *stream);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_GB300_EXT_H */
