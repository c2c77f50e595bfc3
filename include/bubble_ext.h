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
                                   the reference's own kernel structure      */
int bubble_ext_set_path(bubble_sim *sim, int32_t path);

/* Tile of the fused kernel: y extent (4 or 8 for FP32, 4 for FP64; x is 32)
 * and z chunk (planes marched per CTA). */
int bubble_ext_set_tile(bubble_sim *sim, int32_t ty, int32_t lz);
int bubble_ext_get_tile(const bubble_sim *sim, int32_t *ty, int32_t *lz);

/* Device pointers of the current slot U^n (valid until the next step). */
int bubble_ext_device_state(bubble_sim *sim, void **field, void **fluid);
/* The cudaStream_t the simulation launches on. */
void *bubble_ext_stream(bubble_sim *sim);
/* Number of kernel launches issued by this simulation so far. */
uint64_t bubble_ext_launches(const bubble_sim *sim);

/* Make the next device allocation of this process fail (host-side fault
 * injection for the failure-handling tests). */
void bubble_ext_inject_allocation_failure(void);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_GB300_EXT_H */
