/*
 * Raw-state checkpoint and resume.  No reference counterpart: the
 * reference's state lives only in its device buffers
 * (src/gpu/sim.rs:180-245) and a run cannot be continued after exit.
 *
 * A checkpoint file holds the spec, the clock (f32 time and step count),
 * the nucleation schedule and how far it has been consumed, and the current
 * slot's field and fluid arrays (FP32 or FP64), followed by a CRC-32.
 * Restoring it and stepping on gives bit for bit the states the original
 * run would have reached.
 */
#ifndef BUBBLE_CHECKPOINT_H
#define BUBBLE_CHECKPOINT_H

#include "bubble.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Writes the simulation's state at the current step boundary to `path`. */
int bubble_checkpoint_save(bubble_sim *sim, const char *path);

/* Replaces the simulation's model, grid (resizing if needed), schedule,
 * clock and state with the checkpoint's.  The arithmetic stays the
 * simulation's own (fast or strict, single or mixed); an FP64 checkpoint
 * needs an FP64 simulation and an FP32 one an FP32 simulation.  The file is
 * checked (magic, sizes, CRC) before anything changes. */
int bubble_checkpoint_restore(bubble_sim *sim, const char *path);

/* The spec stored in a checkpoint, without touching the device. */
int bubble_checkpoint_spec(const char *path, bubble_spec *out);

/* bubble_create with the checkpoint's spec, then bubble_checkpoint_restore. */
int bubble_checkpoint_open(const char *path, bubble_sim **out);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_CHECKPOINT_H */
