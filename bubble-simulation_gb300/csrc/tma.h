// Tensor maps for the TMA staging of the fused stage kernel.
//
// One pair per RK slot used as a stage input: `fluid` views the slot's
// (E, Zx, Zy, Zz) array as a 4-d tensor (4, nx, ny, nz) and `field` views
// the (phi, pi) array as a 3-d tensor (2 nx, ny, nz), both of the state's
// element type, with a box of one (TX + 4) x (TY + 4) plane of the tile.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>

namespace bubble {

struct StageMaps {
    CUtensorMap fluid;
    CUtensorMap field;
};

// Encodes the maps for a slot.  Returns true when TMA can address this
// lattice (the field row pitch 2 nx elements must be a multiple of 16
// bytes); false leaves the kernel on its per-element staging path.
bool encode_stage_maps(StageMaps *out, const void *field, const void *fluid, int nx, int ny, int nz,
                       int tile_x, int tile_y, size_t elem_bytes);

}  // namespace bubble
