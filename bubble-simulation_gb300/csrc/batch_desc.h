// Descriptor of one lattice of a batch, shared by the host driver (which
// fills it) and the persistent batch kernel (which reads it from global
// memory).
#pragma once

#include <cstdint>

#include "params.h"
#include "tma.h"

namespace bubble {

struct alignas(64) BatchLattice {
    StageMaps maps[3];  // TMA maps of each slot as a stage input
    V2<float> *field[3];
    V4<float> *fluid[3];
    LatticeParams<float> P;
    float dt;
    int32_t lz, tiles_xy, chunks;
    int32_t item_begin, cur0, tma_ok, _pad;
};

}  // namespace bubble
