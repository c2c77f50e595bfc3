// The opaque handle behind `bubble_sim *` (include/bubble.h), shared by the
// translation units that implement its entry points.
#pragma once

#include <memory>

#include "simulation.h"

struct bubble_sim {
    std::unique_ptr<bubble::Simulation> impl;
};
