// gdp_learned.h -- launchers of the learned-marking round loop (gdp_learned.cu).
#pragma once

#include <cuda_runtime.h>

#include "gdp_internal.h"

namespace gdp {

// Resets the per-row learning state and runs every round in one cooperative
// launch (P.learned: 1 learned rounds, 2 trace rounds).
int launch_learned(const DevProblem &P, int grid, int vec_blocks, cudaStream_t s);
int learned_occupancy(int *blocks_per_sm);

}  // namespace gdp
