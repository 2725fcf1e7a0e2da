// Rollout hooks of the learned lidar surrogate (surrogate.cu), for api.cu.
#pragma once
#include <cuda_runtime.h>

#include "objects.h"

// Allocates the surrogate's inference buffers for the sim's cars (call before capture).
int surrogate_prepare(racer_surrogate* s, racer_sim* sim);
// Lidar rows of obs after the physics step: prediction, audit or exact fallback. The step
// (*step_base if given, read on the device, + step_add) picks the spot check's beam offset.
int surrogate_lidar(racer_surrogate* s, racer_sim* sim, float* obs, bool audit, float fallback, cudaStream_t st,
                    const int64_t* step_base, int64_t step_add);
// Host-side bookkeeping of a replayed rollout (`audits` of its `steps` were audit steps).
void surrogate_account(racer_surrogate* s, racer_sim* sim, int steps, int audits);
