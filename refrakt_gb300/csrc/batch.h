// Batched persistent chaos launch (batch.cu): instance table, work units, launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_args.h"

namespace rfk {

cudaError_t launch_batch(int threads, int slots, const BatchArgs& a, cudaStream_t st, int* grid_out);
// a genome-specialised batch kernel (specialize.cpp): sets its shared-memory limit and returns
// its persistent grid (0 on failure); then launches it
int batch_spec_grid(const void* kernel, int threads, int slots, uint32_t max_prog_words);
cudaError_t launch_batch_spec(const void* kernel, int threads, int slots, int grid, const BatchArgs& a,
                              cudaStream_t st);

}  // namespace rfk
