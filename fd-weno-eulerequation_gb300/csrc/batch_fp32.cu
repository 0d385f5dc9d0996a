// Batched persistent kernel, FP32 precision form (the per-solve FP32 stage
// and the two-pass time-step reduction, inside one cooperative launch).
#include "batch_kernel.cuh"

namespace wenofd {

cudaError_t launch_batch_fp32(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                              int *grid) {
  switch (tile_i) {
    case 0:
    case 15: return dev::launch_batch_tile<float, 15, 256>(b, scheme, blocks_per_sm, s, grid);
    case 31: return dev::launch_batch_tile<float, 31, 512>(b, scheme, blocks_per_sm, s, grid);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wenofd
