// Batched persistent kernel, learned form: the FP32 batched kernel whose
// stage tiles route each face with the member's indicator flags (linear
// upwind flux unless a node around the face is flagged), as the per-solve
// learned form does.  The indicator itself runs between launches
// (launch_indicator_batch, learned.cu).
#include "batch_kernel.cuh"

namespace wenofd {

cudaError_t launch_batch_learned(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                                 int *grid) {
  switch (tile_i) {
    case 0:
    case 15: return dev::launch_batch_tile<float, 15, 256, false, true>(b, scheme, blocks_per_sm, s, grid);
    case 31: return dev::launch_batch_tile<float, 31, 512, false, true>(b, scheme, blocks_per_sm, s, grid);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wenofd
