// FP64 stage kernels: the parity path.  This translation unit is compiled
// with -fmad=false so that no multiply-add is contracted into an FMA; with
// IEEE division and square root every operation then rounds as in the
// reference built with -ffp-contract=off.
#include "stage_kernel.cuh"

namespace wenofd {

// The tile's halo arrives by TMA through the map in `tma` (make_stage_tma
// for this tile height).
cudaError_t launch_stage_fp64(const Geom &g, const StageArgs &a, const StageTma &tma, int scheme, int tile_i,
                              cudaStream_t s) {
  switch (tile_i) {
    case 0:
    case 15: return dev::launch_stage_tile<double, 15, 256>(g, a, tma, scheme, s);
    case 7: return dev::launch_stage_tile<double, 7, 256>(g, a, tma, scheme, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wenofd
