// FP32-arithmetic stage kernels (the precision form): split fluxes,
// eigenvectors, projection, WENO reconstruction and flux differences in
// FP32; the state is read and written as FP64 and the RK combination
// a*Un + b*U + c*dt*rhs is evaluated in FP64.
#include "stage_kernel.cuh"

namespace wenofd {

// With a.flags set the kernel routes each face: linear upwind flux unless a
// node around it is flagged, characteristic WENO otherwise.
cudaError_t launch_stage_fp32(const Geom &g, const StageArgs &a, int scheme, int tile_i, cudaStream_t s) {
  if (a.flags) {
    switch (tile_i) {
      case 0:
      case 15: return dev::launch_stage_tile<float, 15, 256, true>(g, a, scheme, s);
      case 31: return dev::launch_stage_tile<float, 31, 512, true>(g, a, scheme, s);
    }
    return cudaErrorInvalidValue;
  }
  switch (tile_i) {
    case 0:
    case 15: return dev::launch_stage_tile<float, 15, 256>(g, a, scheme, s);
    case 31: return dev::launch_stage_tile<float, 31, 512>(g, a, scheme, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wenofd
