// FP32-arithmetic stage kernels (the precision form): split fluxes,
// eigenvectors, projection, WENO reconstruction and flux differences in
// FP32; the state is read and written as FP64 and the RK combination
// a*Un + b*U + c*dt*rhs is evaluated in FP64.
#include <cudaTypedefs.h>

#include <mutex>

#include "stage_kernel.cuh"

namespace wenofd {

// With a.flags set the kernel routes each face: linear upwind flux unless a
// node around it is flagged, characteristic WENO otherwise.
cudaError_t launch_stage_fp32(const Geom &g, const StageArgs &a, const StageTma &tma, int scheme, int tile_i,
                              cudaStream_t s) {
  if (a.flags) {
    switch (tile_i) {
      case 0:
      case 15: return dev::launch_stage_tile<float, 15, 256, true>(g, a, tma, scheme, s);
      case 31: return dev::launch_stage_tile<float, 31, 512, true>(g, a, tma, scheme, s);
    }
    return cudaErrorInvalidValue;
  }
  switch (tile_i) {
    case 0:
    case 15: return dev::launch_stage_tile<float, 15, 256>(g, a, tma, scheme, s);
    case 31: return dev::launch_stage_tile<float, 31, 512>(g, a, tma, scheme, s);
  }
  return cudaErrorInvalidValue;
}

namespace {

// cuTensorMapEncodeTiled, reached through the runtime (the library does
// not link the driver library itself).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

}  // namespace

cudaError_t make_stage_tma(const Geom &g, const double *state, const unsigned char *flags, int tile_i,
                           StageTma *out) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode || !out || !state) return cudaErrorInvalidValue;
  const int ti = (tile_i == 31 || tile_i == 7) ? tile_i : 15;
  *out = StageTma{};
  {
    using S = dev::StageSmem32<15, 32>;
    const cuuint64_t dims[3] = {cuuint64_t(g.pitch), cuuint64_t(g.nxt), 4};
    const cuuint64_t strides[2] = {cuuint64_t(g.pitch) * sizeof(double), cuuint64_t(g.plane) * sizeof(double)};
    const cuuint32_t box[3] = {cuuint32_t(S::kBoxJ), cuuint32_t(ti + 6), 4}, step[3] = {1, 1, 1};
    if (encode(&out->u, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(state), dims, strides, box, step,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  if (flags) {
    using S = dev::StageSmem32<15, 32>;
    const cuuint64_t dims[2] = {cuuint64_t(g.pitch), cuuint64_t(g.nxt)};
    const cuuint64_t strides[1] = {cuuint64_t(g.pitch)};
    const cuuint32_t box[2] = {cuuint32_t(S::kFlagBoxJ), cuuint32_t(ti + 4)}, step[2] = {1, 1};
    if (encode(&out->flags, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<unsigned char *>(flags), dims, strides, box,
               step, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

}  // namespace wenofd
