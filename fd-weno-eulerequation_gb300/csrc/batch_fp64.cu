// Batched persistent kernel, FP64 parity arithmetic (compiled with
// -fmad=false like the per-solve FP64 stage), plus the batch's small
// control kernels.
#include "batch_kernel.cuh"

namespace wenofd {

namespace {

// k_advance_setup of every member: the step budget of this advance call
// and a clean reduction state (no tile bounds: the batch's tiles may differ
// from the single solve's, so the first step screens every node).
__global__ void k_batch_setup(BatchMember *members, int n, long long max_steps) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    Ctrl *c = members[m].ctrl;
    c->max_steps = max_steps < 0 ? 0x7fffffffffffffffLL : c->steps + max_steps;
    c->done = !(fabs(c->now - c->t_end) > 1e-9);
    c->max_s_bits = 0ull;
    c->screen_bits = 0u;
    c->nan_flag = 0;
    c->bounds_valid = 0;
  }
}

__global__ void k_batch_gather(const BatchMember *members, int n, BatchMemberStatus *out) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    const Ctrl *c = members[m].ctrl;
    out[m].now = c->now;
    out[m].steps = c->steps;
    out[m].error = c->error;
    out[m].done = c->done;
  }
}

}  // namespace

cudaError_t launch_batch_fp64(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                              int *grid) {
  switch (tile_i) {
    case 7: return dev::launch_batch_tile<double, 7, 256>(b, scheme, blocks_per_sm, s, grid);
    case 0:
    case 15: return dev::launch_batch_tile<double, 15, 256>(b, scheme, blocks_per_sm, s, grid);
  }
  return cudaErrorInvalidValue;
}

// With b.members null: attributes and grid of the test instance (its own
// occupancy); else the cooperative launch on that grid.
cudaError_t launch_batch_fp64_withhold(const BatchArgs &b, cudaStream_t s, int *grid) {
  return dev::launch_batch_tile<double, 15, 256, true>(b, kWenoZ, 0, s, grid);
}

cudaError_t launch_batch_setup(BatchMember *members, int n, long long max_steps, cudaStream_t s) {
  k_batch_setup<<<(n + 127) / 128, 128, 0, s>>>(members, n, max_steps);
  return cudaGetLastError();
}

cudaError_t launch_batch_gather(const BatchMember *members, int n, BatchMemberStatus *out, cudaStream_t s) {
  k_batch_gather<<<(n + 127) / 128, 128, 0, s>>>(members, n, out);
  return cudaGetLastError();
}

}  // namespace wenofd
