// wenofd_calc_dt_noalloc: the time-step reduction of calculateDeltaT for a
// caller-owned device state, with no memory allocation of any kind.
//
// Who needs this: a caller that must not allocate while it runs -- for
// instance a coupled simulation whose GPU memory is owned by a host
// framework's pool and which hands this library only its own state buffers,
// or a time loop that cannot afford cudaMalloc/cudaFree, which synchronise
// the whole device and stall every other stream the caller has in flight.
// The handle API (wenofd_create) allocates its buffers up front; this entry
// point needs no handle at all.
//
// Scratch: the per-block partial maxima live in a file-scope __device__
// array, g_dt_block_max[kMaxBlocks] (8 KiB), which every GPU that loads the
// library holds until the process exits.  Host code cannot use the symbol
// g_dt_block_max as a device address (on the host it names a stand-in), so
// the first call on each device, with that device current, looks the address
// up once with cudaGetSymbolAddress and caches it; that first call should
// therefore come before any stream capture on that device.  The cache is
// keyed on the device's context as well: after cudaDeviceReset (or any
// other teardown of the primary context) the module is loaded again and the
// array may move, so the next call sees a new context id and looks the
// address up again -- make that call, too, before any stream capture.
//
// Every call shares the one array and leaves its last contents behind.
// Nothing in it has to start at zero: each call's first kernel writes every
// slot that its second kernel reads.  Calls that overlap on the GPU (on two
// streams, or from two threads, on the same device) race on the array.
#include "../../include/wenofd.h"

#include <cuda.h>  // CUresult, CUcontext and cuCtxGetId's type; no link to libcuda
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "guard.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;
constexpr long long kMaxNodes = 1LL << 28;  // 16384 x 16384
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_dt_block_max[kMaxBlocks];

std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // id of the context the address belongs to

// Id of the calling thread's current context (cuCtxGetId, unique for the
// life of the process: a context created after a reset gets a new one), 0
// if none is current.  The driver function is reached through the runtime,
// so the library does not link libcuda.
unsigned long long current_context_id() {
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_setup_mutex
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(fn);
    looked_up = true;
  }
  unsigned long long id = 0;
  if (!get_id || get_id(nullptr, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Per node: s = lx/dx + ly/dy with lx = |u*1 + v*0| + c, ly = |u*0 + v*1| + c
// (getMaxEigenValue(U, 1, 0) / (U, 0, 1), utils/equations.hpp:137-147), as
// src/WENOFD.cpp:419-423 forms it; each block writes its maximum, or NaN if
// any node gave NaN.  This file is compiled without FMA contraction, so the
// values round exactly as in the reference.
__global__ void k_noalloc_block_max(const double *U, long long n, double dx, double dy, double gamma,
                                    double *block_max, unsigned long long *guard) {
  double smax = 0.0;
  int nan_seen = 0;
  // a node whose four values are bit for bit those of the last node this
  // thread evaluated has the same s (uniform regions): skipped
  long long k0 = 0, k1 = 0, k2 = 0, k3 = 0;
  bool have = false;
  for (long long t = blockIdx.x * (long long)kThreads + threadIdx.x; t < n; t += (long long)gridDim.x * kThreads) {
    const double rho = U[t], mu = U[n + t], mv = U[2 * n + t], E = U[3 * n + t];
    const long long a0 = __double_as_longlong(rho), a1 = __double_as_longlong(mu), a2 = __double_as_longlong(mv),
                    a3 = __double_as_longlong(E);
    if (have && a0 == k0 && a1 == k1 && a2 == k2 && a3 == k3) continue;
    k0 = a0;
    k1 = a1;
    k2 = a2;
    k3 = a3;
    have = true;
    const double u = mu / rho, v = mv / rho;
    const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
    const double cs = sqrt(gamma * p / rho);
    const double lx = fabs(u * 1.0 + v * 0.0) + cs;
    const double ly = fabs(u * 0.0 + v * 1.0) + cs;
    const double s = lx / dx + ly / dy;
    if (s != s) nan_seen = 1;
    else if (s > smax) smax = s;
  }
  __shared__ double wmax[kThreads / 32];
  __shared__ int wnan[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, smax, o);
    smax = other > smax ? other : smax;
    nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
  }
  if ((threadIdx.x & 31) == 0) {
    wmax[threadIdx.x >> 5] = smax;
    wnan[threadIdx.x >> 5] = nan_seen;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    int nn = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      m = wmax[w] > m ? wmax[w] : m;
      nn |= wnan[w];
    }
    block_max[WENOFD_IX(guard, blockIdx.x, kMaxBlocks)] = nn ? __longlong_as_double(0x7ff8000000000000LL) : m;
  }
}

// dt = min(1.0, cfl / max s), clipped to t_end - now (src/WENOFD.cpp:401,
// 426-435); NaN when any node's wave speed was NaN (lines 437-442).
__global__ void k_noalloc_finish(const double *block_max, int nblk, double cfl, double now, double t_end,
                                 double *dt_out, unsigned long long *guard) {
  if (threadIdx.x != 0) return;
  double m = 0.0;
  int nn = 0;
  for (int b = 0; b < nblk; ++b) {
    const double x = block_max[WENOFD_IX(guard, b, kMaxBlocks)];
    if (x != x) nn = 1;
    else if (x > m) m = x;
  }
  if (nn) {
    *dt_out = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const double cand = cfl / m;
  double timestep = 1.0;
  if (!(cand > timestep)) timestep = cand;
  if (t_end - now < timestep) timestep = t_end - now;
  *dt_out = timestep;
}

}  // namespace

namespace wenofd {
void set_last_error(const std::string &msg);  // capi.cpp: the text wenofd_last_error() returns
}

namespace {
int fail(int code, const std::string &msg) {
  wenofd::set_last_error(msg);
  return code;
}
}  // namespace

extern "C" int wenofd_calc_dt_noalloc(const double *dev_state, int nx, int ny, double dx, double dy, double gamma,
                                      double cfl, double now, double t_end, double *dev_dt, void *cuda_stream) {
  if (!dev_state || !dev_dt) return fail(WENOFD_BAD_ARG, "wenofd_calc_dt_noalloc: null state or output pointer");
  if (nx < 1 || ny < 1) return fail(WENOFD_BAD_ARG, "wenofd_calc_dt_noalloc: nx and ny must be positive");
  const long long n = (long long)nx * ny;
  if (n > kMaxNodes)
    return fail(WENOFD_BAD_ARG, "wenofd_calc_dt_noalloc: nx*ny = " + std::to_string(n) +
                                    " nodes exceeds the maximum of " + std::to_string(kMaxNodes));
  if (!(dx > 0.0) || !(dy > 0.0)) return fail(WENOFD_BAD_ARG, "wenofd_calc_dt_noalloc: dx and dy must be positive");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(WENOFD_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(WENOFD_BAD_ARG, "wenofd_calc_dt_noalloc: device index too large");
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    // Set-up: once per device (with that device current), and again when the
    // device's context is not the one the cached address belongs to.  A
    // thread with no current context yet reads id 0 and also sets up;
    // cudaGetSymbolAddress makes the device's primary context current.
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_dt_block_max);
      if (e != cudaSuccess)
        return fail(WENOFD_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double *>(p);
      g_scratch_ctx[dev] = current_context_id();
    }
    scratch = g_scratch_ptr[dev];
  }
  long long blocks = (n + kThreads - 1) / kThreads;
  if (blocks > kMaxBlocks) blocks = kMaxBlocks;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  // (the bounds-checked build's guard record; null in the release build,
  // which allocates nothing here)
  unsigned long long *guard = wenofd::guard_record();
  k_noalloc_block_max<<<int(blocks), kThreads, 0, s>>>(dev_state, n, dx, dy, gamma, scratch, guard);
  k_noalloc_finish<<<1, 32, 0, s>>>(scratch, int(blocks), cfl, now, t_end, dev_dt, guard);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WENOFD_CUDA_ERROR, std::string("launch: ") + cudaGetErrorString(e));
  return WENOFD_OK;
}
