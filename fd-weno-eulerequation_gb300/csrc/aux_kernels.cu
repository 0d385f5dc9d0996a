// Boundary fill, time-step reduction, time-loop control and FP64 norm
// kernels.  Compiled with -fmad=false like the FP64 stage: the time step is
// part of the parity contract.
#include "aux_device.cuh"

#include <math.h>

#include <mutex>

namespace wenofd {

namespace {

constexpr int kReduceThreads = 256;
constexpr int kReduceBlocks = 2 * 152;  // two CTAs per SM of a GB300


__global__ void k_bc_fill(Geom g, double *U, const double *special, const int *active) {
  if (active && *active == 0) return;
  const int total = dev::bc_entries(g);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    dev::bc_fill_entry(g, U, special, t);
}

// calculateDeltaT (src/WENOFD.cpp:398-452).  Per node the reference forms
// tmp = cfl / (lx/dx + ly/dy) with lx = |u*1 + v*0| + c, ly = |u*0 + v*1| + c
// (getMaxEigenValue(U, 1, 0) and (U, 0, 1), utils/equations.hpp:137-147) and
// keeps the minimum.  Correctly rounded division is monotone, so
// min(cfl/s) == cfl/max(s): the reduction keeps max(s), as IEEE bits (all s
// are >= 0, where bit order is value order), and k_dt_finalize divides once.
// A NaN s sets a flag instead of entering the maximum.
__global__ void k_dt_reduce(Geom g, const double *U, Ctrl *c) {
  if (!c->active) return;
  const long long n = (long long)g.nx * g.ny;
  const double gamma = g.gamma;
  double smax = 0.0;
  int nan_seen = 0;
  dev::SpeedMemo memo;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = int(t / g.ny), j = int(t - (t / g.ny) * g.ny);
    const long long base = WENOFD_NODE(g, i, j);
    const double rho = U[base], mu = U[g.plane + base], mv = U[2 * g.plane + base], E = U[3 * g.plane + base];
    if (memo.repeat(rho, mu, mv, E)) continue;
    const double u = mu / rho, v = mv / rho;
    const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
    const double cs = sqrt(gamma * p / rho);
    const double lx = fabs(u * 1.0 + v * 0.0) + cs;
    const double ly = fabs(u * 0.0 + v * 1.0) + cs;
    const double s = lx / g.dx + ly / g.dy;
    if (s != s) nan_seen = 1;
    else if (s > smax) smax = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, smax, o);
    smax = other > smax ? other : smax;
    nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
  }
  __shared__ double wmax[32];
  __shared__ int wnan[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wmax[warp] = smax;
    wnan[warp] = nan_seen;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    int nn = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      m = wmax[w] > m ? wmax[w] : m;
      nn |= wnan[w];
    }
    atomicMax(&c->max_s_bits, (unsigned long long)__double_as_longlong(m));
    if (nn) atomicOr(&c->nan_flag, 1);
  }
}

// Pass 1: L = max over nodes of (s32 - e), a lower bound of max s.
__global__ void k_dt_screen(Geom g, const double *U, Ctrl *c) {
  if (!c->active || c->bounds_valid) return;
  const long long n = (long long)g.nx * g.ny;
  float lo = 0.0f;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = int(t / g.ny), j = int(t - (t / g.ny) * g.ny);
    const long long b = WENOFD_NODE(g, i, j);
    float s, e;
    dev::screen_speed(g, U[b], U[g.plane + b], U[2 * g.plane + b], U[3 * g.plane + b], s, e);
    lo = fmaxf(lo, s - e);
  }
  for (int o = 16; o > 0; o >>= 1) lo = fmaxf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
  __shared__ float wl[32];
  if ((threadIdx.x & 31) == 0) wl[threadIdx.x >> 5] = lo;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, wl[w]);
    atomicMax(&c->screen_bits, __float_as_uint(m));
  }
}

// Pass 2: the exact FP64 s of every node with s32 + e >= L (the node holding
// the maximum is one of them), max-reduced as in k_dt_reduce.  With valid
// per-tile bounds (the last stage of the previous step screened the nodes it
// wrote) a warp per tile skips the tiles whose upper bound stays below L.
__global__ void k_dt_refine(Geom g, const double *U, Ctrl *c, const float2 *bounds, int tile_i) {
  if (!c->active) return;
  const float L = __uint_as_float(c->screen_bits);
  double smax = 0.0;
  int nan_seen = 0;
  dev::SpeedMemo memo;
  auto visit = [&](int i, int j) {
    const long long b = WENOFD_NODE(g, i, j);
    const double rho = U[b], mu = U[g.plane + b], mv = U[2 * g.plane + b], E = U[3 * g.plane + b];
    float s32, e;
    dev::screen_speed(g, rho, mu, mv, E, s32, e);
    if (s32 + e >= L && !memo.repeat(rho, mu, mv, E)) {
      const double s = dev::exact_speed(g, rho, mu, mv, E);
      if (s != s) nan_seen = 1;
      else if (s > smax) smax = s;
    }
  };
  if (bounds && c->bounds_valid) {
    const int tiles_j = (g.ny + 31) / 32, ntiles = ((g.nx + tile_i - 1) / tile_i) * tiles_j;
    const int lane = threadIdx.x & 31;
    const int warps = int(gridDim.x * blockDim.x) >> 5;
    for (int t = int(blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += warps) {
      // (bounds are allocated for tiles of 15 rows, the most tiles)
      if (bounds[WENOFD_IX(g.guard, t, ((g.nx + 14) / 15) * tiles_j)].y < L) continue;  // warp-uniform
      const int i0 = (t / tiles_j) * tile_i, j = (t - (t / tiles_j) * tiles_j) * 32 + lane;
      const int i1 = i0 + tile_i < g.nx ? i0 + tile_i : g.nx;
      if (j < g.ny)
        for (int i = i0; i < i1; ++i) visit(i, j);
    }
  } else {
    const long long n = (long long)g.nx * g.ny;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
      const int i = int(t / g.ny), j = int(t - (t / g.ny) * g.ny);
      visit(i, j);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, smax, o);
    smax = other > smax ? other : smax;
    nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
  }
  __shared__ double wmax[32];
  __shared__ int wnan[32];
  if ((threadIdx.x & 31) == 0) {
    wmax[threadIdx.x >> 5] = smax;
    wnan[threadIdx.x >> 5] = nan_seen;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    int nn = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      m = wmax[w] > m ? wmax[w] : m;
      nn |= wnan[w];
    }
    atomicMax(&c->max_s_bits, (unsigned long long)__double_as_longlong(m));
    if (nn) atomicOr(&c->nan_flag, 1);
  }
}

// Open the gate for one host-driven operation (calc_dt, rk_step, step).
__global__ void k_ctrl_open(Ctrl *c) {
  c->active = 1;
  c->bounds_valid = 0;
  c->max_s_bits = 0ull;
  c->screen_bits = 0u;
  c->nan_flag = 0;
  c->error = 0;
}

// Start of a graph-driven step: run while |now - t_end| > 1e-9 (the loop
// condition of src/WENOFD.cpp:213), no error, and under the step cap.
__global__ void k_step_begin(Ctrl *c) {
  c->active = (!c->done && !c->error && c->steps < c->max_steps) ? 1 : 0;
}

// dt = min(1.0, cfl / max s), then clipped to t_end - now
// (src/WENOFD.cpp:401, 426-435).  NaN -> error NAN_DT (the reference aborts,
// lines 437-442).
__global__ void k_dt_finalize(Ctrl *c) {
  if (!c->active) return;
  const double ms = __longlong_as_double((long long)c->max_s_bits);
  c->max_s_bits = 0ull;
  c->screen_bits = 0u;
  if (c->nan_flag) {
    c->nan_flag = 0;
    c->error = 3;  // WENOFD_NAN_DT
    c->active = 0;
    return;
  }
  const double cand = c->cfl / ms;
  double timestep = 1.0;
  if (!(cand > timestep)) timestep = cand;
  if (c->t_end - c->now < timestep) timestep = c->t_end - c->now;
  if (timestep != timestep) {
    c->error = 3;
    c->active = 0;
    return;
  }
  c->dt = timestep;
}

// m_now += dt; count++ (src/WENOFD.cpp:238-239), then the loop condition.
__global__ void k_step_end(Ctrl *c, int fused) {
  if (!c->active) return;
  c->now += c->dt;
  c->steps += 1;
  c->done = !(fabs(c->now - c->t_end) > 1e-9);
  c->bounds_valid = fused;
}

__global__ void k_set_dt(Ctrl *c, double dt) {
  c->dt = dt;
  c->active = 1;
}

__global__ void k_set_time(Ctrl *c, double now) {
  c->now = now;
  c->bounds_valid = 0;
  c->done = !(fabs(now - c->t_end) > 1e-9);
  c->error = 0;
}

__global__ void k_advance_setup(Ctrl *c, long long max_steps) {
  c->max_steps = max_steps < 0 ? 0x7fffffffffffffffLL : c->steps + max_steps;
  c->done = !(fabs(c->now - c->t_end) > 1e-9);
  c->max_s_bits = 0ull;
  c->screen_bits = 0u;
  c->nan_flag = 0;
  c->bounds_valid = 0;
  c->ind_base = c->steps;
}

__global__ void k_copy_interior(Geom g, const double *src, double *dst, const int *active) {
  if (active && *active == 0) return;
  const long long n = 4LL * g.nx * g.ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int r = int(t / ((long long)g.nx * g.ny));
    const long long rem = t - r * ((long long)g.nx * g.ny);
    const int i = int(rem / g.ny), j = int(rem - (rem / g.ny) * g.ny);
    const long long idx = dev::at(g, r, kGhost + i, kGhost + j);
    dst[idx] = src[idx];
  }
}

// FP64 reductions in a fixed order: each block reduces a fixed slice to
// partials[blk*4 + q]; k_reduce_final combines the blocks in index order.
// kind 0: {max err, sum err, sum err^2} of density against the smooth case's
// exact solution 1 + 0.2 sin(pi (x + y - t)) (utils/equations.hpp:438-439);
// kind 1: sums of the four conserved variables.
// getVitalVarVal (utils/equations.hpp:679-694) of every interior node: rho,
// u, v, pre, c, E as planes k = 0..5 of nx x ny (j fastest), planes 0-3 at
// out03, 4-5 at out45, each in the reference's operation order (this unit
// has no multiply-add contraction).
__global__ void k_output_vars(Geom g, const double *U, double *out03, double *out45) {
  const long long n = (long long)g.nx * g.ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = int(t / g.ny), j = int(t - (t / g.ny) * g.ny);
    const long long k = WENOFD_NODE(g, i, j);
    const double rho = U[k];
    const double u = U[g.plane + k] / U[k];
    const double v = U[2 * g.plane + k] / U[k];
    const double E = U[3 * g.plane + k];
    const double pre = (g.gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
    const double c = sqrt(g.gamma * pre / rho);
    out03[t] = rho;
    out03[n + t] = u;
    out03[2 * n + t] = v;
    out03[3 * n + t] = pre;
    out45[t] = c;
    out45[n + t] = E;
  }
}

__global__ void k_reduce_blocks(Geom g, const double *U, int kind, double t, double xl, double yl,
                                double *partials) {
  const long long n = (long long)g.nx * g.ny;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const double gx = (xl + 0 * g.dx) - g.dx * kGhost;  // ghost-origin coordinate (src/WENOFD.cpp:76-79)
  const double gy = yl - g.dy * kGhost;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int i = int(p / g.ny), j = int(p - (p / g.ny) * g.ny);
    const long long base = WENOFD_NODE(g, i, j);
    if (kind == 0) {
      const double x = gx + (kGhost + i) * g.dx, y = gy + (kGhost + j) * g.dy;
      const double uref = 1 + 0.2 * sin(M_PI * (x + y - t));
      const double err = fabs(uref - U[base]);
      acc[0] = err > acc[0] ? err : acc[0];
      acc[1] += err;
      acc[2] += err * err;
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] += U[r * g.plane + base];
    }
  }
  __shared__ double sh[4][kReduceThreads];
#pragma unroll
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double o = sh[q][threadIdx.x + w];
        if (kind == 0 && q == 0) sh[q][threadIdx.x] = o > sh[q][threadIdx.x] ? o : sh[q][threadIdx.x];
        else sh[q][threadIdx.x] += o;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[WENOFD_IX(g.guard, blockIdx.x * 4 + threadIdx.x, 4 * kReduceBlocks)] = sh[threadIdx.x][0];
}

__global__ void k_reduce_final(Geom g, int kind, const double *partials, int nblk, double *out) {
  if (threadIdx.x != 0) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < nblk; ++b)
    for (int q = 0; q < 4; ++q) {
      const double o = partials[b * 4 + q];
      if (kind == 0 && q == 0) acc[0] = o > acc[0] ? o : acc[0];
      else acc[q] += o;
    }
  if (kind == 0) {  // src/WENOFD.cpp:1359-1360
    out[0] = acc[0];
    out[1] = acc[1] / g.nx / g.ny;
    out[2] = sqrt(acc[2] / g.nx / g.ny);
  } else {
    for (int q = 0; q < 4; ++q) out[q] = acc[q];
  }
}

// One index one past the end of buf[4] through the always-on guard (not the
// macro, so the access is guarded in either build): the guard sends it to
// buf[0] and records the violation in rec.
constexpr unsigned long long kSelftestSite = guard_site(__FILE__, __LINE__);
__global__ void k_guard_selftest(unsigned long long *rec, int *buf) {
  const int i = dev::guard_ix<kSelftestSite>(rec, true, 4, 4);
  buf[i] += 1;
}

int grid_for(long long work, int threads) {
  long long b = (work + threads - 1) / threads;
  if (b > 152LL * 16) b = 152LL * 16;
  return int(b < 1 ? 1 : b);
}

}  // namespace

Geom make_geom(int nx, int ny, double dx, double dy, double gamma, double zp_lambda, int bc_left,
               int bc_right, int bc_y, int gravity) {
  Geom g;
  g.nx = nx;
  g.ny = ny;
  g.nxt = nx + 2 * kGhost;
  g.nyt = ny + 2 * kGhost;
  g.pitch = (g.nyt + 31) / 32 * 32;
  g.plane = (long long)g.nxt * g.pitch;
  g.dx = dx;
  g.dy = dy;
  g.gamma = gamma;
  g.zp_lambda = zp_lambda;
  g.bc_left = bc_left;
  g.bc_right = bc_right;
  g.bc_y = bc_y;
  g.gravity = gravity;
  g.gamma32 = float(gamma);
  g.zpl32 = float(zp_lambda);
  g.inv_dx32 = float(1.0 / dx);
  g.inv_dy32 = float(1.0 / dy);
  g.guard = guard_record();
  return g;
}

cudaError_t launch_guard_selftest(unsigned long long *rec, int *buf, unsigned long long *site, cudaStream_t s) {
  k_guard_selftest<<<1, 1, 0, s>>>(rec, buf);
  *site = kSelftestSite;
  return cudaGetLastError();
}

#ifdef WENOFD_BOUNDS_CHECK
unsigned long long *guard_record() {
  static std::mutex mu;
  static unsigned long long *rec[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (rec[dev] == nullptr) {
    unsigned long long *p = nullptr;
    if (cudaMalloc(&p, kGuardWords * sizeof(unsigned long long)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, kGuardWords * sizeof(unsigned long long)) != cudaSuccess) {
      cudaFree(p);
      return nullptr;
    }
    rec[dev] = p;
  }
  return rec[dev];
}
#else
unsigned long long *guard_record() { return nullptr; }
#endif

cudaError_t launch_bc_fill(const Geom &g, double *U, const double *special, const int *active, cudaStream_t s) {
  const long long work = dev::bc_entries(g);
  k_bc_fill<<<grid_for(work, 256), 256, 0, s>>>(g, U, special, active);
  return cudaGetLastError();
}

cudaError_t launch_dt_reduce(const Geom &g, const double *U, Ctrl *c, cudaStream_t s) {
  k_dt_reduce<<<grid_for((long long)g.nx * g.ny, 256), 256, 0, s>>>(g, U, c);
  return cudaGetLastError();
}

cudaError_t launch_dt_reduce_two_pass(const Geom &g, const double *U, Ctrl *c, const float2 *bounds, int tile_i,
                                      cudaStream_t s) {
  const int grid = grid_for((long long)g.nx * g.ny, 256);
  k_dt_screen<<<grid, 256, 0, s>>>(g, U, c);
  k_dt_refine<<<grid, 256, 0, s>>>(g, U, c, bounds, tile_i > 0 ? tile_i : 15);
  return cudaGetLastError();
}

cudaError_t launch_ctrl_open(Ctrl *c, cudaStream_t s) {
  k_ctrl_open<<<1, 1, 0, s>>>(c);
  return cudaGetLastError();
}
cudaError_t launch_step_begin(Ctrl *c, cudaStream_t s) {
  k_step_begin<<<1, 1, 0, s>>>(c);
  return cudaGetLastError();
}
cudaError_t launch_dt_finalize(Ctrl *c, cudaStream_t s) {
  k_dt_finalize<<<1, 1, 0, s>>>(c);
  return cudaGetLastError();
}
cudaError_t launch_step_end(Ctrl *c, int fused, cudaStream_t s) {
  k_step_end<<<1, 1, 0, s>>>(c, fused);
  return cudaGetLastError();
}
cudaError_t launch_set_dt(Ctrl *c, double dt, cudaStream_t s) {
  k_set_dt<<<1, 1, 0, s>>>(c, dt);
  return cudaGetLastError();
}
cudaError_t launch_set_time(Ctrl *c, double now, cudaStream_t s) {
  k_set_time<<<1, 1, 0, s>>>(c, now);
  return cudaGetLastError();
}
cudaError_t launch_advance_setup(Ctrl *c, long long max_steps, cudaStream_t s) {
  k_advance_setup<<<1, 1, 0, s>>>(c, max_steps);
  return cudaGetLastError();
}
cudaError_t launch_copy_interior(const Geom &g, const double *src, double *dst, const int *active, cudaStream_t s) {
  k_copy_interior<<<grid_for(4LL * g.nx * g.ny, 256), 256, 0, s>>>(g, src, dst, active);
  return cudaGetLastError();
}

int reduce_blocks() { return kReduceBlocks; }

cudaError_t launch_output_vars(const Geom &g, const double *U, double *out03, double *out45, cudaStream_t s) {
  k_output_vars<<<grid_for((long long)g.nx * g.ny, 256), 256, 0, s>>>(g, U, out03, out45);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const Geom &g, const double *U, int kind, double t, double xl, double yl,
                          double *partials, double *out, cudaStream_t s) {
  k_reduce_blocks<<<kReduceBlocks, kReduceThreads, 0, s>>>(g, U, kind, t, xl, yl, partials);
  k_reduce_final<<<1, 32, 0, s>>>(g, kind, partials, kReduceBlocks, out);
  return cudaGetLastError();
}

}  // namespace wenofd
