// Training data of the learned troubled-cell indicator (learned.cu):
//  - k_features: 5x5 windows of density and pressure per cell, normalised
//    (FP32), the network's 50 inputs;
//  - k_labels: 1 where WENO-Z's nonlinear weights leave the linear weights
//    (FP64, the training target).
// Compiled with -fmad=false: features and labels then round exactly like the
// oracle's restatement (oracle/wenofd_oracle.c), which tests hold them to.
#include "guard.cuh"
#include "learned_common.cuh"
#include "physics.cuh"

namespace wenofd {
namespace lrn {

// ------------------------------------------------------------- features

// The 50 features of interior node c (index i * ny + j) into row[0..49].
__device__ __forceinline__ void cell_features(const Geom &g, const double *U, long long c, float *row) {
  const float gam = float(g.gamma);
  {
    c = WENOFD_IX(g.guard, c, (long long)g.nx * g.ny);
    const int i = int(c / g.ny), j = int(c - (c / g.ny) * g.ny);
    float wr[25], wp[25];
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) {
        const long long base = WENOFD_GNODE(g, kGhost + i + a - 2, kGhost + j + b - 2);
        const float r = float(U[base]), mu = float(U[g.plane + base]), mv = float(U[2 * g.plane + base]),
                    E = float(U[3 * g.plane + base]);
        wr[a * 5 + b] = r;
        wp[a * 5 + b] = pressure32(gam, r, mu, mv, E);
      }
    float o[25];
    normalise(wr, o);
    for (int k = 0; k < 25; ++k) row[k] = o[k];
    normalise(wp, o);
    for (int k = 0; k < 25; ++k) row[25 + k] = o[k];
  }
}

__global__ void k_features(Geom g, const double *U, float *feat) {
  const long long n = (long long)g.nx * g.ny;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
    cell_features(g, U, c, feat + c * kIn);
}

// ----------------------------------------------------- balanced sampling
//
// wenofd_indicator_sample: every node of class y (its label) is kept when a
// 32-bit hash of (seed, node) lies below thr[y] = k_y / count_y * 2^32, so
// about k_y nodes of each class are kept, independently, and the same seed
// keeps the same nodes.  Kept nodes are written in node order: block b of
// kSampleBlocks scans the contiguous node range [b * R, (b + 1) * R).

constexpr int kSampleBlocks = 1024, kSampleThreads = 256;

__device__ __forceinline__ unsigned sample_hash(unsigned long long seed, long long node) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(node + 1);  // splitmix64
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return unsigned(z >> 32);
}

__device__ __forceinline__ bool sample_keep(const unsigned char *labels, long long c, unsigned long long seed,
                                            unsigned long long thr0, unsigned long long thr1) {
  return (unsigned long long)sample_hash(seed, c) < (labels[c] ? thr1 : thr0);
}

__global__ void k_count_positive(const unsigned char *labels, long long n, unsigned long long *count) {
  unsigned local = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
    local += labels[c] ? 1u : 0u;
  local = __reduce_add_sync(0xffffffffu, local);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, (unsigned long long)local);
}

// Pass 1: kept nodes per block.  Pass 2 (offsets[b] = kept nodes of the
// blocks before b): each kept node's output row, in node order; rows past
// `capacity` are dropped.
template <bool WRITE>
__global__ void k_sample_pass(const unsigned char *labels, long long n, unsigned long long seed,
                              unsigned long long thr0, unsigned long long thr1, unsigned *block_count,
                              const long long *offsets, long long capacity, long long *cells, float *y) {
  __shared__ unsigned warp_total[kSampleThreads / 32];
  const long long per = (n + kSampleBlocks - 1) / kSampleBlocks;
  const long long first = blockIdx.x * per, last = first + per < n ? first + per : n;
  long long base = WRITE ? offsets[blockIdx.x] : 0;
  unsigned kept = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long c0 = first; c0 < last; c0 += kSampleThreads) {
    const long long c = c0 + threadIdx.x;
    const bool keep = c < last && sample_keep(labels, c, seed, thr0, thr1);
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_total[warp] = __popc(ballot);
    __syncthreads();
    unsigned before = __popc(ballot & ((1u << lane) - 1u)), chunk = 0;
    for (int w = 0; w < kSampleThreads / 32; ++w) {
      if (w < warp) before += warp_total[w];
      chunk += warp_total[w];
    }
    if (WRITE && keep) {
      const long long row = base + before;
      if (row < capacity) {
        cells[row] = c;
        y[row] = labels[c] ? 1.0f : 0.0f;
      }
    }
    base += chunk;
    kept += chunk;
    __syncthreads();
  }
  if (!WRITE && threadIdx.x == 0) block_count[blockIdx.x] = kept;
}

__global__ void k_features_of(Geom g, const double *U, const long long *cells, long long rows, float *feat) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x)
    cell_features(g, U, cells[r], feat + r * kIn);
}

// --------------------------------------------------------------- labels

// Row k of the left eigenvectors (utils/equations.hpp:174-236) from the
// face-average state's primitives.
template <int DIR>
__device__ __forceinline__ void left_row(int k, double u, double v, double c, double B1, double B2, double l[4]) {
  const double ic = 1.0 / c, nc = (DIR == 0 ? u : v) / c;
  if (DIR == 0) {
    if (k == 0) { l[0] = (B2 + nc) / 2; l[1] = -(B1 * u + ic) / 2; l[2] = -(B1 * v) / 2; l[3] = B1 / 2; }
    if (k == 1) { l[0] = v; l[1] = 0; l[2] = -1; l[3] = 0; }
    if (k == 2) { l[0] = 1 - B2; l[1] = B1 * u; l[2] = B1 * v; l[3] = -B1; }
    if (k == 3) { l[0] = (B2 - nc) / 2; l[1] = -(B1 * u - ic) / 2; l[2] = -B1 * v / 2; l[3] = B1 / 2; }
  } else {
    if (k == 0) { l[0] = (B2 + nc) / 2; l[1] = -(B1 * u) / 2; l[2] = -(B1 * v + ic) / 2; l[3] = B1 / 2; }
    if (k == 1) { l[0] = -u; l[1] = 1; l[2] = 0; l[3] = 0; }
    if (k == 2) { l[0] = 1 - B2; l[1] = B1 * u; l[2] = B1 * v; l[3] = -B1; }
    if (k == 3) { l[0] = (B2 - nc) / 2; l[1] = -(B1 * u) / 2; l[2] = -(B1 * v - ic) / 2; l[3] = B1 / 2; }
  }
}

__device__ double side_deviation(const double v[5], double scale) {
  double lo = v[0], hi = v[0];
  for (int s = 1; s < 5; ++s) {
    lo = v[s] < lo ? v[s] : lo;
    hi = v[s] > hi ? v[s] : hi;
  }
  if (hi - lo <= 1e-2 * scale) return 0.0;
  double w0, w1, w2;
  dev::wenoz_weights<double>(v[0], v[1], v[2], v[3], v[4], w0, w1, w2);
  return fmax(fabs(w0 - 0.1), fmax(fabs(w1 - 0.6), fabs(w2 - 0.3)));
}

// Largest WENO-Z weight deviation over the characteristic fields and sides
// of the face between (ei-1, ej) and (ei, ej) (DIR 0) or (ei, ej-1), (ei, ej).
template <int DIR>
__device__ double face_deviation(const Geom &g, const double *U, int ei, int ej) {
  const int di = DIR == 0 ? 1 : 0, dj = DIR == 0 ? 0 : 1;
  double ave[4];
  for (int r = 0; r < 4; ++r)
    ave[r] = 0.5 * (U[r * g.plane + WENOFD_GNODE(g, ei - di, ej - dj)] + U[r * g.plane + WENOFD_GNODE(g, ei, ej)]);
  double u, v, p;
  dev::primitives<double>(g.gamma, ave, u, v, p);
  const double c = sqrt(g.gamma * p / ave[0]);
  const double B1 = (g.gamma - 1) / (c * c);
  const double B2 = B1 * (u * u + v * v) / 2;
  double fp[6][4], fm[6][4];
  for (int s = 0; s < 6; ++s) {
    double q[4];
    for (int r = 0; r < 4; ++r) q[r] = U[r * g.plane + WENOFD_GNODE(g, ei + (s - 3) * di, ej + (s - 3) * dj)];
    dev::flux_split<double, DIR>(g.gamma, q, fm[s], fp[s]);
  }
  double vp[4][5], vm[4][5], scale = 0.0;
  for (int k = 0; k < 4; ++k) {
    double l[4];
    left_row<DIR>(k, u, v, c, B1, B2, l);
    for (int s = 0; s < 5; ++s) {
      vp[k][s] = l[0] * fp[s][0] + l[1] * fp[s][1] + l[2] * fp[s][2] + l[3] * fp[s][3];
      vm[k][4 - s] = l[0] * fm[s + 1][0] + l[1] * fm[s + 1][1] + l[2] * fm[s + 1][2] + l[3] * fm[s + 1][3];
      scale = fmax(scale, fmax(fabs(vp[k][s]), fabs(vm[k][4 - s])));
    }
  }
  double dev = 0.0;
  for (int k = 0; k < 4; ++k) dev = fmax(dev, fmax(side_deviation(vp[k], scale), side_deviation(vm[k], scale)));
  return dev;
}

__global__ void k_labels(Geom g, const double *U, unsigned char *labels, double deviation) {
  const long long n = (long long)g.nx * g.ny;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int ei = kGhost + int(c / g.ny), ej = kGhost + int(c - (c / g.ny) * g.ny);
    double d = face_deviation<0>(g, U, ei, ej);
    d = fmax(d, face_deviation<0>(g, U, ei + 1, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej + 1));
    labels[c] = d > deviation ? 1 : 0;
  }
}


}  // namespace lrn

cudaError_t launch_features(const Geom &g, const double *U, float *feat, cudaStream_t s) {
  lrn::k_features<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, feat);
  return cudaGetLastError();
}

cudaError_t launch_labels(const Geom &g, const double *U, unsigned char *labels, double deviation, cudaStream_t s) {
  lrn::k_labels<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, labels, deviation);
  return cudaGetLastError();
}

int sample_blocks() { return lrn::kSampleBlocks; }

cudaError_t launch_count_positive(const unsigned char *labels, long long n, unsigned long long *count,
                                  cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  lrn::k_count_positive<<<lrn::grid_for(n, 256, 152 * 8), 256, 0, s>>>(labels, n, count);
  return cudaGetLastError();
}

cudaError_t launch_sample_count(const unsigned char *labels, long long n, unsigned long long seed,
                                unsigned long long thr0, unsigned long long thr1, unsigned *block_count,
                                cudaStream_t s) {
  lrn::k_sample_pass<false><<<lrn::kSampleBlocks, lrn::kSampleThreads, 0, s>>>(labels, n, seed, thr0, thr1,
                                                                                block_count, nullptr, 0, nullptr,
                                                                                nullptr);
  return cudaGetLastError();
}

cudaError_t launch_sample_write(const Geom &g, const double *U, const unsigned char *labels, unsigned long long seed,
                                unsigned long long thr0, unsigned long long thr1, const long long *offsets,
                                long long capacity, long long rows, long long *cells, float *x, float *y,
                                cudaStream_t s) {
  const long long n = (long long)g.nx * g.ny;
  lrn::k_sample_pass<true><<<lrn::kSampleBlocks, lrn::kSampleThreads, 0, s>>>(labels, n, seed, thr0, thr1, nullptr,
                                                                               offsets, capacity, cells, y);
  if (rows > 0) lrn::k_features_of<<<lrn::grid_for(rows, 128, 152 * 32), 128, 0, s>>>(g, U, cells, rows, x);
  return cudaGetLastError();
}

}  // namespace wenofd
