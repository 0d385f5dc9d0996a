// Learned troubled-cell indicator: a per-cell MLP (50 -> 32 -> 32 -> 1, GELU,
// sigmoid) that decides which faces need characteristic WENO-Z and which can
// take the linear fifth-order upwind flux.  No counterpart in the reference;
// WENO-Z (include/Utility.hpp:457-504) is both its label source and its
// fallback.
//
//  - k_features: 5x5 windows of density and pressure per cell, normalised
//    (FP32), the network's 50 inputs;
//  - k_labels: 1 where WENO-Z's nonlinear weights leave the linear weights
//    (FP64, the training target);
//  - k_mlp_forward / k_mlp_backward / k_adam: FP32 training kernels;
//  - k_indicator_tc: inference on the 5th-generation tensor cores -- BF16
//    operands in shared memory, tcgen05.mma with FP32 accumulators in tensor
//    memory, tcgen05.ld for the epilogue -- writing one flag per cell.
//
// Compiled with -fmad=false: features and labels then round exactly like the
// oracle's restatement (oracle/wenofd_oracle.c), which tests hold them to.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wenofd.h"
#include "convert.cuh"
#include "physics.cuh"
#include "wenofd_internal.h"

namespace wenofd {
namespace lrn {

constexpr int kIn = 50, kHid = 32;
constexpr int oW1 = 0, oB1 = 1600, oW2 = 1632, oB2 = 2656, oW3 = 2688, oB3 = 2720;
constexpr int kParams = 2721;
constexpr float kFlat = 1e-4f;  // relative range below which a window counts as flat

__device__ __forceinline__ float gelu(float z) {
  const float k = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * z * (1.0f + tanhf(k * (z + 0.044715f * z * z * z)));
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float k = 0.7978845608028654f;
  const float t = tanhf(k * (z + 0.044715f * z * z * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * k * (1.0f + 3.0f * 0.044715f * z * z);
}

__device__ __forceinline__ float pressure32(float gamma, float r, float mu, float mv, float E) {
  const float u = mu / r, v = mv / r;
  return (gamma - 1.0f) * (E - 0.5f * r * (u * u + v * v));
}

// (v - centre) * (1 / max|v - centre|) over the 25-point window, or zeros when the
// window is flat (range <= 1e-4 (|centre| + 1e-12)).
__device__ __forceinline__ void normalise(const float w[25], float out[25]) {
  const float c = w[12];
  float R = 0.0f;
#pragma unroll
  for (int k = 0; k < 25; ++k) R = fmaxf(R, fabsf(w[k] - c));
  if (R <= kFlat * (fabsf(c) + 1e-12f)) {
#pragma unroll
    for (int k = 0; k < 25; ++k) out[k] = 0.0f;
    return;
  }
  const float inv = 1.0f / R;
#pragma unroll
  for (int k = 0; k < 25; ++k) out[k] = (w[k] - c) * inv;
}

// GELU for inference: the same tanh form with the hardware tanh
// approximation (the BF16 operands that follow are coarser than its error).
__device__ __forceinline__ float gelu_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.7978845608028654f * (z + 0.044715f * z * z * z)));
  return 0.5f * z * (1.0f + t);
}

// ------------------------------------------------------------- features

__global__ void k_features(Geom g, const double *U, float *feat) {
  const long long n = (long long)g.nx * g.ny;
  const float gam = float(g.gamma);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = int(c / g.ny), j = int(c - (c / g.ny) * g.ny);
    float wr[25], wp[25];
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) {
        const long long base = (long long)(kGhost + i + a - 2) * g.pitch + (kGhost + j + b - 2);
        const float r = float(U[base]), mu = float(U[g.plane + base]), mv = float(U[2 * g.plane + base]),
                    E = float(U[3 * g.plane + base]);
        wr[a * 5 + b] = r;
        wp[a * 5 + b] = pressure32(gam, r, mu, mv, E);
      }
    float o[25];
    normalise(wr, o);
    for (int k = 0; k < 25; ++k) feat[c * kIn + k] = o[k];
    normalise(wp, o);
    for (int k = 0; k < 25; ++k) feat[c * kIn + 25 + k] = o[k];
  }
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
    ave[r] = 0.5 * (U[r * g.plane + (long long)(ei - di) * g.pitch + (ej - dj)] +
                    U[r * g.plane + (long long)ei * g.pitch + ej]);
  double u, v, p;
  dev::primitives<double>(g.gamma, ave, u, v, p);
  const double c = sqrt(g.gamma * p / ave[0]);
  const double B1 = (g.gamma - 1) / (c * c);
  const double B2 = B1 * (u * u + v * v) / 2;
  double fp[6][4], fm[6][4];
  for (int s = 0; s < 6; ++s) {
    double q[4];
    for (int r = 0; r < 4; ++r) q[r] = U[r * g.plane + (long long)(ei + (s - 3) * di) * g.pitch + (ej + (s - 3) * dj)];
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

__global__ void k_labels(Geom g, const double *U, unsigned char *labels) {
  const long long n = (long long)g.nx * g.ny;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int ei = kGhost + int(c / g.ny), ej = kGhost + int(c - (c / g.ny) * g.ny);
    double d = face_deviation<0>(g, U, ei, ej);
    d = fmax(d, face_deviation<0>(g, U, ei + 1, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej + 1));
    labels[c] = d > 1e-2 ? 1 : 0;
  }
}

// ---------------------------------------------------- FP32 training kernels

__global__ void k_mlp_forward(const float *P, const float *X, long long n, float *logits) {
  __shared__ float sp[kParams];
  for (int k = threadIdx.x; k < kParams; k += blockDim.x) sp[k] = P[k];
  __syncthreads();
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
    float h1[kHid];
    for (int o = 0; o < kHid; ++o) {
      float z = sp[oB1 + o];
      for (int k = 0; k < kIn; ++k) z += sp[oW1 + o * kIn + k] * X[s * kIn + k];
      h1[o] = gelu(z);
    }
    float out = sp[oB3];
    for (int o = 0; o < kHid; ++o) {
      float z = sp[oB2 + o];
      for (int k = 0; k < kHid; ++k) z += sp[oW2 + o * kHid + k] * h1[k];
      out += sp[oW3 + o] * gelu(z);
    }
    logits[s] = out;
  }
}

// One block = kBB samples of the batch.  Per sample: forward, dL/dlogit of
// the mean binary cross-entropy (scaled by inv_n), back-propagation to dz1,
// dz2.  Then the block sums the weight gradients over its samples and adds
// them (and its loss share) to grad / loss with one atomic per entry.
constexpr int kBB = 128;

__global__ void __launch_bounds__(kBB) k_mlp_backward(const float *P, const float *X, const float *Y, long long n,
                                                      float inv_n, float *grad, float *loss) {
  extern __shared__ float sm[];
  float *sp = sm;                  // kParams
  float *sx = sp + kParams;        // kBB * kIn
  float *sdz1 = sx + kBB * kIn;    // kBB * kHid
  float *sh1 = sdz1 + kBB * kHid;  // kBB * kHid
  float *sdz2 = sh1 + kBB * kHid;  // kBB * kHid
  float *sh2 = sdz2 + kBB * kHid;  // kBB * kHid
  float *sd = sh2 + kBB * kHid;    // kBB
  float *sl = sd + kBB;            // kBB
  for (int k = threadIdx.x; k < kParams; k += kBB) sp[k] = P[k];
  const long long s0 = (long long)blockIdx.x * kBB;
  for (int k = threadIdx.x; k < kBB * kIn; k += kBB) {
    const long long s = s0 + k / kIn;
    sx[k] = s < n ? X[s0 * kIn + k] : 0.0f;
  }
  __syncthreads();
  const int t = threadIdx.x;
  const bool valid = s0 + t < n;
  float z1[kHid];
  const float *x = sx + t * kIn;
  for (int o = 0; o < kHid; ++o) {
    float z = sp[oB1 + o];
    for (int k = 0; k < kIn; ++k) z += sp[oW1 + o * kIn + k] * x[k];
    z1[o] = z;
    sh1[t * kHid + o] = gelu(z);
  }
  float z2[kHid];
  float logit = sp[oB3];
  for (int o = 0; o < kHid; ++o) {
    float z = sp[oB2 + o];
    for (int k = 0; k < kHid; ++k) z += sp[oW2 + o * kHid + k] * sh1[t * kHid + k];
    z2[o] = z;
    const float h = gelu(z);
    sh2[t * kHid + o] = h;
    logit += sp[oW3 + o] * h;
  }
  const float y = valid ? Y[s0 + t] : 0.0f;
  const float pr = 1.0f / (1.0f + expf(-logit));
  const float d = valid ? (pr - y) * inv_n : 0.0f;
  sd[t] = d;
  sl[t] = valid ? (fmaxf(logit, 0.0f) - logit * y + log1pf(expf(-fabsf(logit)))) * inv_n : 0.0f;
  for (int o = 0; o < kHid; ++o) sdz2[t * kHid + o] = d * sp[oW3 + o] * gelu_grad(z2[o]);
  for (int k = 0; k < kHid; ++k) {
    float dh = 0.0f;
    for (int o = 0; o < kHid; ++o) dh += sp[oW2 + o * kHid + k] * sdz2[t * kHid + o];
    sdz1[t * kHid + k] = dh * gelu_grad(z1[k]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kParams; e += kBB) {
    float acc = 0.0f;
    if (e < oB1) {
      const int o = e / kIn, k = e - (e / kIn) * kIn;
      for (int s = 0; s < kBB; ++s) acc += sdz1[s * kHid + o] * sx[s * kIn + k];
    } else if (e < oW2) {
      for (int s = 0; s < kBB; ++s) acc += sdz1[s * kHid + (e - oB1)];
    } else if (e < oB2) {
      const int o = (e - oW2) / kHid, k = (e - oW2) - o * kHid;
      for (int s = 0; s < kBB; ++s) acc += sdz2[s * kHid + o] * sh1[s * kHid + k];
    } else if (e < oW3) {
      for (int s = 0; s < kBB; ++s) acc += sdz2[s * kHid + (e - oB2)];
    } else if (e < oB3) {
      for (int s = 0; s < kBB; ++s) acc += sd[s] * sh2[s * kHid + (e - oW3)];
    } else {
      for (int s = 0; s < kBB; ++s) acc += sd[s];
    }
    atomicAdd(&grad[e], acc);
  }
  if (threadIdx.x == 0) {
    float l = 0.0f;
    for (int s = 0; s < kBB; ++s) l += sl[s];
    atomicAdd(loss, l);
  }
}

__global__ void k_adam(float *P, const float *G, float *M, float *V, int step, float lr) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float g = G[k];
  const float m = b1 * M[k] + (1.0f - b1) * g;
  const float v = b2 * V[k] + (1.0f - b2) * g * g;
  M[k] = m;
  V[k] = v;
  const float mh = m / (1.0f - powf(b1, float(step)));
  const float vh = v / (1.0f - powf(b2, float(step)));
  P[k] -= lr * mh / (sqrtf(vh) + eps);
}

// ------------------------------------------- tensor-core inference (tcgen05)
//
// One CTA of 128 threads runs tiles of 4 x 32 cells (x by y).  Per tile:
//   1. density and pressure of the 8 x 36 node patch around the tile -> smem;
//   2. each thread builds its cell's 50 features, writes them as BF16 into
//      A1 [128 x 64] (K padded with zeros) in the no-swizzle K-major layout:
//      8-row x 16-byte core matrices, K-adjacent cores 128 B apart (LBO),
//      8-row groups KC*128 B apart (SBO);
//   3. one thread issues 4 x tcgen05.mma (M=128, N=32, K=16, BF16 in, FP32
//      accumulate) D1 = A1 * W1^T into tensor memory columns [0, 32);
//   4. each warp reads its 32 rows back (tcgen05.ld 32x32b.x32), adds b1,
//      applies GELU, writes BF16 A2 [128 x 32];
//   5. 2 x tcgen05.mma D2 = A2 * W2^T into columns [32, 64);
//   6. read back, GELU, the 32 -> 1 layer on the CUDA cores, threshold ->
//      flag.
// MMA completion is signalled through an mbarrier (tcgen05.commit); every
// wait on it is bounded and on give-up the kernel records an error and
// stops issuing work, then releases its tensor memory.

constexpr int kTileI = 4, kTileJ = 32, kCells = kTileI * kTileJ;  // 128 = MMA M
constexpr int kPI = kTileI + 4, kPJ = kTileJ + 4;                   // node patch
constexpr int kK1 = 64, kK2 = 32;
constexpr unsigned kWaitLimit = 1u << 22;

struct IndicatorWeights {       // device buffer prepared by the host
  __nv_bfloat16 w1[kHid * kK1];  // canonical no-swizzle K-major layout
  __nv_bfloat16 w2[kHid * kK2];
  float b1[kHid], b2[kHid], w3[kHid], b3;
};

// element (row, k) of a K-major operand with KC = K/8 core columns
__device__ __forceinline__ int canon_off(int row, int k, int kc) {
  return ((row >> 3) * kc + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7);  // in elements (2 bytes)
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, LBO, SBO in 16-byte units, version
// 1 (bits 46-47), no swizzle.
__device__ __forceinline__ unsigned long long mdesc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFF) | ((unsigned long long)((lbo >> 4) & 0x3FFF) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulate (bits 4-5 = 1), A and B
// BF16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at
// bit 24.
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (unsigned(N >> 3) << 17) | (unsigned(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc,
                                         unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(unsigned mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned parity) {
  for (unsigned it = 0; it < kWaitLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
        " selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld32(unsigned taddr, float v[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__global__ void __launch_bounds__(kCells) k_indicator_tc(Geom g, const double *U, const IndicatorWeights *W,
                                                         float logit_threshold, unsigned char *flags, int flag_pitch,
                                                         int *error, const int *active) {
  if (active && *active == 0) return;
  __shared__ __align__(128) __nv_bfloat16 sA1[kCells * kK1];
  __shared__ __align__(128) __nv_bfloat16 sA2[kCells * kK2];
  __shared__ __align__(128) __nv_bfloat16 sB1[kHid * kK1];
  __shared__ __align__(128) __nv_bfloat16 sB2[kHid * kK2];
  __shared__ float sRho[kPI * kPJ], sPre[kPI * kPJ];
  __shared__ float sb1[kHid], sb2[kHid], sw3[kHid];
  __shared__ float sb3;
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ unsigned tmem_base_sh;
  __shared__ int abort_sh;

  const int tid = threadIdx.x, warp = tid >> 5;
  for (int k = tid; k < kHid * kK1; k += kCells) sB1[k] = W->w1[k];
  for (int k = tid; k < kHid * kK2; k += kCells) sB2[k] = W->w2[k];
  if (tid < kHid) {
    sb1[tid] = W->b1[tid];
    sb2[tid] = W->b2[tid];
    sw3[tid] = W->w3[tid];
  }
  if (tid == 0) {
    sb3 = W->b3;
    abort_sh = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&tmem_base_sh)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = tmem_base_sh;
  const unsigned mb = smem_u32(&mbar);
  const unsigned lane_base = unsigned(32 * warp) << 16;
  const float gam = float(g.gamma);
  const int tiles_j = (g.ny + kTileJ - 1) / kTileJ;
  const int ntiles = ((g.nx + kTileI - 1) / kTileI) * tiles_j;
  unsigned parity = 0;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int i0 = (tile / tiles_j) * kTileI, j0 = (tile % tiles_j) * kTileJ;
    // 1. node patch: nodes (i0-2 .. i0+5, j0-2 .. j0+33) of the interior index space
    for (int k = tid; k < kPI * kPJ; k += kCells) {
      const int pi = k / kPJ, pj = k - (k / kPJ) * kPJ;
      const int ei = kGhost + i0 - 2 + pi, ej = kGhost + j0 - 2 + pj;
      float r = 1.0f, p = 1.0f;
      if (ei < g.nxt && ej < g.nyt) {
        const long long b = (long long)ei * g.pitch + ej;
        r = dev::f64_to_f32(U[b]);
        p = pressure32(gam, r, dev::f64_to_f32(U[g.plane + b]), dev::f64_to_f32(U[2 * g.plane + b]),
                       dev::f64_to_f32(U[3 * g.plane + b]));
      }
      sRho[k] = r;
      sPre[k] = p;
    }
    __syncthreads();
    // 2. features of cell (i0 + warp, j0 + lane) -> row tid of A1
    {
      const int ci = warp, cj = tid & 31;
      float f[kK1];
      float w[25];
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) w[a * 5 + b] = sRho[(ci + a) * kPJ + cj + b];
      normalise(w, f);
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) w[a * 5 + b] = sPre[(ci + a) * kPJ + cj + b];
      normalise(w, f + 25);
#pragma unroll
      for (int k = 50; k < kK1; ++k) f[k] = 0.0f;
#pragma unroll
      for (int c = 0; c < kK1 / 8; ++c) {
        uint4 q;
        __nv_bfloat162 h0 = __floats2bfloat162_rn(f[8 * c + 0], f[8 * c + 1]);
        __nv_bfloat162 h1 = __floats2bfloat162_rn(f[8 * c + 2], f[8 * c + 3]);
        __nv_bfloat162 h2 = __floats2bfloat162_rn(f[8 * c + 4], f[8 * c + 5]);
        __nv_bfloat162 h3 = __floats2bfloat162_rn(f[8 * c + 6], f[8 * c + 7]);
        q.x = *reinterpret_cast<unsigned *>(&h0);
        q.y = *reinterpret_cast<unsigned *>(&h1);
        q.z = *reinterpret_cast<unsigned *>(&h2);
        q.w = *reinterpret_cast<unsigned *>(&h3);
        *reinterpret_cast<uint4 *>(&sA1[canon_off(tid, 8 * c, kK1 / 8)]) = q;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    // 3. layer 1 on the tensor cores
    if (tid == 0 && !abort_sh) {
      tc_fence_after();
      const unsigned a0 = smem_u32(sA1), b0 = smem_u32(sB1);
#pragma unroll
      for (int kk = 0; kk < kK1 / 16; ++kk)
        mma_bf16(tmem, mdesc(a0 + kk * 256, 128, (kK1 / 8) * 128), mdesc(b0 + kk * 256, 128, (kK1 / 8) * 128),
                 idesc_bf16(128, 32), kk > 0);
      mma_commit(mb);
    }
    if (!mbar_wait(mb, parity)) {
      atomicExch(error, 1);
      abort_sh = 1;
    }
    parity ^= 1u;
    tc_fence_after();
    // 4. epilogue 1
    {
      float z[32];
      tmem_ld32(tmem + lane_base, z);
#pragma unroll
      for (int c = 0; c < kK2 / 8; ++c) {
        uint4 q;
        unsigned *qq = reinterpret_cast<unsigned *>(&q);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int o = 8 * c + 2 * h;
          __nv_bfloat162 v = __floats2bfloat162_rn(gelu_fast(z[o] + sb1[o]), gelu_fast(z[o + 1] + sb1[o + 1]));
          qq[h] = *reinterpret_cast<unsigned *>(&v);
        }
        *reinterpret_cast<uint4 *>(&sA2[canon_off(tid, 8 * c, kK2 / 8)]) = q;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (abort_sh) break;
    // 5. layer 2
    if (tid == 0) {
      tc_fence_after();
      const unsigned a0 = smem_u32(sA2), b0 = smem_u32(sB2);
#pragma unroll
      for (int kk = 0; kk < kK2 / 16; ++kk)
        mma_bf16(tmem + 32, mdesc(a0 + kk * 256, 128, (kK2 / 8) * 128), mdesc(b0 + kk * 256, 128, (kK2 / 8) * 128),
                 idesc_bf16(128, 32), kk > 0);
      mma_commit(mb);
    }
    if (!mbar_wait(mb, parity)) {
      atomicExch(error, 1);
      abort_sh = 1;
    }
    parity ^= 1u;
    tc_fence_after();
    // 6. epilogue 2 and the output layer
    {
      float z[32];
      tmem_ld32(tmem + lane_base + 32, z);
      float logit = sb3;
#pragma unroll
      for (int o = 0; o < kHid; ++o) logit += sw3[o] * gelu_fast(z[o] + sb2[o]);
      const int i = i0 + warp, j = j0 + (tid & 31);
      if (i < g.nx && j < g.ny && !abort_sh)
        flags[(long long)(kGhost + i) * flag_pitch + (kGhost + j)] = logit > logit_threshold ? 1 : 0;
    }
    tc_fence_before();
    __syncthreads();
    if (abort_sh) break;
  }
  tc_fence_after();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

int grid_for(long long work, int threads, int cap) {
  long long b = (work + threads - 1) / threads;
  if (b > cap) b = cap;
  return int(b < 1 ? 1 : b);
}

}  // namespace lrn

size_t indicator_weights_bytes() { return sizeof(lrn::IndicatorWeights); }

// Host-side packing of FP32 parameters into the device weight block: BF16
// (round to nearest even) in the canonical layout, K of layer 1 padded to 64.
static unsigned short bf16_rne(float f) {
  unsigned u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (unsigned short)((u >> 16) | ((u & 0xffff) ? 0x40 : 0));
  u += 0x7fffu + ((u >> 16) & 1u);
  return (unsigned short)(u >> 16);
}

void pack_indicator_weights(const float *params, void *host_out) {
  lrn::IndicatorWeights *w = static_cast<lrn::IndicatorWeights *>(host_out);
  std::memset(w, 0, sizeof(*w));
  auto canon = [](int row, int k, int kc) { return ((row >> 3) * kc + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7); };
  for (int o = 0; o < lrn::kHid; ++o)
    for (int k = 0; k < lrn::kK1; ++k) {
      const float v = k < lrn::kIn ? params[lrn::oW1 + o * lrn::kIn + k] : 0.0f;
      const unsigned short b = bf16_rne(v);
      std::memcpy(&w->w1[canon(o, k, lrn::kK1 / 8)], &b, 2);
    }
  for (int o = 0; o < lrn::kHid; ++o)
    for (int k = 0; k < lrn::kK2; ++k) {
      const unsigned short b = bf16_rne(params[lrn::oW2 + o * lrn::kHid + k]);
      std::memcpy(&w->w2[canon(o, k, lrn::kK2 / 8)], &b, 2);
    }
  for (int o = 0; o < lrn::kHid; ++o) {
    w->b1[o] = params[lrn::oB1 + o];
    w->b2[o] = params[lrn::oB2 + o];
    w->w3[o] = params[lrn::oW3 + o];
  }
  w->b3 = params[lrn::oB3];
}

cudaError_t launch_features(const Geom &g, const double *U, float *feat, cudaStream_t s) {
  lrn::k_features<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, feat);
  return cudaGetLastError();
}

cudaError_t launch_labels(const Geom &g, const double *U, unsigned char *labels, cudaStream_t s) {
  lrn::k_labels<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, labels);
  return cudaGetLastError();
}

cudaError_t launch_indicator(const Geom &g, const double *U, const void *weights, float logit_threshold,
                             unsigned char *flags, int *error, const int *active, cudaStream_t s) {
  const int tiles = ((g.nx + lrn::kTileI - 1) / lrn::kTileI) * ((g.ny + lrn::kTileJ - 1) / lrn::kTileJ);
  const int grid = tiles < 152 * 8 ? tiles : 152 * 8;
  lrn::k_indicator_tc<<<grid, lrn::kCells, 0, s>>>(g, U, static_cast<const lrn::IndicatorWeights *>(weights),
                                                   logit_threshold, flags, g.pitch, error, active);
  return cudaGetLastError();
}

}  // namespace wenofd

// ------------------------------------------------------------- C ABI

extern "C" int wenofd_mlp_forward(const float *dev_params, const float *dev_x, long long n, float *dev_logits,
                                  void *stream) {
  if (!dev_params || !dev_x || !dev_logits || n < 0) return WENOFD_BAD_ARG;
  if (n == 0) return WENOFD_OK;
  wenofd::lrn::k_mlp_forward<<<wenofd::lrn::grid_for(n, 128, 152 * 16), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      dev_params, dev_x, n, dev_logits);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

extern "C" int wenofd_mlp_backward(const float *dev_params, const float *dev_x, const float *dev_y, long long n,
                                   float *dev_grad, float *dev_loss, void *stream) {
  using namespace wenofd::lrn;
  if (!dev_params || !dev_x || !dev_y || !dev_grad || !dev_loss || n <= 0) return WENOFD_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = sizeof(float) * (kParams + kBB * kIn + 4 * kBB * kHid + 2 * kBB);
  static bool configured = false;
  if (!configured) {
    if (cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
      return WENOFD_CUDA_ERROR;
    configured = true;
  }
  if (cudaMemsetAsync(dev_grad, 0, kParams * sizeof(float), s) != cudaSuccess ||
      cudaMemsetAsync(dev_loss, 0, sizeof(float), s) != cudaSuccess)
    return WENOFD_CUDA_ERROR;
  const long long blocks = (n + kBB - 1) / kBB;
  k_mlp_backward<<<int(blocks), kBB, smem, s>>>(dev_params, dev_x, dev_y, n, 1.0f / float(n), dev_grad, dev_loss);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

extern "C" int wenofd_mlp_adam(float *dev_params, const float *dev_grad, float *dev_m, float *dev_v, int step,
                               float lr, void *stream) {
  if (!dev_params || !dev_grad || !dev_m || !dev_v || step < 1) return WENOFD_BAD_ARG;
  wenofd::lrn::k_adam<<<(wenofd::lrn::kParams + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      dev_params, dev_grad, dev_m, dev_v, step, lr);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

// Training loop: per epoch a seeded shuffle of the mini-batch order, and per
// mini-batch one backward pass and one Adam step.  The epoch's mean loss is
// read back once per epoch.
extern "C" int wenofd_mlp_train(float *dev_params, const float *dev_x, const float *dev_y, long long n, int epochs,
                                int batch, float lr, unsigned long long seed, float *host_epoch_loss, void *stream) {
  using namespace wenofd::lrn;
  if (!dev_params || !dev_x || !dev_y || n <= 0 || epochs < 1 || batch < 1) return WENOFD_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float *buf = nullptr;  // grad | m | v | loss | epoch loss
  if (cudaMalloc(&buf, sizeof(float) * (3 * kParams + 2)) != cudaSuccess) return WENOFD_CUDA_ERROR;
  float *grad = buf, *m = buf + kParams, *v = buf + 2 * kParams, *loss = buf + 3 * kParams;
  int rc = WENOFD_OK;
  if (cudaMemsetAsync(m, 0, sizeof(float) * 2 * kParams, s) != cudaSuccess) rc = WENOFD_CUDA_ERROR;
  const long long nb = (n + batch - 1) / batch;
  std::vector<long long> order(nb);
  for (long long b = 0; b < nb; ++b) order[b] = b;
  unsigned long long st = seed ? seed : 0x9E3779B97F4A7C15ULL;
  int step = 0;
  for (int e = 0; e < epochs && rc == WENOFD_OK; ++e) {
    for (long long b = nb - 1; b > 0; --b) {  // Fisher-Yates with splitmix64
      unsigned long long z = (st += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      std::swap(order[b], order[z % (unsigned long long)(b + 1)]);
    }
    // the loss of every 16th mini-batch (and the last) estimates the epoch's mean
    double epoch_loss = 0.0;
    int sampled = 0;
    for (long long k = 0; k < nb && rc == WENOFD_OK; ++k) {
      const long long off = order[k] * batch;
      const long long cnt = off + batch <= n ? batch : n - off;
      rc = wenofd_mlp_backward(dev_params, dev_x + off * kIn, dev_y + off, cnt, grad, loss, stream);
      if (rc == WENOFD_OK) rc = wenofd_mlp_adam(dev_params, grad, m, v, ++step, lr, stream);
      if (rc == WENOFD_OK && host_epoch_loss && (k == nb - 1 || k % 16 == 0)) {
        float l = 0.0f;
        if (cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
          rc = WENOFD_CUDA_ERROR;
        epoch_loss += l;
        ++sampled;
      }
    }
    if (host_epoch_loss && sampled) host_epoch_loss[e] = float(epoch_loss / sampled);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = WENOFD_CUDA_ERROR;
  cudaFree(buf);
  return rc;
}
