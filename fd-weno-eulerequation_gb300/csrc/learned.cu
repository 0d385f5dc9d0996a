// Learned troubled-cell indicator: a per-cell MLP (50 -> 32 -> 32 -> 1, GELU,
// sigmoid) that decides which faces need characteristic WENO-Z and which can
// take the linear fifth-order upwind flux.  No counterpart in the reference;
// WENO-Z (include/Utility.hpp:457-504) is both its label source and its
// fallback.  Its training data (features, labels) is learned_data.cu.
//
//  - k_mlp_forward / k_mlp_backward / k_adam: FP32 training kernels;
//  - k_indicator_tc: inference on the 5th-generation tensor cores -- BF16
//    operands in shared memory, tcgen05.mma with FP32 accumulators in tensor
//    memory, tcgen05.ld for the epilogues -- writing one flag per cell.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wenofd.h"

#include "aux_device.cuh"
#include "guard.cuh"
#include "learned_common.cuh"
#include "trace.h"

namespace wenofd {
namespace lrn {

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
// them (and its loss share) to grad / loss with one atomic per entry, or,
// given `part`, writes them to its own row there for an ordered sum.
constexpr int kBB = 128;

// rows: with idx set, sample s of the mini-batch is row idx[s] of X and Y
// (rows of them in all).
__global__ void __launch_bounds__(kBB) k_mlp_backward(const float *P, const float *X, const float *Y, long long n,
                                                      float inv_n, float *grad, float *loss, float *part,
                                                      const long long *idx, long long rows,
                                                      unsigned long long *guard) {
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
    if (s >= n) sx[k] = 0.0f;
    else if (idx) sx[k] = X[WENOFD_IX(guard, idx[s], rows) * kIn + (k - (k / kIn) * kIn)];
    else sx[k] = X[s0 * kIn + k];
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
  const float y = valid ? Y[WENOFD_IX(guard, idx ? idx[s0 + t] : s0 + t, rows)] : 0.0f;
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
    if (part) part[(long long)blockIdx.x * (kParams + 1) + e] = acc;
    else atomicAdd(&grad[e], acc);
  }
  if (threadIdx.x == 0) {
    float l = 0.0f;
    for (int s = 0; s < kBB; ++s) l += sl[s];
    if (part) part[(long long)blockIdx.x * (kParams + 1) + kParams] = l;
    else atomicAdd(loss, l);
  }
}

// The blocks' partial gradients (and loss shares) summed in block order:
// the training loop's gradient does not depend on the order in which the
// blocks finished, so a training run is repeatable bit for bit.
__global__ void k_grad_reduce(const float *part, int blocks, float *grad, float *loss) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e > kParams) return;
  float acc = 0.0f;
  for (int b = 0; b < blocks; ++b) acc += part[(long long)b * (kParams + 1) + e];
  if (e < kParams) grad[e] = acc;
  else *loss = acc;
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
//   2. each thread builds its cell's 50 features and writes them as BF16
//      into A1 [128 x 64]: the 25 density features in columns 0..24, 1.0 in
//      columns 25 and 26 so that the bias of layer 1 (split into a BF16
//      high and low part, the same columns of W1) is added by the tensor
//      core, the 25 pressure features in columns 32..56, zeros elsewhere;
//      each window's features go out in 16-byte chunks as they are formed.
//      Operands use the no-swizzle K-major layout: 8-row x 16-byte core
//      matrices, K-adjacent cores 128 B apart (LBO), 8-row groups KC*128 B
//      apart (SBO);
//   3. one thread issues 4 x tcgen05.mma (M=128, N=32, K=16, BF16 in, FP32
//      accumulate): D1 = A1 * W1^T into tensor-memory columns [0, 32);
//   4. each warp reads its 32 rows back (tcgen05.ld 32x32b.x32), applies
//      GELU in packed BF16 pairs and writes A2 [128 x 48] (columns 32 and 33
//      are 1.0 for the bias of layer 2, the rest zero) over A1, which layer 1
//      has finished reading;
//   5. 3 x tcgen05.mma: D2 = A2 * W2^T into columns [32, 64);
//   6. read back, GELU, write the activations over A2;
//   7. 3 x tcgen05.mma (N = 16): D3 = A2 * W3^T into columns [0, 16), with
//      W3 row 0 = the output weights' BF16 high parts (and b3), row 1 their
//      low parts; logit = D3[0] + D3[1], compared with the threshold.
// MMA completion is signalled through an mbarrier (tcgen05.commit); every
// wait on it is bounded and on give-up the kernel records an error and
// stops issuing work, then releases its tensor memory.
//
// Occupancy: 27 KB of shared memory, at most 64 registers and 64 tensor-
// memory columns per CTA, so eight CTAs (32 warps) share an SM and its 512
// tensor-memory columns; their load, CUDA-core and tensor-core phases
// overlap.

constexpr int kTileI = 4, kTileJ = 32, kCells = kTileI * kTileJ;  // 128 = MMA M
constexpr int kPI = kTileI + 4, kPJ = kTileJ + 4;                   // node patch
constexpr int kK1 = 64, kK2 = 48, kN3 = 16;
constexpr unsigned kWaitLimit = 1u << 22;

constexpr int kColBias1 = 25, kColP = 32;  // A1 / W1 columns: bias 1 (hi, lo), first pressure feature

struct IndicatorWeights {  // device buffer prepared by the host (BF16, canonical layout)
  __nv_bfloat16 w1[kHid * kK1];  // [32 x 64]: W1 rho part | b1 hi | b1 lo | 0 | W1 p part | 0
  __nv_bfloat16 w2[kHid * kK2];  // [32 x 48]: W2 | b2 hi | b2 lo | 0
  __nv_bfloat16 w3[kN3 * kK2];   // [16 x 48]: row 0 w3 hi | b3 hi | b3 lo, row 1 w3 lo, rest 0
};

// element (row, k) of a K-major operand with KC = K/8 core columns
__host__ __device__ __forceinline__ int canon_off(int row, int k, int kc) {
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

// D[tmem_d] = A[128 x K] * B[N x K]^T, K a multiple of 16, both operands in
// the canonical layout with K/8 core columns.
template <int K, int N>
__device__ __forceinline__ void mma_layer(unsigned tmem_d, const void *A, const void *B) {
  const unsigned a0 = smem_u32(A), b0 = smem_u32(B);
#pragma unroll
  for (int kk = 0; kk < K / 16; ++kk)
    mma_bf16(tmem_d, mdesc(a0 + kk * 256, 128, (K / 8) * 128), mdesc(b0 + kk * 256, 128, (K / 8) * 128),
             idesc_bf16(128, N), kk > 0);
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

__device__ __forceinline__ void tmem_ld2(unsigned taddr, float v[2]) {
  unsigned r0, r1;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  v[0] = __uint_as_float(r0);
  v[1] = __uint_as_float(r1);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ unsigned bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<unsigned *>(&v); }
__device__ __forceinline__ __nv_bfloat162 bits_bf2(unsigned u) { return *reinterpret_cast<__nv_bfloat162 *>(&u); }

// Twice the GELU (tanh form) of two pre-activations in packed BF16
// arithmetic with the hardware tanh: z (1 + tanh(sqrt(2/pi) (z + 0.044715
// z^3))).  The factor 1/2 of GELU is folded into the next layer's BF16
// weights (pack_indicator_weights halves them, exactly), which gives the
// same MMA products as 0.5 z (1 + t) against unhalved weights and saves one
// packed multiply per pair.  The result is the next layer's BF16 operand,
// so BF16 intermediates lose nothing that the operand rounding keeps.
__device__ __forceinline__ unsigned gelu2_bf16x2(float z0, float z1) {
  const __nv_bfloat162 z = __floats2bfloat162_rn(z0, z1);
  const __nv_bfloat162 k1 = __float2bfloat162_rn(0.7978845608028654f);
  const __nv_bfloat162 k3 = __float2bfloat162_rn(0.7978845608028654f * 0.044715f);
  const __nv_bfloat162 u = __hmul2(z, __hfma2(__hmul2(z, z), k3, k1));
  unsigned t;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(bf2_bits(u)));
  return bf2_bits(__hfma2(z, bits_bf2(t), z));
}

// 2 x GELU of the 32 accumulator columns of this thread's row into columns
// 0..31 of A2 [128 x 48], and columns 32..47 = 1, 1, 0, ... (bias inputs).
// (rec: the guard record, bounds-checked build)
__device__ __forceinline__ void gelu_row_store(const float z[32], __nv_bfloat16 *A, int row,
                                               unsigned long long *rec) {
  constexpr int kc = kK2 / 8;
  constexpr long long n = kCells * kK2;  // elements of A2
  (void)n;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint4 q;
    q.x = gelu2_bf16x2(z[8 * c + 0], z[8 * c + 1]);
    q.y = gelu2_bf16x2(z[8 * c + 2], z[8 * c + 3]);
    q.z = gelu2_bf16x2(z[8 * c + 4], z[8 * c + 5]);
    q.w = gelu2_bf16x2(z[8 * c + 6], z[8 * c + 7]);
    *reinterpret_cast<uint4 *>(&A[WENOFD_SPAN(rec, canon_off(row, 8 * c, kc), canon_off(row, 8 * c, kc) + 7, n)]) = q;
  }
  *reinterpret_cast<uint4 *>(&A[WENOFD_SPAN(rec, canon_off(row, 32, kc), canon_off(row, 32, kc) + 7, n)]) =
      make_uint4(0x3F803F80u, 0u, 0u, 0u);  // two BF16 1.0
  *reinterpret_cast<uint4 *>(&A[WENOFD_SPAN(rec, canon_off(row, 40, kc), canon_off(row, 40, kc) + 7, n)]) =
      make_uint4(0u, 0u, 0u, 0u);
}

// Normalised 5x5 window (normalise() in learned_common.cuh, same arithmetic)
// written as BF16 into columns col0 .. col0+24 of row `row` of A1 in four
// 16-byte chunks; columns col0+25 .. col0+31 take `tail` (two values, then
// zeros).  Returns the window's range R = max |v - v_centre|.
__device__ __forceinline__ float window_store(const float w[25], __nv_bfloat16 *A, int row, int col0, float tail0,
                                              float tail1, unsigned long long *rec) {
  constexpr int kc = kK1 / 8;
  const float c = w[12];
  // differences and scaling on packed FP32 pairs (two operations per
  // instruction); a flat window scales by 0, which gives the GEMM the same
  // zero inputs as the explicit zeros of the training-side features
  float d[26];
#pragma unroll
  for (int k = 0; k < 24; k += 2) {
    const float2 q = __fadd2_rn(make_float2(w[k], w[k + 1]), make_float2(-c, -c));
    d[k] = q.x;
    d[k + 1] = q.y;
  }
  d[24] = w[24] - c;
  d[25] = 0.0f;
  float R = 0.0f;
#pragma unroll
  for (int k = 0; k < 25; ++k) R = fmaxf(R, fabsf(d[k]));
  const bool flat = R <= kFlat * (fabsf(c) + 1e-12f);
  const float inv = flat ? 0.0f : 1.0f / R;
#pragma unroll
  for (int k = 0; k < 26; k += 2) {
    const float2 q = __fmul2_rn(make_float2(d[k], d[k + 1]), make_float2(inv, inv));
    d[k] = q.x;
    d[k + 1] = q.y;
  }
  auto val = [&](int k) -> float {
    if (k < 25) return d[k];
    return k == 25 ? tail0 : (k == 26 ? tail1 : 0.0f);
  };
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    uint4 q;
    q.x = bf2_bits(__floats2bfloat162_rn(val(8 * ch + 0), val(8 * ch + 1)));
    q.y = bf2_bits(__floats2bfloat162_rn(val(8 * ch + 2), val(8 * ch + 3)));
    q.z = bf2_bits(__floats2bfloat162_rn(val(8 * ch + 4), val(8 * ch + 5)));
    q.w = bf2_bits(__floats2bfloat162_rn(val(8 * ch + 6), val(8 * ch + 7)));
    const int o = canon_off(row, col0 + 8 * ch, kc);
    *reinterpret_cast<uint4 *>(&A[WENOFD_SPAN(rec, o, o + 7, kCells * kK1)]) = q;
  }
  return R;
}

constexpr int kResident = 8;  // CTAs per SM: 28 KB shared memory, 64 registers, 64 TMEM columns each

// Shared memory of one indicator CTA: the BF16 operands and the node patch.
struct IndSmem {
  __nv_bfloat16 *A;                 // A1, then A2 [128 x 48] (and the layer-3 input)
  const __nv_bfloat16 *B1, *B2, *B3;  // the layers' weights
  float *rho, *pre;                 // the node patch ring
};

// Per-CTA tensor-core state: TMEM columns, the completion mbarrier and its
// phase, and whether a wait gave up.
struct IndTc {
  unsigned tmem, mb, parity;
  bool failed;
};

// One band of indicator tiles: tiles first .. last-1 (4 rows x 32 columns of
// cells each) down strip `strip` of the grid g, state U (ghosts filled),
// flags written at flags[(kGhost + i) * flag_pitch + kGhost + j].  With
// guard > 0 a cell is also flagged when the range of its density or pressure
// window exceeds guard times the centre value (INDICATOR_GUARD).  Every
// thread of the CTA calls it.  The node patch is a ring of 8 rows, node row
// i in slot i & 7: consecutive tiles of a band share 4 of their 8 patch
// rows, so every tile after the band's first loads 4 rows.  Returns false
// when a tensor-core wait gave up (recorded in *error); the CTA then stops.
__device__ __forceinline__ bool indicator_band(const Geom &g, const double *U, float logit_threshold, float guard,
                                               unsigned char *flags, int flag_pitch, int *error, int strip, int first,
                                               int last, const IndSmem &sm, IndTc &tc) {
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned lane_base = unsigned(32 * warp) << 16;
  const float gam = float(g.gamma);
  __nv_bfloat16 *const sA1 = sm.A, *const sA2 = sm.A;
  float *const sRho = sm.rho, *const sPre = sm.pre;
  static_assert(kPI == 2 * kTileI, "ring of two tiles' rows");

  // One layer: barrier (the operand writes are visible to the tensor core),
  // MMA issue by thread 0, completion wait by every thread.  A wait that
  // gives up marks this thread failed; the next barrier (a vote) turns that
  // into a uniform stop of the whole CTA.
  auto layer = [&](auto issue) -> bool {
    fence_async_smem();
    tc_fence_before();
    if (__syncthreads_or(tc.failed)) return false;
    if (tid == 0) {
      tc_fence_after();
      issue();
      mma_commit(tc.mb);
    }
    if (!mbar_wait(tc.mb, tc.parity)) {
      tc.failed = true;
      atomicExch(error, 1);
    }
    tc.parity ^= 1u;
    tc_fence_after();
    return true;
  };

  for (int ti = first; ti < last; ++ti) {
    const int i0 = ti * kTileI, j0 = strip * kTileJ;
    const int row0 = ti > first ? kPI - kTileI : 0;  // first patch row to load
    // 1. node patch rows row0..7: nodes (i0-2+row, j0-2 .. j0+33) of the
    // interior index space, into ring slot (i0-2+row) & 7; every load of a
    // thread is issued before any is used
    {
      constexpr int NP = (kPI * kPJ + kCells - 1) / kCells;
      const int count = (kPI - row0) * kPJ;
      double v[NP][4];
      bool ok[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int k = tid + q * kCells;
        const int pi = row0 + k / kPJ, pj = k - (k / kPJ) * kPJ;
        const int ei = kGhost + i0 - 2 + pi, ej = kGhost + j0 - 2 + pj;
        ok[q] = k < count && ei < g.nxt && ej < g.nyt;
        const double *src = U + WENOFD_GNODE_IF(g, ok[q], ei, ej);
#pragma unroll
        for (int r = 0; r < 4; ++r) v[q][r] = ok[q] ? __ldg(src + r * g.plane) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int k = tid + q * kCells;
        if (k < count) {
          const int pi = row0 + k / kPJ, pj = k - (k / kPJ) * kPJ;
          float r = 1.0f, p = 1.0f;
          if (ok[q]) {
            r = dev::f64_to_f32(v[q][0]);
            p = pressure32(gam, r, dev::f64_to_f32(v[q][1]), dev::f64_to_f32(v[q][2]), dev::f64_to_f32(v[q][3]));
          }
          const int slot = WENOFD_IX(g.guard, ((i0 - 2 + pi) & (kPI - 1)) * kPJ + pj, kPI * kPJ);
          sRho[slot] = r;
          sPre[slot] = p;
        }
      }
    }
    __syncthreads();
    // 2. features of cell (i0 + warp, j0 + lane) -> row tid of A1
    bool guarded = false;
    {
      const int ci = warp, cj = tid & 31;
      int rows[5];  // ring slots of node rows i0 + ci - 2 .. i0 + ci + 2
#pragma unroll
      for (int a = 0; a < 5; ++a) rows[a] = ((i0 + ci - 2 + a) & (kPI - 1)) * kPJ + cj;
      float w[25];
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) w[a * 5 + b] = sRho[WENOFD_IX(g.guard, rows[a] + b, kPI * kPJ)];
      const float Rr = window_store(w, sA1, tid, 0, 1.0f, 1.0f, g.guard);  // columns 25, 26: bias inputs
      guarded = guard > 0.0f && Rr > guard * fabsf(w[12]);
#pragma unroll
      for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) w[a * 5 + b] = sPre[WENOFD_IX(g.guard, rows[a] + b, kPI * kPJ)];
      const float Rp = window_store(w, sA1, tid, kColP, 0.0f, 0.0f, g.guard);
      guarded = guarded || (guard > 0.0f && Rp > guard * fabsf(w[12]));
    }
    // 3. layer 1 (bias included)
    if (!layer([&] { mma_layer<kK1, kHid>(tc.tmem, sA1, sm.B1); })) return false;
    // 4. GELU -> A2
    {
      float z[32];
      tmem_ld32(tc.tmem + lane_base, z);
      gelu_row_store(z, sA2, tid, g.guard);
    }
    // 5. layer 2
    if (!layer([&] { mma_layer<kK2, kHid>(tc.tmem + 32, sA2, sm.B2); })) return false;
    // 6. GELU -> A2 (layer 2 has read it)
    {
      float z[32];
      tmem_ld32(tc.tmem + lane_base + 32, z);
      gelu_row_store(z, sA2, tid, g.guard);
    }
    // 7. output layer on the tensor cores, into the columns of D1
    if (!layer([&] { mma_layer<kK2, kN3>(tc.tmem, sA2, sm.B3); })) return false;
    {
      float d[2];
      tmem_ld2(tc.tmem + lane_base, d);
      const float logit = d[0] + d[1];
      const int i = i0 + warp, j = j0 + (tid & 31);
      if (i < g.nx && j < g.ny && !tc.failed)
        flags[WENOFD_IX(g.guard, (long long)(kGhost + i) * flag_pitch + (kGhost + j), (long long)g.nxt * flag_pitch)] =
            (logit > logit_threshold || guarded) ? 1 : 0;
    }
    tc_fence_before();
    if (__syncthreads_or(tc.failed)) return false;
  }
  return true;
}

// Copies the packed weights into the CTA's operand buffers (all threads).
__device__ __forceinline__ void load_weights(const IndicatorWeights *W, __nv_bfloat16 *B1, __nv_bfloat16 *B2,
                                             __nv_bfloat16 *B3) {
  for (int k = threadIdx.x; k < kHid * kK1; k += kCells) B1[k] = W->w1[k];
  for (int k = threadIdx.x; k < kHid * kK2; k += kCells) B2[k] = W->w2[k];
  for (int k = threadIdx.x; k < kN3 * kK2; k += kCells) B3[k] = W->w3[k];
}

// CTA set-up: the completion mbarrier and 64 tensor-memory columns.
__device__ __forceinline__ IndTc indicator_open(unsigned long long *mbar, unsigned *tmem_base_sh) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tmem_base_sh)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  IndTc tc;
  tc.tmem = *tmem_base_sh;
  tc.mb = smem_u32(mbar);
  tc.parity = 0;
  tc.failed = false;
  return tc;
}

// CTA tear-down: the tensor memory is released (after every MMA completed
// or the CTA stopped).
__device__ __forceinline__ void indicator_close(const IndTc &tc) {
  tc_fence_after();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tc.tmem));
}

__global__ void __launch_bounds__(kCells, kResident) k_indicator_tc(Geom g, const double *U, const IndicatorWeights *W,
                                                            float logit_threshold, float guard, unsigned char *flags,
                                                            int flag_pitch, int *error, const int *active,
                                                            const Ctrl *ctrl, int interval) {
  if (active && *active == 0) return;
  if (ctrl && interval > 1 && (ctrl->steps - ctrl->ind_base) % interval != 0) return;
  __shared__ __align__(128) __nv_bfloat16 sA[kCells * kK1];
  __shared__ __align__(128) __nv_bfloat16 sB1[kHid * kK1];
  __shared__ __align__(128) __nv_bfloat16 sB2[kHid * kK2];
  __shared__ __align__(128) __nv_bfloat16 sB3[kN3 * kK2];
  __shared__ float sRho[kPI * kPJ], sPre[kPI * kPJ];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ unsigned tmem_base_sh;

  load_weights(W, sB1, sB2, sB3);
  IndTc tc = indicator_open(&mbar, &tmem_base_sh);
  // CTA b walks one band of rows down one strip (a strip = 32 columns, tiles
  // of 4 rows each): strip b % tiles_j, band b / tiles_j of the grid's
  // gridDim.x / tiles_j bands.  CTAs of neighbouring strips and the same band
  // start at the same row and move down together, so the patch columns they
  // share are read from L2 while both need them.
  const int tiles_i = (g.nx + kTileI - 1) / kTileI;
  const int tiles_j = (g.ny + kTileJ - 1) / kTileJ;
  const int bands = int(gridDim.x) / tiles_j;
  const int strip = int(blockIdx.x) % tiles_j, band = int(blockIdx.x) / tiles_j;
  const int first = int((long long)tiles_i * band / bands), last = int((long long)tiles_i * (band + 1) / bands);
  const IndSmem sm{sA, sB1, sB2, sB3, sRho, sPre};
  indicator_band(g, U, logit_threshold, guard, flags, flag_pitch, error, strip, first, last, sm, tc);
  indicator_close(tc);
}

// The indicator runs of a learned batch (launch_indicator_batch).  Work item
// = (member, strip, band): the member from the prefix array, then strip =
// local % tiles_j and band = local / tiles_j of the member's ind_bands bands
// (its tiles split evenly among them).  A CTA claims items from *counter
// until none is left, skips members that cannot step or have no weights,
// and reloads the weights only when the member's weights differ from the
// ones it holds.
__global__ void __launch_bounds__(kCells, kResident)
    k_indicator_batch(const BatchMember *members, const int *prefix, int n, unsigned *counter, int *error,
                      unsigned long long *guard) {
  __shared__ __align__(128) __nv_bfloat16 sA[kCells * kK1];
  __shared__ __align__(128) __nv_bfloat16 sB1[kHid * kK1];
  __shared__ __align__(128) __nv_bfloat16 sB2[kHid * kK2];
  __shared__ __align__(128) __nv_bfloat16 sB3[kN3 * kK2];
  __shared__ float sRho[kPI * kPJ], sPre[kPI * kPJ];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ unsigned tmem_base_sh;
  __shared__ int s_item, s_m, s_on;
  __shared__ BatchMember sM;  // the record of the member whose items run

  IndTc tc = indicator_open(&mbar, &tmem_base_sh);
  const IndSmem sm{sA, sB1, sB2, sB3, sRho, sPre};
  const int total = __ldg(&prefix[n]);
  int cur = -1;                  // member staged in sM
  const void *loaded = nullptr;  // weights now in sB1..sB3
  for (;;) {
    __syncthreads();  // every thread has read the last claim and sM
    if (threadIdx.x == 0) {
      const int item = int(atomicAdd(counter, 1u));
      s_item = item;
      if (item < total) {
        const int m = WENOFD_IX(guard, dev::owner(prefix, n, item), n);
        s_m = m;
        const BatchMember *M = members + m;
        s_on = M->ind_weights != nullptr && *(volatile const int *)&M->ctrl->active != 0;
      }
    }
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    if (!s_on) continue;  // block-uniform: the member cannot step or has no weights
    const int m = s_m;
    if (m != cur) {  // block-uniform: stage the member record
      const unsigned *src = reinterpret_cast<const unsigned *>(members + m);
      unsigned *dst = reinterpret_cast<unsigned *>(&sM);
      for (int w = threadIdx.x; w < int(sizeof(BatchMember) / 4); w += kCells) dst[w] = __ldg(&src[w]);
      __syncthreads();
      cur = m;
      if (sM.ind_weights != loaded) {
        // every MMA that read the old weights has completed (each layer waits)
        load_weights(static_cast<const IndicatorWeights *>(sM.ind_weights), sB1, sB2, sB3);
        loaded = sM.ind_weights;
      }
    }
    const Geom &g = sM.g;
    const int tiles_i = (g.nx + kTileI - 1) / kTileI;
    const int tiles_j = (g.ny + kTileJ - 1) / kTileJ;
    const int bands = sM.ind_bands;
    const int local = item - __ldg(&prefix[m]);
    const int strip = local % tiles_j, band = local / tiles_j;
    const int first = int((long long)tiles_i * band / bands), last = int((long long)tiles_i * (band + 1) / bands);
    if (!indicator_band(g, sM.S, sM.ind_logit_threshold, sM.ind_guard, sM.flags, g.pitch, error, strip, first, last,
                        sm, tc))
      break;
  }
  indicator_close(tc);
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
  using namespace lrn;
  IndicatorWeights *w = static_cast<IndicatorWeights *>(host_out);
  std::memset(w, 0, sizeof(*w));
  auto put = [](__nv_bfloat16 *M, int row, int k, int kc, float v) {
    const unsigned short b = bf16_rne(v);
    std::memcpy(&M[canon_off(row, k, kc)], &b, 2);
  };
  // v = hi + lo with hi, lo in BF16 (about 16 significant bits together)
  auto hi_lo = [](float v, float &hi, float &lo) {
    const unsigned short h = bf16_rne(v);
    const unsigned u = unsigned(h) << 16;
    std::memcpy(&hi, &u, 4);
    lo = v - hi;
  };
  float hi, lo;
  for (int o = 0; o < kHid; ++o) {
    for (int k = 0; k < kIn; ++k)  // density features 0..24 -> columns 0..24, pressure 25..49 -> 32..56
      put(w->w1, o, k < 25 ? k : kColP + (k - 25), kK1 / 8, params[oW1 + o * kIn + k]);
    hi_lo(params[oB1 + o], hi, lo);
    put(w->w1, o, kColBias1, kK1 / 8, hi);
    put(w->w1, o, kColBias1 + 1, kK1 / 8, lo);
    // layers 2 and 3 take 2 x GELU (gelu2_bf16x2): their weights on it are
    // halved here, exactly (a power of two); their bias columns are not
    for (int k = 0; k < kHid; ++k) put(w->w2, o, k, kK2 / 8, 0.5f * params[oW2 + o * kHid + k]);
    hi_lo(params[oB2 + o], hi, lo);
    put(w->w2, o, kHid, kK2 / 8, hi);
    put(w->w2, o, kHid + 1, kK2 / 8, lo);
    hi_lo(params[oW3 + o], hi, lo);
    put(w->w3, 0, o, kK2 / 8, 0.5f * hi);
    put(w->w3, 1, o, kK2 / 8, 0.5f * lo);
  }
  hi_lo(params[oB3], hi, lo);
  put(w->w3, 0, kHid, kK2 / 8, hi);
  put(w->w3, 0, kHid + 1, kK2 / 8, lo);
}

cudaError_t launch_indicator(const Geom &g, const double *U, const void *weights, float logit_threshold, float guard,
                             unsigned char *flags, int *error, const int *active, const Ctrl *ctrl, int interval,
                             cudaStream_t s) {
  const int tiles_i = (g.nx + lrn::kTileI - 1) / lrn::kTileI, tiles_j = (g.ny + lrn::kTileJ - 1) / lrn::kTileJ;
  // CTAs: one per (strip, band of rows); as many bands as let every CTA be
  // resident at once (kResident per SM, the kernel's launch bound, which its
  // shared memory, registers and tensor memory meet), at least one
  static int sms_of[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int &sms = sms_of[dev & 63];
  if (sms == 0 && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  int bands = (sms * lrn::kResident) / tiles_j;
  bands = bands < 1 ? 1 : (bands > tiles_i ? tiles_i : bands);
  const int grid = tiles_j * bands;
  lrn::k_indicator_tc<<<grid, lrn::kCells, 0, s>>>(g, U, static_cast<const lrn::IndicatorWeights *>(weights),
                                                   logit_threshold, guard, flags, g.pitch, error, active, ctrl,
                                                   interval);
  return cudaGetLastError();
}

cudaError_t launch_indicator_batch(const BatchMember *members, const int *ind_prefix, int n, unsigned *counter,
                                   int *error, unsigned long long *guard, int items, cudaStream_t s) {
  static int sms_of[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int &sms = sms_of[dev & 63];
  if (sms == 0 && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  // every CTA resident at once; no more CTAs than work items
  const int grid = std::max(1, std::min(items, sms * lrn::kResident));
  lrn::k_indicator_batch<<<grid, lrn::kCells, 0, s>>>(members, ind_prefix, n, counter, error, guard);
  return cudaGetLastError();
}

}  // namespace wenofd

// ------------------------------------------------------------- C ABI

namespace wenofd {
void set_last_error(const std::string &msg);  // capi.cpp: the text wenofd_last_error() returns
}

// He-uniform initial parameters from a seeded splitmix64 sequence: W1 from
// U(-1, 1) * sqrt(6 / 50), W2 and w3 from U(-1, 1) * sqrt(6 / 32), biases 0.
// Host only; the same seed gives the same parameters on any machine.
extern "C" int wenofd_mlp_init(float *host_params, unsigned long long seed) {
  if (!host_params) {
    wenofd::set_last_error("null parameter buffer");
    return WENOFD_BAD_ARG;
  }
  unsigned long long st = seed;
  auto uniform = [&st]() {  // in [-1, 1)
    unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return 2.0 * double(z >> 11) * (1.0 / 9007199254740992.0) - 1.0;
  };
  for (int k = 0; k < wenofd::lrn::kParams; ++k) host_params[k] = 0.0f;
  const double s1 = std::sqrt(6.0 / 50.0), s2 = std::sqrt(6.0 / 32.0);
  for (int k = 0; k < wenofd::lrn::oB1; ++k) host_params[wenofd::lrn::oW1 + k] = float(uniform() * s1);
  for (int k = 0; k < wenofd::lrn::oB2 - wenofd::lrn::oW2; ++k) host_params[wenofd::lrn::oW2 + k] = float(uniform() * s2);
  for (int k = 0; k < wenofd::lrn::oB3 - wenofd::lrn::oW3; ++k) host_params[wenofd::lrn::oW3 + k] = float(uniform() * s2);
  return WENOFD_OK;
}

extern "C" int wenofd_mlp_forward(const float *dev_params, const float *dev_x, long long n, float *dev_logits,
                                  void *stream) {
  if (!dev_params || !dev_x || !dev_logits || n < 0) return WENOFD_BAD_ARG;
  if (n == 0) return WENOFD_OK;
  wenofd::lrn::k_mlp_forward<<<wenofd::lrn::grid_for(n, 128, 152 * 16), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      dev_params, dev_x, n, dev_logits);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

namespace {

// One backward pass over n samples: with part null the blocks add their
// gradients into grad / loss with atomics (after zeroing them); with part
// (room for one row of kParams + 1 floats per block) they write partials and
// k_grad_reduce sums them in block order.
// (rows: the rows of x and y that idx indexes)
int launch_backward(const float *params, const float *x, const float *y, long long n, float *grad, float *loss,
                    float *part, cudaStream_t s, const long long *idx = nullptr, long long rows = 0) {
  using namespace wenofd::lrn;
  const size_t smem = sizeof(float) * (kParams + kBB * kIn + 4 * kBB * kHid + 2 * kBB);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WENOFD_CUDA_ERROR;
  static unsigned long long configured = 0;  // one bit per device
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    if (cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
      return WENOFD_CUDA_ERROR;
    configured |= bit;
  }
  const long long blocks = (n + kBB - 1) / kBB;
  if (!part && (cudaMemsetAsync(grad, 0, kParams * sizeof(float), s) != cudaSuccess ||
                cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess))
    return WENOFD_CUDA_ERROR;
  k_mlp_backward<<<int(blocks), kBB, smem, s>>>(params, x, y, n, 1.0f / float(n), grad, loss, part, idx,
                                                idx ? rows : n, wenofd::guard_record());
  if (part) k_grad_reduce<<<(kParams + 1 + 255) / 256, 256, 0, s>>>(part, int(blocks), grad, loss);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

}  // namespace

extern "C" int wenofd_mlp_backward(const float *dev_params, const float *dev_x, const float *dev_y, long long n,
                                   float *dev_grad, float *dev_loss, void *stream) {
  if (!dev_params || !dev_x || !dev_y || !dev_grad || !dev_loss || n <= 0) return WENOFD_BAD_ARG;
  return launch_backward(dev_params, dev_x, dev_y, n, dev_grad, dev_loss, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int wenofd_mlp_adam(float *dev_params, const float *dev_grad, float *dev_m, float *dev_v, int step,
                               float lr, void *stream) {
  if (!dev_params || !dev_grad || !dev_m || !dev_v || step < 1) return WENOFD_BAD_ARG;
  wenofd::lrn::k_adam<<<(wenofd::lrn::kParams + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      dev_params, dev_grad, dev_m, dev_v, step, lr);
  return cudaGetLastError() == cudaSuccess ? WENOFD_OK : WENOFD_CUDA_ERROR;
}

// Training loop: per epoch a seeded permutation of the samples (so the data
// may come in any order, e.g. grouped by snapshot and node), cut into
// mini-batches, and per mini-batch one backward pass and one Adam step.  The
// epoch's mean loss is estimated from every 16th mini-batch's loss.  Each
// mini-batch's gradient is summed in block order (k_grad_reduce), so the same
// data and seed give the same parameters bit for bit.
extern "C" int wenofd_mlp_train(float *dev_params, const float *dev_x, const float *dev_y, long long n, int epochs,
                                int batch, float lr, unsigned long long seed, float *host_epoch_loss, void *stream) {
  WENOFD_TRACE("wenofd_mlp_train");
  using namespace wenofd::lrn;
  if (!dev_params || !dev_x || !dev_y || n <= 0 || epochs < 1 || batch < 1) return WENOFD_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // grad | m | v | loss | epoch loss | the backward blocks' partial rows
  const long long part_rows = (std::min<long long>(batch, n) + kBB - 1) / kBB;
  float *buf = nullptr;
  long long *perm_dev = nullptr;
  if (cudaMalloc(&buf, sizeof(float) * (3 * kParams + 2 + part_rows * (kParams + 1))) != cudaSuccess)
    return WENOFD_CUDA_ERROR;
  if (cudaMalloc(&perm_dev, sizeof(long long) * size_t(n)) != cudaSuccess) {
    cudaFree(buf);
    return WENOFD_CUDA_ERROR;
  }
  float *grad = buf, *m = buf + kParams, *v = buf + 2 * kParams, *loss = buf + 3 * kParams;
  float *part = buf + 3 * kParams + 2;
  int rc = WENOFD_OK;
  if (cudaMemsetAsync(m, 0, sizeof(float) * 2 * kParams, s) != cudaSuccess) rc = WENOFD_CUDA_ERROR;
  const long long nb = (n + batch - 1) / batch;
  std::vector<long long> perm(n);
  for (long long r = 0; r < n; ++r) perm[r] = r;
  unsigned long long st = seed ? seed : 0x9E3779B97F4A7C15ULL;
  int step = 0;
  for (int e = 0; e < epochs && rc == WENOFD_OK; ++e) {
    for (long long r = n - 1; r > 0; --r) {  // Fisher-Yates with splitmix64
      unsigned long long z = (st += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      std::swap(perm[r], perm[z % (unsigned long long)(r + 1)]);
    }
    // the previous epoch's mini-batches read the permutation buffer: copy
    // after they ran (same stream; the copy from pageable memory returns
    // once the host buffer is staged)
    if (cudaMemcpyAsync(perm_dev, perm.data(), sizeof(long long) * size_t(n), cudaMemcpyHostToDevice, s) !=
        cudaSuccess)
      rc = WENOFD_CUDA_ERROR;
    // the loss of every 16th mini-batch (and the last) estimates the epoch's mean
    double epoch_loss = 0.0;
    int sampled = 0;
    for (long long k = 0; k < nb && rc == WENOFD_OK; ++k) {
      const long long off = k * batch;
      const long long cnt = off + batch <= n ? batch : n - off;
      rc = launch_backward(dev_params, dev_x, dev_y, cnt, grad, loss, part, s, perm_dev + off, n);
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
  cudaFree(perm_dev);
  return rc;
}
