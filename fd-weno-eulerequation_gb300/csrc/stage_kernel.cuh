// One RK stage of the WENO-FD hot path as a single fused tile kernel:
// halo load, x sweep (flux split, characteristic WENO faces), y sweep, flux
// differences, source term and the RK combination, with nothing but the
// state in global memory.
//
// Replaces, per stage: assembleRHS (src/WENOFD.cpp:454-465) with
// assembleBoundaryTerm's x sweep (513-649) and y sweep (652-797),
// assembleSourceTerm (800-821), and the stage update of RunRK1/2/3
// (301-396).  The boundary fill runs before it (k_bc_fill).
//
// Tile: TI nodes in x by TJ = 32 nodes in y (y is the contiguous axis, so a
// warp spans one tile row).  The block stages the state of the tile plus a
// 3-node halo in shared memory, computes the split fluxes of every node the
// tile's faces need once, then the (TI+1) x TJ x-faces and TI x (TJ+1)
// y-faces, and keeps the per-node x term in registers between the sweeps.
// Shared-memory regions for the split fluxes and face fluxes are reused by
// the y sweep.
//
// This file holds the FP64 tile (bitwise the reference) and the kernel and
// launcher shared by both precisions; the FP32 tile (FP32 form and learned
// form) is stage_f32.cuh.
#pragma once

#include "convert.cuh"
#include "physics.cuh"
#include "stage_f32.cuh"

namespace wenofd {
namespace dev {

// Shared memory of the FP64 tile, structure of arrays [component][row][col].
// The state tile's rows are kBoxJ = 40 doubles wide, halo node hj at column
// hj + 1: the TMA box of the per-solve kernel (40 columns from the even,
// 16-byte aligned column before the halo, TI + 6 rows, 4 planes) lands in
// place, with no copy; the batched kernel's per-thread loads use the same
// layout.
template <int TI, int TJ>
struct StageSmem {
  static constexpr int HI = TI + 6, HJ = TJ + 6;
  static constexpr int kBoxJ = 40;
  static_assert(HJ + 2 <= kBoxJ, "box width");
  static constexpr int kU = 4 * HI * kBoxJ;                                 // state + halo
  static constexpr unsigned kBoxBytes = unsigned(kU) * 8u;
  static constexpr int kSplit = 4 * (HI * TJ > TI * HJ ? HI * TJ : TI * HJ);  // one of F+, F-
  static constexpr int kFace = 4 * ((TI + 1) * TJ > TI * (TJ + 1) ? (TI + 1) * TJ : TI * (TJ + 1));
  // 128 bytes of slack: the base is rounded up to 128 bytes (TMA destination)
  static constexpr size_t bytes = 128 + sizeof(double) * (size_t(kU) + 2 * kSplit + kFace);
  // index of state component r at halo node (hi, hj)
  static __device__ __forceinline__ int u(int r, int hi, int hj) { return (r * HI + hi) * kBoxJ + hj + 1; }
};

// One FP64 tile (TI x TJ interior nodes starting at i0, j0) of one RK stage,
// executed by all NT threads of a block; smem_raw holds StageSmem::bytes.
// Every operation follows the reference's evaluation order (the unit is
// compiled with -fmad=false).  Shared by the per-solve kernel k_stage and
// the persistent batched kernel.  COH: the tile's inputs may have been
// written earlier in the same kernel by other blocks (the persistent batched
// kernel): loads then go through L2 only (ld.global.cg) instead of the
// non-coherent read-only path.  TMA (the per-solve kernel): the halo box
// arrives by TMA through the map in `tma` (one thread issues it; a bounded
// wait, on give-up the block records the error in a.wait_error and leaves
// the tile); otherwise every thread loads nodes.
template <int SCHEME, int TI, int TJ, int NT, bool COH = false, bool TMA = false>
__device__ __forceinline__ void stage_tile_f64(const Geom &g, const StageArgs &a, const int i0, const int j0,
                                               unsigned char *smem_raw, const StageTma *tma = nullptr) {
  using T = double;
  using S = StageSmem<TI, TJ>;
  constexpr int HI = S::HI, HJ = S::HJ;
  unsigned char *base = smem_raw + (((tma_smem_addr(smem_raw) + 127u) & ~127u) - tma_smem_addr(smem_raw));
  T *Us = reinterpret_cast<T *>(base);
  T *Fp = Us + S::kU;
  T *Fm = Fp + S::kSplit;
  T *Hf = Fm + S::kSplit;
  const T gamma = g.gamma, zpl = g.zp_lambda;

  // --- state tile with halo: nodes ei = 4+i0-3+hi, ej = 4+j0-3+hj.
  if constexpr (TMA) {
    // box column c = ghosted column j0 + c = halo node hj = c - 1; box row 0 =
    // ghosted row 1 + i0 (rows or columns past the array read as zero, like
    // the per-thread loads, and feed only faces that are not computed)
    __shared__ __align__(8) unsigned long long tma_bar;
    if (threadIdx.x == 0) tma_bar_init(tma_smem_addr(&tma_bar), 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned bar = tma_smem_addr(&tma_bar);
      tma_fence_proxy();
      tma_bar_expect(bar, S::kBoxBytes);
      // first coordinate x * 8 bytes a multiple of 16 (j0 is a multiple of
      // 32; an unissued copy leaves the wait below to give up)
      if (WENOFD_REQUIRE(g.guard, (j0 & 1) == 0, j0, 2)) tma_load_3d(tma_smem_addr(Us), &tma->u, j0, 1 + i0, 0, bar);
    }
    const bool ok = tma_bar_wait(tma_smem_addr(&tma_bar), 0, kTmaWaitLimit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        if (a.wait_error) atomicExch(a.wait_error, 1);
        tma_bar_wait(tma_smem_addr(&tma_bar), 0, kTmaWaitLimit);
      }
      __syncthreads();
      return;
    }
  } else {
    // All of a thread's loads are issued before any is used, so they are in
    // flight together.
    constexpr int NLD = (4 * HI * HJ + NT - 1) / NT;
    double v[NLD];
#pragma unroll
    for (int k = 0; k < NLD; ++k) {
      const int t = threadIdx.x + k * NT;
      const int r = t / (HI * HJ);
      const int rem = t - r * (HI * HJ);
      const int hi = rem / HJ, hj = rem - hi * HJ;
      const int ei = 1 + i0 + hi, ej = 1 + j0 + hj;
      const bool ok = t < 4 * HI * HJ && ei < g.nxt && ej < g.nyt;
      if constexpr (COH) v[k] = ok ? __ldcg(&a.uin[WENOFD_STATE(g, r * g.plane + WENOFD_GNODE(g, ei, ej))]) : 0.0;
      else v[k] = ok ? __ldg(&a.uin[WENOFD_STATE(g, r * g.plane + WENOFD_GNODE(g, ei, ej))]) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < NLD; ++k) {
      const int t = threadIdx.x + k * NT;
      if (t < 4 * HI * HJ) {
        const int r = t / (HI * HJ);
        const int rem = t - r * (HI * HJ);
        const int hi = rem / HJ, hj = rem - hi * HJ;
        Us[WENOFD_IX(g.guard, S::u(r, hi, hj), S::kU)] = v[k];
      }
    }
  }
  __syncthreads();

  // --- x sweep: split fluxes of halo rows 0..HI-1, columns 3..3+TJ
  for (int t = threadIdx.x; t < HI * TJ; t += NT) {
    const int hi = t / TJ, j = t - hi * TJ;
    T q[4], fm[4], fp[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) q[r] = Us[WENOFD_IX(g.guard, S::u(r, hi, j + 3), S::kU)];
    flux_split<T, 0>(gamma, q, fm, fp);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      Fp[WENOFD_IX(g.guard, (r * HI + hi) * TJ + j, S::kSplit)] = fp[r];
      Fm[WENOFD_IX(g.guard, (r * HI + hi) * TJ + j, S::kSplit)] = fm[r];
    }
  }
  __syncthreads();
  // x faces f = 0..TI: face between tile nodes f-1 and f (halo rows f+2, f+3)
  for (int t = threadIdx.x; t < (TI + 1) * TJ; t += NT) {
    const int f = t / TJ, j = t - f * TJ;
    if (i0 + f > g.nx || j0 + j >= g.ny) continue;
    T um[4], u0[4], out[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      um[r] = Us[WENOFD_IX(g.guard, S::u(r, f + 2, j + 3), S::kU)];
      u0[r] = Us[WENOFD_IX(g.guard, S::u(r, f + 3, j + 3), S::kU)];
    }
    // stencils: nodes 0..4 TJ apart, components HI TJ apart
    face_flux<T, 0, SCHEME>(gamma, zpl, um, u0,
                            Fp + WENOFD_SPAN(g.guard, f * TJ + j, f * TJ + j + 4 * TJ + 3 * HI * TJ, S::kSplit),
                            Fm + WENOFD_SPAN(g.guard, (f + 1) * TJ + j, (f + 5) * TJ + j + 3 * HI * TJ, S::kSplit),
                            TJ, HI * TJ, out);
#pragma unroll
    for (int r = 0; r < 4; ++r) Hf[WENOFD_IX(g.guard, (r * (TI + 1) + f) * TJ + j, S::kFace)] = out[r];
  }
  __syncthreads();

  // rhs = 0 + x term  (rhs zeroed in assembleRHS, then += in the x sweep)
  constexpr int PPT = (TI * TJ + NT - 1) / NT;
  T rhs[PPT][4];
  const T dx = g.dx, dy = g.dy;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int t = threadIdx.x + k * NT;
    const int i = t / TJ, j = t - (t / TJ) * TJ;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (t < TI * TJ) {
        const T hr = Hf[WENOFD_IX(g.guard, (r * (TI + 1) + i + 1) * TJ + j, S::kFace)],
                hl = Hf[WENOFD_IX(g.guard, (r * (TI + 1) + i) * TJ + j, S::kFace)];
        rhs[k][r] = T(0.0) + tdiv(-(hr - hl), dx);
      }
    }
  }
  __syncthreads();

  // --- y sweep: split fluxes of tile rows, halo columns 0..HJ-1
  for (int t = threadIdx.x; t < TI * HJ; t += NT) {
    const int i = t / HJ, hj = t - i * HJ;
    T q[4], fm[4], fp[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) q[r] = Us[WENOFD_IX(g.guard, S::u(r, i + 3, hj), S::kU)];
    flux_split<T, 1>(gamma, q, fm, fp);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      Fp[WENOFD_IX(g.guard, (r * TI + i) * HJ + hj, S::kSplit)] = fp[r];
      Fm[WENOFD_IX(g.guard, (r * TI + i) * HJ + hj, S::kSplit)] = fm[r];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < TI * (TJ + 1); t += NT) {
    const int i = t / (TJ + 1), f = t - i * (TJ + 1);
    if (i0 + i >= g.nx || j0 + f > g.ny) continue;
    T um[4], u0[4], out[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      um[r] = Us[WENOFD_IX(g.guard, S::u(r, i + 3, f + 2), S::kU)];
      u0[r] = Us[WENOFD_IX(g.guard, S::u(r, i + 3, f + 3), S::kU)];
    }
    // stencils: nodes 0..4 adjacent, components TI HJ apart
    face_flux<T, 1, SCHEME>(gamma, zpl, um, u0,
                            Fp + WENOFD_SPAN(g.guard, i * HJ + f, i * HJ + f + 4 + 3 * TI * HJ, S::kSplit),
                            Fm + WENOFD_SPAN(g.guard, i * HJ + f + 1, i * HJ + f + 5 + 3 * TI * HJ, S::kSplit), 1,
                            TI * HJ, out);
#pragma unroll
    for (int r = 0; r < 4; ++r) Hf[WENOFD_IX(g.guard, (r * TI + i) * (TJ + 1) + f, S::kFace)] = out[r];
  }
  __syncthreads();

  // --- y term, source, RK combination, store
  const double dt = COH ? __ldcg(a.dt) : *a.dt;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int t = threadIdx.x + k * NT;
    if (t >= TI * TJ) continue;
    const int i = t / TJ, j = t - i * TJ;
    if (i0 + i >= g.nx || j0 + j >= g.ny) continue;
    T rr[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const T hr = Hf[WENOFD_IX(g.guard, (r * TI + i) * (TJ + 1) + j + 1, S::kFace)],
              hl = Hf[WENOFD_IX(g.guard, (r * TI + i) * (TJ + 1) + j, S::kFace)];
      rr[r] = rhs[k][r] + tdiv(-(hr - hl), dy);
    }
    const long long gidx = WENOFD_NODE(g, i0 + i, j0 + j);
    if (g.gravity) {  // RTI, g = 1 (src/WENOFD.cpp:807-813)
      const T g_g0 = T(1.0);
      rr[3] += Us[WENOFD_IX(g.guard, S::u(2, i + 3, j + 3), S::kU)] * g_g0;
      rr[2] += Us[WENOFD_IX(g.guard, S::u(0, i + 3, j + 3), S::kU)] * g_g0;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const long long ix = r * g.plane + gidx;
      if (a.mode == kModeRHS) {
        a.uout[ix] = rr[r];
      } else {
        const double un = COH ? __ldcg(&a.un[ix]) : a.un[ix], ui = COH ? __ldcg(&a.uin[ix]) : a.uin[ix];
        a.uout[ix] = a.a * un + a.b * ui + a.c * dt * rr[r];
      }
    }
  }
}

// Residency: the FP32 tiles read their FP64 inputs back in the epilogue
// instead of staging them, and ask for four (routed) or three resident
// 256-thread blocks per SM: the stage is issue-bound and latency-bound, and
// trading registers for resident warps pays.  The FP64 tile is bound by the
// FP64 pipe and keeps the registers.
template <typename T, bool ROUTE, int NT>
__host__ __device__ constexpr int stage_blocks_per_sm() {
  if constexpr (sizeof(T) == 8) return 1;
  else return NT <= 256 ? (ROUTE ? 4 : 3) : (ROUTE ? 2 : 1);
}
// FP32 tiles stage their FP64 inputs in shared memory only at one block per SM.
template <typename T, bool ROUTE, int NT>
__host__ __device__ constexpr bool stage_keeps_inputs() {
  return stage_blocks_per_sm<T, ROUTE, NT>() == 1;
}

// The FP32 tiles take their halo (and flags) by TMA through the maps in
// `tma`; the FP64 tile ignores them.
template <typename T, int SCHEME, int TI, int TJ, int NT, bool ROUTE>
__global__ void __launch_bounds__(NT, stage_blocks_per_sm<T, ROUTE, NT>())
    k_stage(Geom g, StageArgs a, const __grid_constant__ StageTma tma) {
  if (*a.active == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // first interior node of the tile (0-based)
  if constexpr (sizeof(T) == 4)
    stage_tile_f32<SCHEME, TI, TJ, NT, ROUTE, false, stage_keeps_inputs<T, ROUTE, NT>(), true>(
        g, a, int(blockIdx.y) * TI, int(blockIdx.x) * TJ, smem_raw, int(blockIdx.y * gridDim.x + blockIdx.x),
        &tma);
  else
    stage_tile_f64<SCHEME, TI, TJ, NT, false, true>(g, a, int(blockIdx.y) * TI, int(blockIdx.x) * TJ, smem_raw,
                                                    &tma);
}

// Dynamic shared memory of one stage tile.
template <typename T, int TI, int TJ, bool ROUTE = false, int NT = 256>
constexpr size_t stage_smem_bytes() {
  if constexpr (sizeof(T) == 4) return StageSmem32<TI, TJ, stage_keeps_inputs<T, ROUTE, NT>()>::bytes;
  else return StageSmem<TI, TJ>::bytes;
}

// Host-side launcher for one precision: picks the kernel instance for the
// scheme and tile height, sets its shared-memory size, launches it.
template <typename T, int TI, int NT, bool ROUTE = false>
cudaError_t launch_stage_tile(const Geom &g, const StageArgs &a, const StageTma &tma, int scheme, cudaStream_t s) {
  constexpr int TJ = 32;
  constexpr size_t smem = stage_smem_bytes<T, TI, TJ, ROUTE, NT>();
  const dim3 grid((g.ny + TJ - 1) / TJ, (g.nx + TI - 1) / TI);
  void (*fn)(Geom, StageArgs, StageTma) = nullptr;
  switch (scheme) {
    case kWenoJS: fn = k_stage<T, kWenoJS, TI, TJ, NT, ROUTE>; break;
    case kWenoZ: fn = k_stage<T, kWenoZ, TI, TJ, NT, ROUTE>; break;
    case kWenoZP: fn = k_stage<T, kWenoZP, TI, TJ, NT, ROUTE>; break;
    case kWenoZPI: fn = k_stage<T, kWenoZPI, TI, TJ, NT, ROUTE>; break;
    default: return cudaErrorInvalidValue;
  }
  // The dynamic shared-memory limit is a per-device function attribute: set
  // it on the first launch per device (before any stream capture; the C ABI
  // runs one plain step before it captures a graph).
  static unsigned long long configured[4] = {0, 0, 0, 0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured[scheme & 3] & bit)) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    configured[scheme & 3] |= bit;
  }
  fn<<<grid, NT, smem, s>>>(g, a, tma);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace wenofd
