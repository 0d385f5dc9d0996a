// One RK stage tile of the FP32 precision form (and of the learned form,
// ROUTE), the FP32 counterpart of stage_tile_f64 in stage_kernel.cuh with the
// same phases and the same per-face arithmetic, laid out for the FP32 pipe:
// every node's four conserved components (and its split fluxes, and every
// face's flux) sit together as one float4 in shared memory, so a stencil
// read is one 128-bit shared load per node instead of four, and the index
// arithmetic is done once per node.
//
// Shared memory (float4 elements unless noted), from a 128-byte aligned base:
//   Fp,Fm[HI][TJ] / [TI][HJ] split fluxes of the x / y sweep
//   Hf   [TI+1][TJ] / [TI][TJ+1] face fluxes of the x / y sweep
//   Us   [HI][HJ]          state tile + 3-node halo (FP32)
//   U64  double [4][TI][TJ] the tile's FP64 input values (kept from the load)
//   Un64 double [4][TI][TJ] the tile's FP64 U^n (stages 2-3, cp.async)
// The TMA form lands the tile's FP64 halo box, [4][HI][40] doubles, at the
// base, over Fp/Fm/Hf, which the sweeps write only after it is converted.
#pragma once

#include "aux_device.cuh"
#include "convert.cuh"
#include "physics.cuh"
#include "tma.cuh"

namespace wenofd {
namespace dev {

// KEEP: the tile's FP64 input values and U^n are staged in shared memory
// (U64, Un64); without KEEP the epilogue reads them from global memory
// (cached, just loaded with the halo), which frees 2 x 15 KB per block for
// a fourth resident block.
template <int TI, int TJ, bool KEEP = true>
struct StageSmem32 {
  static constexpr int HI = TI + 6, HJ = TJ + 6;
  static constexpr int kU = HI * HJ;
  static constexpr int kSplit = HI * TJ > TI * HJ ? HI * TJ : TI * HJ;
  static constexpr int kFace = (TI + 1) * TJ > TI * (TJ + 1) ? (TI + 1) * TJ : TI * (TJ + 1);
  static constexpr int kKeep = KEEP ? 2 * 4 * TI * TJ : 0;  // doubles
  // TMA halo box: 40 columns (the 38 halo columns from the even column
  // before them) x HI rows x 4 planes of FP64; the flag box 48 x (TI + 4)
  static constexpr int kBoxJ = 40, kFlagBoxJ = 48;
  static constexpr unsigned kBoxBytes = 4u * HI * kBoxJ * 8u;
  static constexpr unsigned kFlagBoxBytes = unsigned(kFlagBoxJ) * (TI + 4);
  static_assert(kBoxBytes <= sizeof(float4) * (2 * kSplit + kFace), "halo box must fit over Fp, Fm and Hf");
  static_assert(TJ + 6 <= kBoxJ && TJ + 8 <= kFlagBoxJ, "box widths");
  // 128 bytes of slack: the base is rounded up to 128 bytes (TMA destination)
  static constexpr size_t bytes =
      128 + sizeof(float4) * (size_t(kU) + 2 * kSplit + kFace) + sizeof(double) * kKeep;
};

__device__ __forceinline__ float4 f4_split_store(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

// Pointwise Lax-Friedrichs split of one node (flux_split in physics.cuh; the
// same operations, F -+ ws U and the halving on packed pairs).
template <int DIR>
__device__ __forceinline__ void split4(float gamma, const float4 q, float4 &fm, float4 &fp) {
  const float U[4] = {q.x, q.y, q.z, q.w};
  float u, v, p;
  primitives(gamma, U, u, v, p);
  const float rho = q.x, E = q.w;
  float F[4];
  if (DIR == 0) {
    F[0] = rho * u;
    F[1] = rho * u * u + p;
    F[2] = rho * u * v;
    F[3] = (E + p) * u;
  } else {
    F[0] = rho * v;
    F[1] = rho * u * v;
    F[2] = rho * v * v + p;
    F[3] = (E + p) * v;
  }
  const float c = tsqrt(tdiv(gamma * p, rho));
  const float ws = (DIR == 0 ? tabs(u) : tabs(v)) + c;
  const float2 h = splat2(0.5f), mws = splat2(-ws), pws = splat2(ws);
  const float2 F01 = make_float2(F[0], F[1]), F23 = make_float2(F[2], F[3]);
  fm = join2(__fmul2_rn(h, __ffma2_rn(mws, lo2(q), F01)), __fmul2_rn(h, __ffma2_rn(mws, hi2(q), F23)));
  fp = join2(__fmul2_rn(h, __ffma2_rn(pws, lo2(q), F01)), __fmul2_rn(h, __ffma2_rn(pws, hi2(q), F23)));
}

// Linear fifth-order upwind flux of one component: WENO with its weights
// frozen at (0.1, 0.6, 0.3), on F+ at nodes face-3..face+1 (p0..p4) and on F-
// mirrored (nodes face+2..face-2, m4..m0): (2a - 13b + 47c + 27d - 3e) / 60
// each.
__device__ __forceinline__ float lin5(float p0, float p1, float p2, float p3, float p4, float m0, float m1, float m2,
                                      float m3, float m4) {
  const float c0 = float(2.0 / 60.0), c1 = float(-13.0 / 60.0), c2 = float(47.0 / 60.0), c3 = float(27.0 / 60.0),
              c4 = float(-3.0 / 60.0);
  const float plus = c0 * p0 + c1 * p1 + c2 * p2 + c3 * p3 + c4 * p4;
  const float minus = c0 * m4 + c1 * m3 + c2 * m2 + c3 * m1 + c4 * m0;
  return plus + minus;
}

// lin5 on two components at once (the same operation order).
__device__ __forceinline__ float2 lin5x2(float2 p0, float2 p1, float2 p2, float2 p3, float2 p4, float2 m0, float2 m1,
                                         float2 m2, float2 m3, float2 m4) {
  const float2 c0 = splat2(float(2.0 / 60.0)), c1 = splat2(float(-13.0 / 60.0)), c2 = splat2(float(47.0 / 60.0)),
               c3 = splat2(float(27.0 / 60.0)), c4 = splat2(float(-3.0 / 60.0));
  float2 plus = __fmul2_rn(c0, p0);
  plus = __ffma2_rn(c1, p1, plus);
  plus = __ffma2_rn(c2, p2, plus);
  plus = __ffma2_rn(c3, p3, plus);
  plus = __ffma2_rn(c4, p4, plus);
  float2 minus = __fmul2_rn(c0, m4);
  minus = __ffma2_rn(c1, m3, minus);
  minus = __ffma2_rn(c2, m2, minus);
  minus = __ffma2_rn(c3, m1, minus);
  minus = __ffma2_rn(c4, m0, minus);
  return __fadd2_rn(plus, minus);
}

__device__ __forceinline__ float4 linear_face4(const float4 *P, const float4 *M, int ss) {
  const float4 p0 = P[0], p1 = P[ss], p2 = P[2 * ss], p3 = P[3 * ss], p4 = P[4 * ss];
  const float4 m0 = M[0], m1 = M[ss], m2 = M[2 * ss], m3 = M[3 * ss], m4 = M[4 * ss];
  return join2(lin5x2(lo2(p0), lo2(p1), lo2(p2), lo2(p3), lo2(p4), lo2(m0), lo2(m1), lo2(m2), lo2(m3), lo2(m4)),
               lin5x2(hi2(p0), hi2(p1), hi2(p2), hi2(p3), hi2(p4), hi2(m0), hi2(m1), hi2(m2), hi2(m3), hi2(m4)));
}

// Characteristic WENO face from float4 stencils (face_flux_st).
template <int DIR, int SCHEME>
__device__ __forceinline__ float4 weno_face4(float gamma, float zpl, const float4 um4, const float4 u04,
                                             const float4 *P, const float4 *M, int ss) {
  const float um[4] = {um4.x, um4.y, um4.z, um4.w}, u0[4] = {u04.x, u04.y, u04.z, u04.w};
  float out[4];
  face_flux_st<float, DIR, SCHEME>(gamma, zpl, um, u0, Float4Stencil{P, ss}, Float4Stencil{M, ss}, out);
  return make_float4(out[0], out[1], out[2], out[3]);
}

// One characteristic field of a WENO face, for the routed form where the
// faces that need WENO are few and would otherwise keep a handful of threads
// busy while the block waits: four consecutive lanes take one face, lane k
// projects the ten stencil fluxes on left eigenvector k and reconstructs
// characteristic field k (face_flux_st's per-field work, same operation
// order), the four fields are exchanged by shuffles, and lane k returns
// component k of R * vh.  All 32 lanes of the warp must call it.
template <int DIR, int SCHEME>
__device__ __forceinline__ float weno_face_lane(float gamma, float zpl, const float4 um4, const float4 u04,
                                                const float4 *P, const float4 *M, int ss, int k) {
  const float um[4] = {um4.x, um4.y, um4.z, um4.w}, u0[4] = {u04.x, u04.y, u04.z, u04.w};
  float ave[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ave[r] = 0.5f * (um[r] + u0[r]);
  float u, v, p;
  primitives(gamma, ave, u, v, p);
  const float rho = ave[0], E = ave[3];
  const float c = tsqrt(tdiv(gamma * p, rho));
  const float B1 = tdiv((gamma - 1.0f), (c * c));
  const float B2 = B1 * (u * u + v * v) * 0.5f;
  const float H = tdiv((E + p), rho);
  const float ic = tdiv(1.0f, c);
  const float nc = tdiv(DIR == 0 ? u : v, c);
  const float B1u = B1 * u, B1v = B1 * v;
  // row k of the left eigenvector matrix (face_flux_st)
  float l0, l1, l2, l3;
  if (DIR == 0) {
    l0 = k == 0 ? (B2 + nc) * 0.5f : (k == 1 ? v : (k == 2 ? (1.0f - B2) : (B2 - nc) * 0.5f));
    l1 = k == 0 ? -(B1u + ic) * 0.5f : (k == 1 ? 0.0f : (k == 2 ? B1u : -(B1u - ic) * 0.5f));
    l2 = k == 0 ? -(B1v) * 0.5f : (k == 1 ? -1.0f : (k == 2 ? B1v : -B1v * 0.5f));
    l3 = k == 0 ? B1 * 0.5f : (k == 1 ? 0.0f : (k == 2 ? -B1 : B1 * 0.5f));
  } else {
    l0 = k == 0 ? (B2 + nc) * 0.5f : (k == 1 ? -u : (k == 2 ? 1.0f - B2 : (B2 - nc) * 0.5f));
    l1 = k == 0 ? -(B1u) * 0.5f : (k == 1 ? 1.0f : (k == 2 ? B1u : -(B1u) * 0.5f));
    l2 = k == 0 ? -(B1v + ic) * 0.5f : (k == 1 ? 0.0f : (k == 2 ? B1v : -(B1v - ic) * 0.5f));
    l3 = k == 0 ? B1 * 0.5f : (k == 1 ? 0.0f : (k == 2 ? -B1 : B1 * 0.5f));
  }
  float vp[5], vm[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const float4 a = P[s * ss], b = M[s * ss];
    float x = l0 * a.x;
    x += l1 * a.y;
    x += l2 * a.z;
    x += l3 * a.w;
    vp[s] = x;
    float y = l0 * b.x;
    y += l1 * b.y;
    y += l2 * b.z;
    y += l3 * b.w;
    vm[s] = y;
  }
  const float vhk = weno_sides<float, SCHEME>(vp, vm, zpl);
  const int base = (threadIdx.x & 31) & ~3;
  const float vh0 = __shfl_sync(0xffffffffu, vhk, base + 0);
  const float vh1 = __shfl_sync(0xffffffffu, vhk, base + 1);
  const float vh2 = __shfl_sync(0xffffffffu, vhk, base + 2);
  const float vh3 = __shfl_sync(0xffffffffu, vhk, base + 3);
  // row k of R (face_flux_st, utils/equations.hpp:239-299)
  const float q2 = (u * u + v * v) * 0.5f;
  float r0, r1, r2, r3;
  if (DIR == 0) {
    r1 = k == 0 ? 0.0f : (k == 1 ? 0.0f : (k == 2 ? -1.0f : -v));
    r2 = k == 0 ? 1.0f : (k == 1 ? u : (k == 2 ? v : q2));
    r3 = k == 0 ? 1.0f : (k == 1 ? u + c : (k == 2 ? v : H + c * u));
    r0 = k == 0 ? 1.0f : (k == 1 ? u - c : (k == 2 ? v : H - c * u));
  } else {
    r1 = k == 0 ? 0.0f : (k == 1 ? 1.0f : (k == 2 ? 0.0f : u));
    r2 = k == 0 ? 1.0f : (k == 1 ? u : (k == 2 ? v : q2));
    r3 = k == 0 ? 1.0f : (k == 1 ? u : (k == 2 ? v + c : H + c * v));
    r0 = k == 0 ? 1.0f : (k == 1 ? u : (k == 2 ? v - c : H - c * v));
  }
  float f = r0 * vh0;
  f += r1 * vh1;
  f += r2 * vh2;
  f += r3 * vh3;
  return f;
}

__device__ __forceinline__ void cp_async8_f32(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all_f32() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Asks L2 for the 128-byte line holding p (a hint: no data moves to the
// thread, and nothing waits for it).
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.L2 [%0];" ::"l"(p)); }

// One tile (TI x TJ interior nodes from i0, j0) of one RK stage, all NT
// threads of the block.  ROUTE: faces take the linear upwind flux unless a
// node of their stencil line is flagged (a.flags).  COH: inputs may have
// been written earlier in the same launch by other blocks (persistent
// batched kernel): loads through L2, U^n read in the epilogue.  TMA (the
// per-solve kernels): the halo box and the flag box arrive by TMA (maps in
// `tma`), one thread issuing both; otherwise every thread loads 128-bit
// node pairs.
// With a.bounds set (last stage of a step), the epilogue also screens the
// time step of the nodes it writes (screen_speed) and stores the tile's
// (max s32 - e, max s32 + e) at a.bounds[tile], raising *a.screen to the
// tile's lower bound.
template <int SCHEME, int TI, int TJ, int NT, bool ROUTE, bool COH = false, bool KEEP = true, bool TMA = false>
__device__ __forceinline__ void stage_tile_f32(const Geom &g, const StageArgs &a, const int i0, const int j0,
                                               unsigned char *smem_raw, const int tile = 0,
                                               const StageTma *tma = nullptr) {
  using S = StageSmem32<TI, TJ, KEEP>;
  constexpr int HI = S::HI, HJ = S::HJ;
  unsigned char *base = smem_raw + (((tma_smem_addr(smem_raw) + 127u) & ~127u) - tma_smem_addr(smem_raw));
  float4 *Fp = reinterpret_cast<float4 *>(base);
  float4 *Fm = Fp + S::kSplit;
  float4 *Hf = Fm + S::kSplit;
  float4 *Us = Hf + S::kFace;
  double *U64 = reinterpret_cast<double *>(Us + S::kU);
  double *Un64 = U64 + 4 * TI * TJ;
  constexpr int FI = TI + 4, FJ = TJ + 4;
  // node flags: flag node (fi, fj) at sflag[fi * FS + fj + FO]; the TMA box
  // starts two columns before the first flag node
  constexpr int FS = TMA ? S::kFlagBoxJ : FJ, FO = TMA ? 2 : 0;
  constexpr int kMaxFaces = S::kFace;
  __shared__ __align__(128) unsigned char sflag[ROUTE ? FI * FS : 1];
  __shared__ short slist[ROUTE ? kMaxFaces : 1];
  __shared__ int scount_x, scount_y;  // WENO faces listed in the x and y sweeps
  __shared__ __align__(8) unsigned long long tma_bar;
  if constexpr (TMA) {
    // The halo box (and the flag box) by TMA, one thread issuing both.
    if (threadIdx.x == 0) tma_bar_init(tma_smem_addr(&tma_bar), 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned bar = tma_smem_addr(&tma_bar);
      tma_fence_proxy();
      tma_bar_expect(bar, S::kBoxBytes + (ROUTE ? S::kFlagBoxBytes : 0u));
      // box column 0 = ghosted column j0 (even: 16-byte aligned); row 0 =
      // ghosted row 1 + i0, the first halo row
      // first coordinates: x * element size a multiple of 16 bytes (an
      // unissued copy leaves the wait below to give up)
      if (WENOFD_REQUIRE(g.guard, (j0 & 1) == 0, j0, 2)) tma_load_3d(tma_smem_addr(base), &tma->u, j0, 1 + i0, 0, bar);
      if constexpr (ROUTE)
        if (WENOFD_REQUIRE(g.guard, (j0 & 15) == 0, j0, 16))
          tma_load_2d(tma_smem_addr(sflag), &tma->flags, j0, 2 + i0, bar);
    }
  }

  const float gamma = g.gamma32, zpl = g.zpl32;
  const bool stage1 = a.form == kFormStage1;

  // Stages 2 and 3 that do not stage U^n by cp.async (without KEEP, or in
  // the persistent batched kernel) read it only in the epilogue, the first
  // touch of those lines in this tile: ask L2 for them now, so that the
  // epilogue's loads hit L2 instead of waiting on DRAM (a hint only; L2 is
  // where the batched kernel's loads see other blocks' writes anyway).  A
  // tile row of 32 doubles from ghosted column j0 + 4 (rows start on
  // 256-byte boundaries, j0 a multiple of 32) spans three 128-byte lines,
  // holding the tile's columns -4..11, 12..27 and 28..43: one prefetch at
  // columns 0, 12 and 28 (clamped to the grid) per row and component.
  if constexpr (COH || !KEEP) {
    if (a.mode == kModeRK && !stage1) {
      constexpr int kLines = 3;
      for (int t = threadIdx.x; t < 4 * TI * kLines; t += NT) {
        const int r = t / (TI * kLines), q = t - r * (TI * kLines);
        const int i = q / kLines, l = q - (q / kLines) * kLines;
        const int ii = min(i0 + i, g.nx - 1), jj = min(j0 + (l == 0 ? 0 : (l == 1 ? 12 : 28)), g.ny - 1);
        prefetch_l2(&a.un[r * g.plane + WENOFD_NODE(g, ii, jj)]);
      }
    }
  }

  // stages 2 and 3: fetch this tile's U^n now, used only by the epilogue
  if constexpr (!COH && KEEP) {
    if (a.mode == kModeRK && !stage1) {
      for (int t = threadIdx.x; t < 4 * TI * TJ; t += NT) {
        const int r = t / (TI * TJ), q = t - r * (TI * TJ);
        const int i = q / TJ, j = q - (q / TJ) * TJ;
        if (i0 + i < g.nx && j0 + j < g.ny)
          cp_async8_f32(&Un64[WENOFD_IX(g.guard, t, 4 * TI * TJ)], &a.un[r * g.plane + WENOFD_NODE(g, i0 + i, j0 + j)]);
      }
    }
  }

  if constexpr (TMA) {
    // Bounded wait for the boxes; on give-up the whole block records the
    // error and leaves the tile (a second bounded wait first lets a late
    // copy land before the block exits).
    const bool ok = tma_bar_wait(tma_smem_addr(&tma_bar), 0, kTmaWaitLimit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        if (a.wait_error) atomicExch(a.wait_error, 1);
        tma_bar_wait(tma_smem_addr(&tma_bar), 0, kTmaWaitLimit);
      }
      __syncthreads();
      return;
    }
    // node pair p of halo row hi: box columns 2p, 2p + 1 = nodes hj = 2p - 1,
    // 2p (20 pairs span the 38 halo columns; the first and last box column
    // are not needed)
    constexpr int PJ = S::kBoxJ / 2;
    const double2 *box = reinterpret_cast<const double2 *>(base);
    for (int t = threadIdx.x; t < HI * PJ; t += NT) {
      const int hi = t / PJ, p = t - (t / PJ) * PJ;
      double2 v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) v[r] = box[WENOFD_IX(g.guard, (r * HI + hi) * PJ + p, S::kBoxBytes / 16)];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int hj = 2 * p - 1 + h;
        if (hj < 0 || hj >= HJ) continue;
        double x[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) x[r] = h ? v[r].y : v[r].x;
        Us[WENOFD_IX(g.guard, hi * HJ + hj, S::kU)] =
            make_float4(f64_to_f32(x[0]), f64_to_f32(x[1]), f64_to_f32(x[2]), f64_to_f32(x[3]));
        if constexpr (KEEP) {
          if (hi >= 3 && hi < 3 + TI && hj >= 3 && hj < 3 + TJ) {
            const int q = (hi - 3) * TJ + hj - 3;
#pragma unroll
            for (int r = 0; r < 4; ++r) U64[WENOFD_IX(g.guard, r * TI * TJ + q, 4 * TI * TJ)] = x[r];
          }
        }
      }
    }
    if constexpr (ROUTE) {
      if (threadIdx.x == 0) scount_x = scount_y = 0;
    }
  } else {
  // --- state tile with halo: node (hi, hj) = global (1 + i0 + hi, 1 + j0 + hj).
  // A thread loads a pair of adjacent nodes per component with one 128-bit
  // load: pair p of halo row hi covers global columns j0 + 2p and j0 + 2p + 1
  // (16-byte aligned: rows start on 256-byte boundaries, j0 is even), i.e.
  // hj = 2p - 1 and 2p; 20 pairs span the 38 halo columns (the first and last
  // loaded node are not needed).  The routed form's node flags (tile + 2-node
  // halo, flag node (fi, fj) = global (2 + i0 + fi, 2 + j0 + fj)) come as
  // aligned 32-bit words the same way.  All loads of a thread are issued
  // before any is used.
  {
    constexpr int PJ = (HJ + 2) / 2;  // pairs per halo row
    constexpr int NLD = (HI * PJ + NT - 1) / NT;
    constexpr int WJ = (FJ + 2 + 3) / 4;  // flag words per row: global columns j0 .. j0 + 4 WJ - 1
    constexpr int NFL = ROUTE ? (FI * WJ + NT - 1) / NT : 1;
    double2 v[NLD][4];
    unsigned fv[NFL];
#pragma unroll
    for (int k = 0; k < NLD; ++k) {
      const int t = threadIdx.x + k * NT;
      const int hi = t / PJ, p = t - (t / PJ) * PJ;
      const int ei = 1 + i0 + hi, ej = j0 + 2 * p;
      const bool ok = t < HI * PJ && ei < g.nxt && ej < g.pitch;
      // (ej even and the pitch a multiple of 32: ej + 1 is in the row too)
      const double2 *src = reinterpret_cast<const double2 *>(a.uin + WENOFD_GNODE_IF(g, ok, ei, ej));
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if constexpr (COH) v[k][r] = ok ? __ldcg(src + r * (g.plane / 2)) : make_double2(0.0, 0.0);
        else v[k][r] = ok ? __ldg(src + r * (g.plane / 2)) : make_double2(0.0, 0.0);
      }
    }
    if constexpr (ROUTE) {
#pragma unroll
      for (int k = 0; k < NFL; ++k) {
        const int t = threadIdx.x + k * NT;
        const int fi = t / WJ, w = t - (t / WJ) * WJ;
        const int ei = 2 + i0 + fi, ej = j0 + 4 * w;
        fv[k] = (t < FI * WJ && ei < g.nxt && ej < g.pitch)
                    ? *reinterpret_cast<const unsigned *>(a.flags + WENOFD_GNODE(g, ei, ej))
                    : 0x01010101u;
      }
    }
#pragma unroll
    for (int k = 0; k < NLD; ++k) {
      const int t = threadIdx.x + k * NT;
      if (t < HI * PJ) {
        const int hi = t / PJ, p = t - (t / PJ) * PJ;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int hj = 2 * p - 1 + h;
          if (hj < 0 || hj >= HJ) continue;
          double x[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) x[r] = h ? v[k][r].y : v[k][r].x;
          Us[WENOFD_IX(g.guard, hi * HJ + hj, S::kU)] =
              make_float4(f64_to_f32(x[0]), f64_to_f32(x[1]), f64_to_f32(x[2]), f64_to_f32(x[3]));
          if constexpr (KEEP) {
            if (hi >= 3 && hi < 3 + TI && hj >= 3 && hj < 3 + TJ) {
              const int q = (hi - 3) * TJ + hj - 3;
#pragma unroll
              for (int r = 0; r < 4; ++r) U64[WENOFD_IX(g.guard, r * TI * TJ + q, 4 * TI * TJ)] = x[r];
            }
          }
        }
      }
    }
    if constexpr (ROUTE) {
#pragma unroll
      for (int k = 0; k < NFL; ++k) {
        const int t = threadIdx.x + k * NT;
        if (t < FI * WJ) {
          const int fi = t / WJ, w = t - (t / WJ) * WJ;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int fj = 4 * w + c - 2;  // global column j0 + 4w + c = 2 + j0 + fj
            if (fj >= 0 && fj < FJ) sflag[WENOFD_IX(g.guard, fi * FJ + fj, FI * FS)] = (unsigned char)(fv[k] >> (8 * c));
          }
        }
      }
      if (threadIdx.x == 0) scount_x = scount_y = 0;
    }
  }
  }  // TMA
  __syncthreads();

  // --- x sweep: split fluxes of halo rows 0..HI-1, tile columns
  for (int t = threadIdx.x; t < HI * TJ; t += NT) {
    const int hi = t / TJ, j = t - (t / TJ) * TJ;
    split4<0>(gamma, Us[WENOFD_IX(g.guard, hi * HJ + j + 3, S::kU)], Fm[WENOFD_IX(g.guard, t, S::kSplit)],
              Fp[WENOFD_IX(g.guard, t, S::kSplit)]);
  }
  __syncthreads();
  // x faces f = 0..TI between tile nodes f-1 and f: F+ rows f..f+4, F- rows f+1..f+5
  for (int t = threadIdx.x; t < (TI + 1) * TJ; t += NT) {
    const int f = t / TJ, j = t - (t / TJ) * TJ;
    if (i0 + f > g.nx || j0 + j >= g.ny) continue;
    if constexpr (ROUTE) {
      Hf[WENOFD_IX(g.guard, t, S::kFace)] =
          linear_face4(Fp + WENOFD_SPAN(g.guard, t, t + 4 * TJ, S::kSplit),
                       Fm + WENOFD_SPAN(g.guard, t + TJ, t + 5 * TJ, S::kSplit), TJ);
      // nodes f-2 .. f+1
      const unsigned char *fl = sflag + WENOFD_SPAN(g.guard, f * FS + (j + 2 + FO), (f + 3) * FS + (j + 2 + FO), FI * FS);
      if (fl[0] | fl[FS] | fl[2 * FS] | fl[3 * FS]) slist[WENOFD_IX(g.guard, atomicAdd(&scount_x, 1), kMaxFaces)] = short(t);
    } else {
      Hf[WENOFD_IX(g.guard, t, S::kFace)] = weno_face4<0, SCHEME>(
          gamma, zpl, Us[WENOFD_IX(g.guard, (f + 2) * HJ + j + 3, S::kU)], Us[WENOFD_IX(g.guard, (f + 3) * HJ + j + 3, S::kU)],
          Fp + WENOFD_SPAN(g.guard, t, t + 4 * TJ, S::kSplit), Fm + WENOFD_SPAN(g.guard, t + TJ, t + 5 * TJ, S::kSplit), TJ);
    }
  }
  // The listed faces (if any) are recomputed with WENO after the barrier;
  // with none listed (block-uniform) the second barrier is not needed.
  __syncthreads();
  if constexpr (ROUTE) {
    const int nw = scount_x;
    if (nw) {
      for (int base = threadIdx.x & ~31; base < 4 * nw; base += NT) {  // 4 lanes per face, whole warps
        const int q4 = base + (threadIdx.x & 31);
        const int t = slist[WENOFD_IX(g.guard, q4 < 4 * nw ? q4 >> 2 : 0, kMaxFaces)];
        const int f = t / TJ, j = t - (t / TJ) * TJ;
        const float o = weno_face_lane<0, SCHEME>(
            gamma, zpl, Us[WENOFD_IX(g.guard, (f + 2) * HJ + j + 3, S::kU)], Us[WENOFD_IX(g.guard, (f + 3) * HJ + j + 3, S::kU)],
            Fp + WENOFD_SPAN(g.guard, t, t + 4 * TJ, S::kSplit), Fm + WENOFD_SPAN(g.guard, t + TJ, t + 5 * TJ, S::kSplit), TJ,
            q4 & 3);
        if (q4 < 4 * nw) reinterpret_cast<float *>(&Hf[WENOFD_IX(g.guard, t, S::kFace)])[q4 & 3] = o;
      }
      __syncthreads();
    }
  }

  // x term of the node's RHS (rhs zeroed, then += in the x sweep)
  constexpr int PPT = (TI * TJ + NT - 1) / NT;
  float4 rhs[PPT];
  const float idx = g.inv_dx32, idy = g.inv_dy32;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int t = threadIdx.x + k * NT;
    if (t < TI * TJ) {
      const float4 hr = Hf[WENOFD_IX(g.guard, t + TJ, S::kFace)], hl = Hf[WENOFD_IX(g.guard, t, S::kFace)];
      const float2 mi = splat2(-idx);  // -(hr - hl) * idx, the negation exact
      rhs[k] = join2(__fmul2_rn(sub2(lo2(hr), lo2(hl)), mi), __fmul2_rn(sub2(hi2(hr), hi2(hl)), mi));
    }
  }
  // No barrier here: the y split writes only Fp and Fm, whose readers (the x
  // faces and the x list) are behind the barriers above; Hf, which the x term
  // reads, is rewritten only after the next barrier.

  // --- y sweep: split fluxes of tile rows, halo columns 0..HJ-1
  for (int t = threadIdx.x; t < TI * HJ; t += NT) {
    const int i = t / HJ, hj = t - (t / HJ) * HJ;
    split4<1>(gamma, Us[WENOFD_IX(g.guard, (i + 3) * HJ + hj, S::kU)], Fm[WENOFD_IX(g.guard, t, S::kSplit)],
              Fp[WENOFD_IX(g.guard, t, S::kSplit)]);
  }
  __syncthreads();
  // y faces f = 0..TJ of row i: F+ columns f..f+4, F- columns f+1..f+5
  for (int t = threadIdx.x; t < TI * (TJ + 1); t += NT) {
    const int i = t / (TJ + 1), f = t - (t / (TJ + 1)) * (TJ + 1);
    if (i0 + i >= g.nx || j0 + f > g.ny) continue;
    const int s = i * HJ + f;
    if constexpr (ROUTE) {
      Hf[WENOFD_IX(g.guard, t, S::kFace)] = linear_face4(Fp + WENOFD_SPAN(g.guard, s, s + 4, S::kSplit),
                                                         Fm + WENOFD_SPAN(g.guard, s + 1, s + 5, S::kSplit), 1);
      // nodes f-2 .. f+1 along y
      const unsigned char *fl = sflag + WENOFD_SPAN(g.guard, (i + 2) * FS + f + FO, (i + 2) * FS + f + FO + 3, FI * FS);
      if (fl[0] | fl[1] | fl[2] | fl[3]) slist[WENOFD_IX(g.guard, atomicAdd(&scount_y, 1), kMaxFaces)] = short(t);
    } else {
      Hf[WENOFD_IX(g.guard, t, S::kFace)] = weno_face4<1, SCHEME>(
          gamma, zpl, Us[WENOFD_IX(g.guard, (i + 3) * HJ + f + 2, S::kU)], Us[WENOFD_IX(g.guard, (i + 3) * HJ + f + 3, S::kU)],
          Fp + WENOFD_SPAN(g.guard, s, s + 4, S::kSplit), Fm + WENOFD_SPAN(g.guard, s + 1, s + 5, S::kSplit), 1);
    }
  }
  __syncthreads();
  if constexpr (ROUTE) {
    const int nw = scount_y;
    if (nw) {
      for (int base = threadIdx.x & ~31; base < 4 * nw; base += NT) {
        const int q4 = base + (threadIdx.x & 31);
        const int t = slist[WENOFD_IX(g.guard, q4 < 4 * nw ? q4 >> 2 : 0, kMaxFaces)];
        const int i = t / (TJ + 1), f = t - (t / (TJ + 1)) * (TJ + 1);
        const int s = i * HJ + f;
        const float o = weno_face_lane<1, SCHEME>(
            gamma, zpl, Us[WENOFD_IX(g.guard, (i + 3) * HJ + f + 2, S::kU)], Us[WENOFD_IX(g.guard, (i + 3) * HJ + f + 3, S::kU)],
            Fp + WENOFD_SPAN(g.guard, s, s + 4, S::kSplit), Fm + WENOFD_SPAN(g.guard, s + 1, s + 5, S::kSplit), 1, q4 & 3);
        if (q4 < 4 * nw) reinterpret_cast<float *>(&Hf[WENOFD_IX(g.guard, t, S::kFace)])[q4 & 3] = o;
      }
      __syncthreads();
    }
  }

  // --- y term, source, RK combination in FP64, store
  const double dt = COH ? __ldcg(a.dt) : *a.dt;
  // FP64 runs at 1/64 of the FP32 rate here, and the RK combination is most
  // of a routed stage's FP64 work: the middle stages with c = b = 2^-k take
  // c * (dt * rhs + (a / c) * U^n + U), two FP64 operations per component
  // instead of three, the power-of-two scale on the integer ALU.  The form
  // comes from the host (StageArgs::form), so no FP64 compare runs here.
  const int form = a.form;
  if constexpr (!COH && KEEP) {
    cp_async_wait_all_f32();
    __syncthreads();
  }
  float lo = 0.0f, hi = 0.0f;  // screen bounds of this thread's nodes
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int t = threadIdx.x + k * NT;
    if (t >= TI * TJ) continue;
    const int i = t / TJ, j = t - (t / TJ) * TJ;
    if (i0 + i >= g.nx || j0 + j >= g.ny) continue;
    const float4 hr = Hf[WENOFD_IX(g.guard, i * (TJ + 1) + j + 1, S::kFace)],
                 hl = Hf[WENOFD_IX(g.guard, i * (TJ + 1) + j, S::kFace)];
    const float2 mi = splat2(-idy);  // rhs - (hr - hl) * idy
    const float2 r01 = __ffma2_rn(sub2(lo2(hr), lo2(hl)), mi, lo2(rhs[k]));
    const float2 r23 = __ffma2_rn(sub2(hi2(hr), hi2(hl)), mi, hi2(rhs[k]));
    float rr[4] = {r01.x, r01.y, r23.x, r23.y};
    if (g.gravity) {  // RTI, g = 1 (src/WENOFD.cpp:807-813)
      const float4 q = Us[WENOFD_IX(g.guard, (i + 3) * HJ + j + 3, S::kU)];
      rr[3] += q.z * 1.0f;
      rr[2] += q.x * 1.0f;
    }
    const long long gidx = WENOFD_NODE(g, i0 + i, j0 + j);
    double ui[4], un[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const long long ix = r * g.plane + gidx;
      if constexpr (KEEP) {
        ui[r] = U64[WENOFD_IX(g.guard, r * TI * TJ + t, 4 * TI * TJ)];
        if constexpr (COH) un[r] = __ldcg(&a.un[ix]);
        else un[r] = Un64[WENOFD_IX(g.guard, r * TI * TJ + t, 4 * TI * TJ)];
      } else if constexpr (COH) {
        ui[r] = __ldcg(&a.uin[ix]);
        un[r] = __ldcg(&a.un[ix]);
      } else {
        ui[r] = __ldg(&a.uin[ix]);
        if (!stage1) un[r] = __ldg(&a.un[ix]);
      }
    }
    double w[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const long long ix = r * g.plane + gidx;
      const double rd = f32_to_f64(rr[r]);
      if (a.mode == kModeRHS) w[r] = rd;
      else if (form == kFormStage1) w[r] = fma(dt, rd, ui[r]);  // (1, 0, 1): c * dt = dt
      else if (form == kFormRK3Mid) w[r] = scale_pow2_down<2>(fma(dt, rd, fma(3.0, un[r], ui[r])));  // (3/4, 1/4, 1/4)
      else if (form == kFormRK2Mid) w[r] = scale_pow2_down<1>(fma(dt, rd, un[r] + ui[r]));          // (1/2, 1/2, 1/2)
      else w[r] = fma(a.c * dt, rd, fma(a.b, ui[r], a.a * un[r]));
      a.uout[ix] = w[r];
    }
    if (a.bounds) {
      float s32, e;
      screen_speed(g, w[0], w[1], w[2], w[3], s32, e);
      lo = fmaxf(lo, s32 - e);
      hi = fmaxf(hi, s32 + e);
    }
  }
  if (a.bounds) {  // block-uniform
    __shared__ float2 sred[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmaxf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = make_float2(lo, hi);
    __syncthreads();
    if (threadIdx.x == 0) {
      float2 b = sred[0];
#pragma unroll
      for (int w = 1; w < NT / 32; ++w) b = make_float2(fmaxf(b.x, sred[w].x), fmaxf(b.y, sred[w].y));
      // (allocated for tiles of 15 rows, the most tiles)
      a.bounds[WENOFD_IX(g.guard, tile, ((g.nx + 14) / 15) * ((g.ny + 31) / 32))] = b;
      atomicMax(a.screen, __float_as_uint(b.x));
    }
  }
}

}  // namespace dev
}  // namespace wenofd
