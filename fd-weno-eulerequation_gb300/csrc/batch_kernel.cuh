// Batched execution: many independent solves of different sizes advanced by
// one persistent, cooperative kernel per launch.
//
// Each launch runs `nsteps` time steps of every member.  A step is a fixed
// sequence of phases separated by grid-wide barriers:
//   time-step reduction (FP64 exact pass; FP32 forms: screen, then refine)
//   -> dt of every member -> 3 x (boundary fill -> stage tiles) -> time update.
// As in the single solve, the FP32 forms' last RK stage screens the nodes it
// writes (per-tile bounds), so from a member's second step on its time-step
// reduction is the exact FP64 pass over the few tiles whose bound reaches
// the maximum lower bound, a warp per tile.
// Inside a phase the blocks take work items (stage tiles, ghost strips, node
// chunks) of all members from one atomic counter, so uneven member sizes
// balance across the GPU.  The per-member control work between phases (dt,
// the time update, the loop gate) is done by the block that arrives last at
// the barrier, before it releases the others.  The per-item bodies are the
// per-solve kernels' own (stage_tile, bc_fill_entry, exact_speed,
// screen_speed), so a member's arithmetic is the single-solve path's.
//
// Data written in one phase is read by other blocks in the next, so loads of
// state and control fields go through L2 (ld.global.cg), never through the
// non-coherent read-only path.
//
// The grid barrier spins on a generation counter with an iteration limit
// (2^24 polls of >= 128 ns, seconds, against work items of microseconds);
// on give-up it records an error (the host reports TIMEOUT) and continues,
// so no wait is unbounded.  The launch is cooperative, which guarantees that
// all blocks are resident.
#pragma once

#include "aux_device.cuh"
#include "stage_kernel.cuh"

namespace wenofd {

namespace dev {

// Grid-wide barrier.  The block that arrives last runs last() with all its
// threads before releasing the others; last() sees every write made before
// the barrier.  WITHHOLD (test instance only): block b.hold_block does not
// arrive at the launch's barrier number b.hold_barrier (`index`), so every
// block's wait there runs into the (short) poll limit.
template <bool WITHHOLD = false, typename F>
__device__ __forceinline__ void grid_barrier(const BatchArgs &b, F last, int index = 0) {
  constexpr unsigned kLimit = WITHHOLD ? kBarrierTestLimit : kBarrierLimit;
  __shared__ int s_last;
  __shared__ unsigned s_gen;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = b.barrier + 1;
    s_gen = *gen;
    __threadfence();
    bool arrive = true;
    if constexpr (WITHHOLD) arrive = !(int(blockIdx.x) == b.hold_block && index == b.hold_barrier);
    const unsigned arrived = arrive ? atomicAdd(b.barrier, 1u) : 0u;
    __threadfence();
    s_last = arrive && arrived == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    last();
    __syncthreads();
    if (threadIdx.x == 0) {
      b.barrier[0] = 0u;
      __threadfence();
      atomicAdd(b.barrier + 1, 1u);
    }
  } else if (threadIdx.x == 0) {
    // Once any wait has given up, arrival counts are no longer trusted and
    // every later wait ends within 1024 polls, so the launch still finishes
    // promptly; the host reports the error.
    volatile unsigned *gen = b.barrier + 1;
    volatile int *err = b.error;
    unsigned it = 0;
    while (*gen == s_gen) {
      ++it;
      if (it > kLimit || ((it & 1023u) == 0u && *err)) {
        atomicExch(b.error, 1);
        break;
      }
      __nanosleep(128);
    }
    __threadfence();
  }
  __syncthreads();
}

struct Nothing {
  __device__ void operator()() const {}
};

// Hand out the items [0, prefix[n]) of one phase to the blocks.  Thread 0
// claims an item from the phase's counter, finds its member and reads the
// member's `active` flag; the claim of the next item is issued before the
// current item runs, so its latency overlaps the work.  f(local item, member)
// runs with the whole block for items of active members, with the member's
// record staged in shared memory (sM).
template <typename F>
__device__ __forceinline__ void for_member_items(const BatchArgs &b, unsigned *counter, const int *prefix,
                                                 BatchMember &sM, F f) {
  __shared__ int s_item[2], s_m[2], s_on[2];
  const int n = b.n, total = __ldg(&prefix[n]);
  auto resolve = [&](int slot, int item) {  // thread 0
    s_item[slot] = item;
    if (item < total) {
      const int m = WENOFD_IX(b.guard, owner(prefix, n, item), n);
      s_m[slot] = m;
      s_on[slot] = __ldcg(&b.members[m].ctrl->active);
    }
  };
  if (threadIdx.x == 0) resolve(0, int(atomicAdd(counter, 1u)));
  __syncthreads();
  int cur = -1;
  for (int it = 0;; ++it) {
    const int slot = it & 1;
    const int item = s_item[slot];
    if (item >= total) break;
    const int m = s_m[slot];
    const bool on = s_on[slot] != 0;
    int next = 0;
    if (threadIdx.x == 0) next = int(atomicAdd(counter, 1u));
    if (on) {
      if (m != cur) {  // block-uniform: stage the member record
        const unsigned *src = reinterpret_cast<const unsigned *>(&b.members[m]);
        unsigned *dst = reinterpret_cast<unsigned *>(&sM);
        for (int w = threadIdx.x; w < int(sizeof(BatchMember) / 4); w += blockDim.x) dst[w] = __ldg(&src[w]);
        __syncthreads();
        cur = m;
      }
      f(item - __ldg(&prefix[m]), static_cast<const BatchMember &>(sM));
    }
    if (threadIdx.x == 0) resolve(slot ^ 1, next);
    __syncthreads();
  }
}

__device__ __forceinline__ int runnable(const Ctrl *c) {
  return (!__ldcg(&c->done) && !__ldcg(&c->error) && __ldcg(&c->steps) < __ldcg(&c->max_steps)) ? 1 : 0;
}

// ROUTE (FP32 only): the learned form; each member's stage tiles route
// their faces with the member's flags (BatchMember::flags), which the
// batched indicator launch between two launches of this kernel writes.
template <typename T, int SCHEME, int TI, int NT, bool WITHHOLD = false, bool ROUTE = false>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? (NT <= 256 ? 3 : 1) : 1) k_batch(BatchArgs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BatchMember sM;
  constexpr int TJ = 32;
  constexpr bool F32 = sizeof(T) == 4;
  const int n = b.n;
  int nbar = 0;  // barriers passed in this launch (the WITHHOLD hook's index)
  auto barrier = [&](auto last) { grid_barrier<WITHHOLD>(b, last, nbar++); };

  // the loop condition of src/WENOFD.cpp:213, per member; FP32 forms: whether
  // every member that can step holds valid tile bounds (BatchArgs::all_bounds)
  auto gate = [&]() {
    int all = 1;
    for (int base = 0; base < n; base += NT) {
      const int m = base + int(threadIdx.x);
      int ok = 1;
      if (m < n) {
        Ctrl *c = b.members[m].ctrl;
        const int can = runnable(c);
        c->active = can;
        ok = !can || __ldcg(&c->bounds_valid);
      }
      all &= __syncthreads_and(ok);
    }
    if (F32 && threadIdx.x == 0) *b.all_bounds = all;
  };
  // dt = min(1, cfl / max s), clipped to t_end - now (src/WENOFD.cpp:401,
  // 426-435); NaN -> error NAN_DT (lines 437-442)
  auto finalize = [&]() {
    for (int m = threadIdx.x; m < n; m += NT) {
      Ctrl *c = b.members[m].ctrl;
      if (!__ldcg(&c->active)) continue;
      const double ms = __longlong_as_double((long long)__ldcg(&c->max_s_bits));
      c->max_s_bits = 0ull;
      c->screen_bits = 0u;
      if (__ldcg(&c->nan_flag)) {
        c->nan_flag = 0;
        c->error = 3;
        c->active = 0;
        continue;
      }
      const double now = __ldcg(&c->now), t_end = __ldcg(&c->t_end);
      const double cand = __ldcg(&c->cfl) / ms;
      double timestep = 1.0;
      if (!(cand > timestep)) timestep = cand;
      if (t_end - now < timestep) timestep = t_end - now;
      if (timestep != timestep) {
        c->error = 3;
        c->active = 0;
        continue;
      }
      c->dt = timestep;
    }
  };

  barrier(gate);
  for (int step = 0; step < b.nsteps; ++step) {
    unsigned *cnt = b.counters + step * kBatchPhases;
    // time-step reduction over each member's interior nodes
    auto node = [&](const BatchMember &M, long long t, double &rho, double &mu, double &mv, double &E) {
      const int i = int(t / M.g.ny), j = int(t - (t / M.g.ny) * M.g.ny);
      const long long p = WENOFD_NODE(M.g, i, j);
      rho = __ldcg(&M.S[p]);
      mu = __ldcg(&M.S[M.g.plane + p]);
      mv = __ldcg(&M.S[2 * M.g.plane + p]);
      E = __ldcg(&M.S[3 * M.g.plane + p]);
    };
    auto exact_pass = [&](int local, const BatchMember &M) {
      const long long first = (long long)local * kPtChunk;
      const long long npts = (long long)M.g.nx * M.g.ny;
      float L = 0.0f;
      if constexpr (F32) L = __uint_as_float(__ldcg(&M.ctrl->screen_bits));
      double smax = 0.0;
      int nan_seen = 0;
      SpeedMemo memo;
      for (long long t = first + threadIdx.x; t < first + kPtChunk && t < npts; t += NT) {
        double rho, mu, mv, E;
        node(M, t, rho, mu, mv, E);
        if constexpr (F32) {  // refine: only nodes that can hold the maximum
          float s32, e;
          screen_speed(M.g, rho, mu, mv, E, s32, e);
          if (!(s32 + e >= L)) continue;
        }
        if (memo.repeat(rho, mu, mv, E)) continue;
        const double s = exact_speed(M.g, rho, mu, mv, E);
        if (s != s) nan_seen = 1;
        else if (s > smax) smax = s;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double other = __shfl_xor_sync(0xffffffffu, smax, o);
        smax = other > smax ? other : smax;
        nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
      }
      if ((threadIdx.x & 31) == 0) {
        atomicMax(&M.ctrl->max_s_bits, (unsigned long long)__double_as_longlong(smax));
        if (nan_seen) atomicOr(&M.ctrl->nan_flag, 1);
      }
    };
    // FP32 forms, members with valid tile bounds: the exact pass over the
    // tiles whose upper bound reaches L (the last stage raised screen_bits to
    // the member's maximum lower bound), a warp per tile over every member's
    // tiles in a fixed stride (k_dt_refine's tile pass)
    auto tile_refine = [&]() {
      const int lane = threadIdx.x & 31;
      const int warps = int(gridDim.x) * (NT / 32);
      const int total = __ldg(&b.work.tile_prefix[n]);
      for (int t = int(blockIdx.x) * (NT / 32) + int(threadIdx.x >> 5); t < total; t += warps) {
        const int m = WENOFD_IX(b.guard, owner(b.work.tile_prefix, n, t), n);
        const BatchMember &M = b.members[m];
        Ctrl *c = M.ctrl;
        if (!__ldcg(&c->active) || !__ldcg(&c->bounds_valid)) continue;  // warp-uniform
        const float L = __uint_as_float(__ldcg(&c->screen_bits));
        const int local = t - __ldg(&b.work.tile_prefix[m]);
        const int tiles_j = M.tiles_j;
        // (bounds are allocated for tiles of 15 rows, the most tiles)
        if (__ldcg(&M.tile_bounds[WENOFD_IX(b.guard, local, ((M.g.nx + 14) / 15) * tiles_j)]).y < L) continue;
        const int i0 = (local / tiles_j) * TI, j = (local - (local / tiles_j) * tiles_j) * TJ + lane;
        const int i1 = i0 + TI < M.g.nx ? i0 + TI : M.g.nx;
        double smax = 0.0;
        int nan_seen = 0;
        SpeedMemo memo;
        if (j < M.g.ny) {
          for (int i = i0; i < i1; ++i) {
            double rho, mu, mv, E;
            node(M, (long long)i * M.g.ny + j, rho, mu, mv, E);
            float s32, e;
            screen_speed(M.g, rho, mu, mv, E, s32, e);
            if (s32 + e >= L && !memo.repeat(rho, mu, mv, E)) {
              const double sp = exact_speed(M.g, rho, mu, mv, E);
              if (sp != sp) nan_seen = 1;
              else if (sp > smax) smax = sp;
            }
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double other = __shfl_xor_sync(0xffffffffu, smax, o);
          smax = other > smax ? other : smax;
          nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
        }
        if (lane == 0) {
          atomicMax(&c->max_s_bits, (unsigned long long)__double_as_longlong(smax));
          if (nan_seen) atomicOr(&c->nan_flag, 1);
        }
      }
    };
    // members without valid bounds: node chunks (FP64 form: every member)
    auto chunk_pass = [&](int local, const BatchMember &M) {
      if constexpr (F32)
        if (__ldcg(&M.ctrl->bounds_valid)) return;  // block-uniform: the tile pass covers it
      exact_pass(local, M);
    };
    if constexpr (F32) {
      const bool all_valid = __ldcg(b.all_bounds) != 0;  // grid-uniform (set before the last release)
      if (!all_valid) {
        // screen of the members without valid bounds: L = max (s32 - e), a
        // lower bound of the member's max s
        for_member_items(b, cnt + 0, b.work.pt_prefix, sM, [&](int local, const BatchMember &M) {
          if (__ldcg(&M.ctrl->bounds_valid)) return;  // block-uniform
          const long long first = (long long)local * kPtChunk;
          const long long npts = (long long)M.g.nx * M.g.ny;
          float lo = 0.0f;
          for (long long t = first + threadIdx.x; t < first + kPtChunk && t < npts; t += NT) {
            double rho, mu, mv, E;
            node(M, t, rho, mu, mv, E);
            float s, e;
            screen_speed(M.g, rho, mu, mv, E, s, e);
            lo = fmaxf(lo, s - e);
          }
          for (int o = 16; o > 0; o >>= 1) lo = fmaxf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
          if ((threadIdx.x & 31) == 0) atomicMax(&M.ctrl->screen_bits, __float_as_uint(lo));
        });
        barrier(Nothing());
        for_member_items(b, cnt + 1, b.work.pt_prefix, sM, chunk_pass);
      }
      tile_refine();
    } else {
      for_member_items(b, cnt + 1, b.work.pt_prefix, sM, exact_pass);
    }
    barrier(finalize);

    // m_now += dt; count++ (src/WENOFD.cpp:213-224), then the next step's
    // gate; after the launch's last step, the host summary
    const bool last_step = step == b.nsteps - 1;
    // FP32 forms, SSP-RK2/3: the last stage screens the nodes it writes
    constexpr bool kFused = F32;
    const bool fused = kFused && b.rk != 0;
    auto step_end = [&]() {
      int alive = 0, err = 0, all = 1;
      for (int base = 0; base < n; base += NT) {
        const int m = base + int(threadIdx.x);
        int can = 0, e = 0;
        if (m < n) {
          Ctrl *c = b.members[m].ctrl;
          if (__ldcg(&c->active)) {
            const double now = __ldcg(&c->now) + __ldcg(&c->dt);
            c->now = now;
            c->steps = __ldcg(&c->steps) + 1;
            c->done = !(fabs(now - __ldcg(&c->t_end)) > 1e-9);
            c->bounds_valid = fused ? 1 : 0;
          }
          can = runnable(c);
          c->active = can;
          e = __ldcg(&c->error) != 0;
        }
        alive += __syncthreads_count(can);
        err |= __syncthreads_or(e);
        all &= __syncthreads_and(!can || (m < n && __ldcg(&b.members[m].ctrl->bounds_valid)));
      }
      if (F32 && threadIdx.x == 0) *b.all_bounds = all;
      if (last_step && threadIdx.x == 0) {
        b.status[0] = alive;
        b.status[1] = err;
      }
    };

    // The stages of RKMETH (src/WENOFD.cpp:301-396), buffers as the single
    // solve uses them: SSP-RK3 S -> A -> B -> S; SSP-RK2 S -> A -> S; RK1
    // S -> A, then A's interior copied to S.
    const int nst = b.rk + 1;
    for (int st = 0; st < nst; ++st) {
      for_member_items(b, cnt + 2 + 2 * st, b.work.bc_prefix, sM, [&](int local, const BatchMember &M) {
        double *in = st == 0 ? M.S : (st == 1 ? M.A : M.B);
        const int first = local * kBcChunk, total = bc_entries(M.g);
        for (int e = first + int(threadIdx.x); e < first + kBcChunk && e < total; e += NT)
          bc_fill_entry(M.g, in, M.special, e);
      });
      barrier(Nothing());
      for_member_items(b, cnt + 3 + 2 * st, b.work.tile_prefix, sM, [&](int local, const BatchMember &M) {
        const int ti = WENOFD_IX(M.g.guard, local / M.tiles_j, (M.g.nx + TI - 1) / TI),
                  tj = local - (local / M.tiles_j) * M.tiles_j;
        StageArgs a;
        a.uin = st == 0 ? M.S : (st == 1 ? M.A : M.B);
        a.un = M.S;
        a.uout = st == 0 ? M.A : (st == nst - 1 ? M.S : M.B);
        if (b.rk == 2) {  // SSP-RK3 (src/WENOFD.cpp:369-383)
          a.a = st == 0 ? 1.0 : (st == 1 ? 3.0 / 4.0 : 1.0 / 3.0);
          a.b = st == 0 ? 0.0 : (st == 1 ? 1.0 / 4.0 : 2.0 / 3.0);
          a.c = st == 0 ? 1.0 : (st == 1 ? 1.0 / 4.0 : 2.0 / 3.0);
          a.form = st == 0 ? kFormStage1 : (st == 1 ? kFormRK3Mid : kFormGeneric);
        } else {  // SSP-RK2 (src/WENOFD.cpp:312-350) and RK1 (301-310): (1, 0, 1), then (1/2, 1/2, 1/2)
          a.a = st == 0 ? 1.0 : 0.5;
          a.b = st == 0 ? 0.0 : 0.5;
          a.c = st == 0 ? 1.0 : 0.5;
          a.form = st == 0 ? kFormStage1 : kFormRK2Mid;
        }
        a.dt = &M.ctrl->dt;
        a.active = &M.ctrl->active;
        a.mode = kModeRK;
        a.flags = ROUTE ? M.flags : nullptr;
        if (fused && st == nst - 1) {  // screen the new U^n into the member's tile bounds
          a.bounds = M.tile_bounds;
          a.screen = &M.ctrl->screen_bits;
        }
        if constexpr (F32)
          stage_tile_f32<SCHEME, TI, TJ, NT, ROUTE, true, !(NT <= 256)>(M.g, a, ti * TI, tj * TJ, smem_raw, local);
        else stage_tile_f64<SCHEME, TI, TJ, NT, true>(M.g, a, ti * TI, tj * TJ, smem_raw);
      });
      if (st < nst - 1 || b.rk == 0) barrier(Nothing());
      else barrier(step_end);
    }
    if (b.rk == 0) {  // RK1: U^{n+1} = A, interior nodes
      for_member_items(b, cnt + 4, b.work.pt_prefix, sM, [&](int local, const BatchMember &M) {
        const long long first = (long long)local * kPtChunk;
        const long long npts = (long long)M.g.nx * M.g.ny;
        for (long long t = first + threadIdx.x; t < first + kPtChunk && t < npts; t += NT) {
          const int i = int(t / M.g.ny), j = int(t - (t / M.g.ny) * M.g.ny);
          const long long p = WENOFD_NODE(M.g, i, j);
#pragma unroll
          for (int r = 0; r < 4; ++r) M.S[r * M.g.plane + p] = __ldcg(&M.A[r * M.g.plane + p]);
        }
      });
      barrier(step_end);
    }
  }
  // the ghost nodes of U^n for the indicator launch that follows (members
  // that can step; `active` was set by the last gate)
  if (b.fill_end) {
    for_member_items(b, b.counters + b.nsteps * kBatchPhases, b.work.bc_prefix, sM,
                     [&](int local, const BatchMember &M) {
                       const int first = local * kBcChunk, total = bc_entries(M.g);
                       for (int e = first + int(threadIdx.x); e < first + kBcChunk && e < total; e += NT)
                         bc_fill_entry(M.g, M.S, M.special, e);
                     });
  }
}

// Cooperative launch of one kernel instance.  With b.members null: sets the
// kernel's shared-memory limit and returns in *grid the SM count times the
// resident blocks per SM (occupancy, or blocks_per_sm if smaller); call it
// outside stream capture.  Otherwise launches *grid blocks, which must come
// from that query.
template <typename T, int TI, int NT, bool WITHHOLD = false, bool ROUTE = false>
cudaError_t launch_batch_tile(const BatchArgs &b, int scheme, int blocks_per_sm, cudaStream_t s, int *grid) {
  constexpr size_t smem = stage_smem_bytes<T, TI, 32, false, NT>();
  void (*fn)(BatchArgs) = nullptr;
  if constexpr (WITHHOLD) {
    if (scheme != kWenoZ) return cudaErrorInvalidValue;
    fn = k_batch<T, kWenoZ, TI, NT, true>;
  } else {
    switch (scheme) {
      case kWenoJS: fn = k_batch<T, kWenoJS, TI, NT, false, ROUTE>; break;
      case kWenoZ: fn = k_batch<T, kWenoZ, TI, NT, false, ROUTE>; break;
      case kWenoZP: fn = k_batch<T, kWenoZP, TI, NT, false, ROUTE>; break;
      case kWenoZPI: fn = k_batch<T, kWenoZPI, TI, NT, false, ROUTE>; break;
      default: return cudaErrorInvalidValue;
    }
  }
  if (!grid) return cudaErrorInvalidValue;
  cudaError_t e;
  if (!b.members) {
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) != cudaSuccess)
      return e;
    int dev = 0, sms = 0, occ = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, NT, smem)) != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    *grid = sms * (blocks_per_sm > 0 && blocks_per_sm < occ ? blocks_per_sm : occ);
    return cudaSuccess;
  }
  if (*grid < 1) return cudaErrorInvalidConfiguration;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(*grid);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BatchArgs args = b;
  return cudaLaunchKernelEx(&cfg, fn, args);
}

}  // namespace dev
}  // namespace wenofd
