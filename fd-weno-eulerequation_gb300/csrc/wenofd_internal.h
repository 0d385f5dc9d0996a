// Internal declarations shared by the CUDA translation units and the C-ABI
// implementation.  Not installed; the public boundary is include/wenofd.h.
#pragma once

#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
#include <stdint.h>

namespace wenofd {

constexpr int kGhost = 4;  // ghost nodes per side (src/WENOFD.cpp:36)

// BOUNDARYTYPE (utils/equations.hpp:45-51)
enum Boundary { kPeriod = 0, kSlip = 1, kSpecial = 2, kSymmetric = 3 };
// SCHEMETYPE (utils/equations.hpp:15-21)
enum Scheme { kWenoJS = 0, kWenoZ = 1, kWenoZP = 2, kWenoZPI = 3 };

// Device layout of one state array: [4][nxt][pitch] float64, element
// (r, ei, ej) at r*plane + ei*pitch + ej, ej (y) fastest, the reference's
// m_Uh[ei][ej].vector[r] in structure-of-arrays form.  Interior nodes are
// ei in [4, 4+nx), ej in [4, 4+ny).  pitch >= ny+8 is a multiple of 32
// elements so every row starts on a 256-byte boundary.
struct Geom {
  int nx, ny;     // interior nodes (ELEMNUMX, ELEMNUMY)
  int nxt, nyt;   // nx + 8, ny + 8
  int pitch;      // row pitch in elements
  long long plane;
  double dx, dy, gamma;
  double zp_lambda;  // pow(dx, 2/3), WENO-ZP (include/Utility.hpp:531; dx also in y, src/WENOFD.cpp:836)
  int bc_left, bc_right, bc_y;  // y uses the bottom condition on both sides (src/WENOFD.cpp:1009)
  int gravity;                  // RTI source term (src/WENOFD.cpp:800-821)
  // FP32-form constants, rounded once on the host: gamma, zp_lambda, 1/dx, 1/dy
  float gamma32, zpl32, inv_dx32, inv_dy32;
  // Bounds-checked build: the device guard record of this device
  // (guard.cuh); null in the release build.
  unsigned long long *guard;
};

// Device-resident control block of the time loop.  All fields are written
// by single-thread control kernels or by the host between launches.
struct Ctrl {
  double now, t_end, cfl, dt;
  unsigned long long max_s_bits;  // max over nodes of lx/dx + ly/dy, as IEEE bits (all >= 0)
  unsigned screen_bits;           // FP32 lower bound of that max (two-pass reduction), as bits
  long long steps, max_steps;
  int active;    // this step runs (set per step)
  int done;      // |now - t_end| <= 1e-9 (src/WENOFD.cpp:213)
  int nan_flag;  // a NaN wave speed was seen by the reduction
  int error;     // sticky wenofd_status of the device loop
  // FP32 forms: the per-tile screen bounds of the current U^n (written by
  // the last RK stage of the previous step, with their maximum lower bound
  // in screen_bits) are valid, so the time-step reduction skips its screen
  // pass.  Cleared at the start of every advance and by every other entry.
  int bounds_valid;
  // Learned form: steps counted from here (set at the start of every
  // advance) decide which steps run the indicator (INDICATOR_INTERVAL).
  long long ind_base;
};

// Arguments of one RK stage launch.  uin is read with a 3-node halo (its
// ghosts must be filled); un is read only at the node itself and may alias
// uout (the last stage writes U^{n+1} over U^n in place).
struct StageArgs {
  const double *uin;
  const double *un;
  double *uout;
  double a, b, c;      // uout = a*un + b*uin + c*dt*rhs  (src/WENOFD.cpp:391-394)
  const double *dt;    // device pointer (Ctrl::dt)
  const int *active;   // device pointer (Ctrl::active); 0 -> return
  int mode;            // kModeRK or kModeRHS (uout = rhs)
  // Learned form only: per-node troubled-cell flags, [nxt][pitch] bytes,
  // ghosts 1.  A face takes characteristic WENO-Z when any of the four nodes
  // around it along its line is flagged, else the linear upwind flux.
  const unsigned char *flags = nullptr;
  // FP32 forms, last stage of a step: per-tile (max s32 - e, max s32 + e)
  // of the time-step screen over the nodes just written, and the running
  // maximum lower bound (Ctrl::screen_bits).
  float2 *bounds = nullptr;
  unsigned *screen = nullptr;
  // Which combination (a, b, c) is, from rk_form(): the FP32 tiles branch
  // on this integer instead of comparing the FP64 coefficients on the
  // device, where every FP64 compare issues on the 1/64-rate FP64 pipe.
  int form = 0;
  // FP32 per-solve tiles: set to 1 if a tile's TMA load wait gave up
  // (the host reports WENOFD_TIMEOUT).
  int *wait_error = nullptr;
};

// TMA descriptors of one FP32 stage launch: `u` tiles the input state
// [4][nxt][pitch] FP64 in boxes of 40 columns x (TI + 6) rows x 4 planes
// (the tile's 38 halo columns from an even, 16-byte aligned first column);
// `flags` tiles the learned form's node flags [nxt][pitch] bytes in boxes of
// 48 columns x (TI + 4) rows.
struct StageTma {
  CUtensorMap u;
  CUtensorMap flags;
};
// Encodes the maps of one state array (and of the flag array, if not null)
// for stage tiles of tile_i rows (FP32 tiles 15 or 31, FP64 tiles 15 or 7).
cudaError_t make_stage_tma(const Geom &g, const double *state, const unsigned char *flags, int tile_i,
                           StageTma *out);
enum { kModeRK = 0, kModeRHS = 1 };
// RK stage forms: a = 1, b = 0 on U^n itself (stage 1); SSP-RK3's middle
// stage (3/4, 1/4, 1/4); RK2's second stage (1/2, 1/2, 1/2); any other.
enum { kFormGeneric = 0, kFormStage1 = 1, kFormRK3Mid = 2, kFormRK2Mid = 3 };
__host__ __device__ inline int rk_form(double a, double b, double c, const double *uin, const double *un) {
  if (a == 1.0 && b == 0.0 && un == uin) return kFormStage1;
  if (a == 0.75 && b == 0.25 && c == 0.25) return kFormRK3Mid;
  if (a == 0.5 && b == 0.5 && c == 0.5) return kFormRK2Mid;
  return kFormGeneric;
}

Geom make_geom(int nx, int ny, double dx, double dy, double gamma, double zp_lambda, int bc_left,
               int bc_right, int bc_y, int gravity);
// Bounds-checked build: the current device's guard record (guard.cuh),
// kGuardWords words allocated and zeroed on first use; null in the release
// build.
unsigned long long *guard_record();
// The guard self-test kernel (aux_kernels.cu): one guarded access one past
// the end of buf[4], recorded in rec (kGuardWords words); returns the
// self-test's source site.
cudaError_t launch_guard_selftest(unsigned long long *rec, int *buf, unsigned long long *site, cudaStream_t s);

// stage kernels (stage_fp64.cu: parity arithmetic; stage_fp32.cu: FP32 form,
// routed by a.flags when it is set); both take their halo by TMA through the
// maps in `tma` (make_stage_tma for the same tile height)
cudaError_t launch_stage_fp64(const Geom &g, const StageArgs &a, const StageTma &tma, int scheme, int tile_i,
                              cudaStream_t s);
// The FP32 tiles load their halo by TMA: `tma` holds the maps of a.uin (and
// of a.flags) for tiles of tile_i rows.
cudaError_t launch_stage_fp32(const Geom &g, const StageArgs &a, const StageTma &tma, int scheme, int tile_i,
                              cudaStream_t s);

// batch_fp64.cu / batch_fp32.cu: the persistent batched kernel
// (batch_kernel.cuh).  tile_i 0 = default; grid receives the launch's block
// count; with b.members null nothing is launched (grid query only).
// One member of a batch (device-resident array of these).
struct BatchMember {
  Geom g;
  double *S, *A, *B;
  const double *special;
  Ctrl *ctrl;
  int tiles_j;  // tiles along y; tiles along x = ceil(nx / TI)
  // Learned form: the member's routing flags ([nxt][pitch], ghosts 1) and
  // packed indicator weights (null: no indicator loaded, the flags stay as
  // they are), its logit threshold, and the bands of indicator tiles per
  // strip (indicator work items = strips x bands).
  unsigned char *flags;
  const void *ind_weights;
  float ind_logit_threshold;
  float ind_guard;  // INDICATOR_GUARD (0: off)
  int ind_bands;
  // FP32 forms: the member's per-stage-tile time-step screen bounds (tiles
  // of the batch's tile height), written by the last stage of a step; null
  // for FP64 members.
  float2 *tile_bounds;
};

// Exclusive prefix sums of work items per member (n+1 entries each).
struct BatchWork {
  const int *tile_prefix;  // stage tiles (depends on TI)
  const int *bc_prefix;    // ghost-fill chunks of kBcChunk entries
  const int *pt_prefix;    // time-step chunks of kPtChunk nodes
  const int *ind_prefix;   // learned form: indicator runs (strip, band of rows)
};

constexpr int kBcChunk = 256;
constexpr int kPtChunk = 4096;
constexpr int kBatchPhases = 8;  // work counters per step: dt x 2, (bc, stage) x 3 (RK1: + copy)
constexpr unsigned kBarrierLimit = 1u << 24;
// Poll limit of the barrier in the withholding test instance (a few ms).
constexpr unsigned kBarrierTestLimit = 1u << 12;

struct BatchArgs {
  BatchMember *members;
  BatchWork work;
  int n;               // members
  int nsteps;          // steps per launch
  int rk;              // RKMETH of every member: 0 RK1, 1 SSP-RK2, 2 SSP-RK3
  unsigned *counters;  // nsteps * kBatchPhases work counters, zeroed before the launch
  unsigned *barrier;   // [0] arrivals (zero before the launch), [1] generation
  int *error;          // set if a barrier wait gave up
  int *status;         // after the launch: [0] members that can still step, [1] any member error
  // After the launch's last step, fill the ghost nodes of every member that
  // can still step (its U^n, S): the learned form's indicator, launched
  // between two batched launches, reads the next step's stage-1 input with
  // its ghosts, as the single solve's indicator does.  Uses the counters of
  // step nsteps (the counter array then holds nsteps + 1 steps).
  int fill_end = 0;
  // FP32 forms: set by the block that releases a barrier when every member
  // that can step holds valid tile bounds of its U^n (Ctrl::bounds_valid):
  // the next time-step reduction then skips its screen and node passes and
  // refines only the candidate tiles.
  int *all_bounds = nullptr;
  // Test instance only (k_batch with WITHHOLD): block `hold_block` skips its
  // arrival at the launch's barrier number `hold_barrier` (counted from 0).
  int hold_block = -1, hold_barrier = -1;
  // Bounds-checked build: the guard record (null in the release build).
  unsigned long long *guard = nullptr;
};

// Per-member summary gathered for the host in one copy.
struct BatchMemberStatus {
  double now;
  long long steps;
  int error, done;
};

cudaError_t launch_batch_fp64(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                              int *grid);
cudaError_t launch_batch_fp32(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                              int *grid);
// batch_learned.cu: the FP32 batched kernel with routed stage tiles (the
// learned form; members' flags route each face).
cudaError_t launch_batch_learned(const BatchArgs &b, int scheme, int tile_i, int blocks_per_sm, cudaStream_t s,
                                 int *grid);
// The FP64 WENO-Z batched kernel (tile 15) built with the withholding test
// hook and a short barrier poll limit: exercises the barrier's give-up path.
// Never launched by wenofd_batch_advance unless wenofd_batch_test_withhold
// armed it.
cudaError_t launch_batch_fp64_withhold(const BatchArgs &b, cudaStream_t s, int *grid);
cudaError_t launch_batch_setup(BatchMember *members, int n, long long max_steps, cudaStream_t s);
cudaError_t launch_batch_gather(const BatchMember *members, int n, BatchMemberStatus *out, cudaStream_t s);

// learned.cu: indicator features, labels, tensor-core inference
size_t indicator_weights_bytes();
void pack_indicator_weights(const float *params, void *host_out);
cudaError_t launch_features(const Geom &g, const double *U, float *feat, cudaStream_t s);
// labels: 1 where a face of the node has a WENO-Z weight deviation above `deviation`
cudaError_t launch_labels(const Geom &g, const double *U, unsigned char *labels, double deviation, cudaStream_t s);
// Balanced sampling of training nodes (wenofd_indicator_sample): positives
// among `labels`; per-block kept counts (sample_blocks() entries) for
// thresholds thr0 / thr1 (out of 2^32) on the negative / positive class;
// then the kept nodes in node order from per-block row offsets: node index
// into cells[row], label into y[row] (0.0 / 1.0), features into x[row][50]
// (rows < capacity; `rows` = the number written).
int sample_blocks();
cudaError_t launch_count_positive(const unsigned char *labels, long long n, unsigned long long *count,
                                  cudaStream_t s);
cudaError_t launch_sample_count(const unsigned char *labels, long long n, unsigned long long seed,
                                unsigned long long thr0, unsigned long long thr1, unsigned *block_count,
                                cudaStream_t s);
cudaError_t launch_sample_write(const Geom &g, const double *U, const unsigned char *labels, unsigned long long seed,
                                unsigned long long thr0, unsigned long long thr1, const long long *offsets,
                                long long capacity, long long rows, long long *cells, float *x, float *y,
                                cudaStream_t s);
// With ctrl set (the time loop), the indicator runs only on steps whose
// count since Ctrl::ind_base is a multiple of `interval`; the flags of the
// last run route the steps in between.
// guard > 0 (INDICATOR_GUARD): a node is also flagged when the range of its
// 5x5 density or pressure window exceeds guard times the centre value.
cudaError_t launch_indicator(const Geom &g, const double *U, const void *weights, float logit_threshold, float guard,
                             unsigned char *flags, int *error, const int *active, const Ctrl *ctrl, int interval,
                             cudaStream_t s);
// Indicator runs of a learned batch: one launch over every member that can
// step and has weights loaded (BatchMember::ind_weights), on its U^n (ghosts
// filled), into its flags.  Work items are (member, strip, band of rows) from
// ind_prefix, claimed through *counter (zeroed before the launch).  The
// tiles and arithmetic are the single solve's, so the flags are too.
// `items` = ind_prefix[n] (the grid is no larger).
cudaError_t launch_indicator_batch(const BatchMember *members, const int *ind_prefix, int n, unsigned *counter,
                                   int *error, unsigned long long *guard, int items, cudaStream_t s);
// Rows of 4-node indicator tiles per batched indicator work item.
constexpr int kIndBandTiles = 16;

// aux_kernels.cu
cudaError_t launch_bc_fill(const Geom &g, double *U, const double *special, const int *active, cudaStream_t s);
cudaError_t launch_dt_reduce(const Geom &g, const double *U, Ctrl *c, cudaStream_t s);
// Same result, bit for bit, in two passes that keep the FP64 pipe nearly
// idle: an FP32 screen with a rigorous error bound, then FP64 only where a
// node can hold the maximum.
// With bounds (per-tile screen bounds of stage tiles `tile_i` x 32) and
// Ctrl::bounds_valid set, the screen pass is skipped and the refine pass
// visits only the tiles whose upper bound reaches the maximum lower bound.
cudaError_t launch_dt_reduce_two_pass(const Geom &g, const double *U, Ctrl *c, const float2 *bounds, int tile_i,
                                      cudaStream_t s);
cudaError_t launch_ctrl_open(Ctrl *c, cudaStream_t s);
cudaError_t launch_step_begin(Ctrl *c, cudaStream_t s);
cudaError_t launch_dt_finalize(Ctrl *c, cudaStream_t s);
// fused: the step's last stage wrote screen bounds of the new U^n
cudaError_t launch_step_end(Ctrl *c, int fused, cudaStream_t s);
cudaError_t launch_set_dt(Ctrl *c, double dt, cudaStream_t s);
cudaError_t launch_set_time(Ctrl *c, double now, cudaStream_t s);
cudaError_t launch_advance_setup(Ctrl *c, long long max_steps, cudaStream_t s);
cudaError_t launch_copy_interior(const Geom &g, const double *src, double *dst, const int *active, cudaStream_t s);
// FP64 reductions over interior nodes into partials[nblk*4] then out[4]
// (deterministic order).  kind 0: {Linf, L1, L2} of density against the
// smooth case's exact solution at time t (xl, yl: domain origin);
// kind 1: sums of the 4 conserved variables.
int reduce_blocks();
// outputAve's variables (rho, u, v, pre, c, E) of every interior node as
// planes of nx * ny doubles (j fastest): planes 0-3 at out03, 4-5 at out45
// (device), FP64 in the reference's order.
cudaError_t launch_output_vars(const Geom &g, const double *U, double *out03, double *out45, cudaStream_t s);
cudaError_t launch_reduce(const Geom &g, const double *U, int kind, double t, double xl, double yl,
                          double *partials, double *out, cudaStream_t s);

}  // namespace wenofd
