// C ABI of batches (include/wenofd.h, "Batches"): many independent solves
// advanced by one persistent cooperative kernel per launch (batch_kernel.cuh),
// replayed from a captured CUDA graph, with a timing autotuner over the
// kernel's tile height and resident blocks per SM.
//
// A batch holds no state of its own beyond its work plan: the members'
// device arrays and control blocks are the ones their handles own, so a
// member's results and time are read through its own handle.
//
// Learned-form batches alternate two launches: the batched tensor-core
// indicator over every member's U^n (learned.cu), then the batched kernel
// for INDICATOR_INTERVAL steps routed by those flags, whose launch ends with
// the ghost fill the next indicator run reads.  An advance call starts with
// a launch of no steps that fills the ghosts, so the indicator runs on the
// first step of every call and then every INDICATOR_INTERVAL steps, as in
// the single solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/wenofd.h"
#include "solver.h"
#include "trace.h"
#include "wenofd_internal.h"

using wenofd::BatchArgs;
using wenofd::BatchMember;
using wenofd::BatchMemberStatus;
using wenofd::Ctrl;

struct wenofd_batch {
  int device = 0, n = 0, precision = 0, scheme = 0, rk = 2;
  // learned form: indicator runs every `interval` steps
  bool learned = false;
  int interval = 1;
  std::vector<wenofd_solver *> members;
  cudaStream_t stream = nullptr;
  // work plan (device)
  BatchMember *d_members = nullptr;
  int *d_prefix = nullptr;  // tile, bc, node-chunk, indicator-run prefix sums, (n+1) each
  int ind_items = 0;        // indicator runs in all
  unsigned *d_counters = nullptr;
  int counter_steps = 0;
  unsigned *d_ind_counter = nullptr;  // the batched indicator's work counter
  unsigned *d_barrier = nullptr;
  int *d_flags = nullptr;  // [0] barrier gave up, [1..2] status, [3] indicator wait gave up, [4] all bounds valid
  BatchMemberStatus *d_gather = nullptr;
  // host mirrors (pinned)
  int *h_flags = nullptr;
  BatchMemberStatus *h_gather = nullptr;
  // configuration
  int tile_i = 15, blocks_per_sm = 0, steps_setting = 0, steps_per_launch = 1, grid = 0;
  // learned form: (indicator, interval steps) pairs per graph replay, and the
  // members' indicator settings the work plan was made with
  int chunks = 1;
  std::vector<std::pair<const void *, float>> ind_plan;
  cudaGraphExec_t graph = nullptr;
  bool graph_tried = false;  // capture attempted for the current configuration
  long long cells = 0, launches = 0;
  double tuned_ms = 0.0;
  // wenofd_batch_test_withhold: the next advance's first launch runs the
  // withholding test instance with these (block, barrier); -1: not armed
  int hold_block = -1, hold_barrier = -1;
};

namespace {

int fail(int code, const std::string &msg) {
  wenofd::set_last_error(msg);
  return code;
}

#define BATCH_TRY(expr)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(WENOFD_CUDA_ERROR, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

bool tile_allowed(int precision, int tile_i) {
  if (tile_i == 0 || tile_i == 15) return true;
  return precision == WENOFD_FP64 ? tile_i == 7 : tile_i == 31;
}

BatchArgs make_args(const wenofd_batch *b, int nsteps) {
  BatchArgs a{};
  a.members = b->d_members;
  a.work.tile_prefix = b->d_prefix;
  a.work.bc_prefix = b->d_prefix + (b->n + 1);
  a.work.pt_prefix = b->d_prefix + 2 * (b->n + 1);
  a.work.ind_prefix = b->d_prefix + 3 * (b->n + 1);
  a.n = b->n;
  a.nsteps = nsteps;
  a.rk = b->rk;
  a.counters = b->d_counters;
  a.barrier = b->d_barrier;
  a.error = b->d_flags;
  a.status = b->d_flags + 1;
  a.all_bounds = b->d_flags + 4;
  a.guard = wenofd::guard_record();
  return a;
}

// With a.members null: sets the kernel's attributes and returns its grid
// (outside any capture); else launches on the configured grid.
cudaError_t launch_kernel(const wenofd_batch *b, const BatchArgs &a, int *grid) {
  if (b->precision == WENOFD_FP64)
    return wenofd::launch_batch_fp64(a, b->scheme, b->tile_i, b->blocks_per_sm, b->stream, grid);
  if (b->learned) return wenofd::launch_batch_learned(a, b->scheme, b->tile_i, b->blocks_per_sm, b->stream, grid);
  return wenofd::launch_batch_fp32(a, b->scheme, b->tile_i, b->blocks_per_sm, b->stream, grid);
}

// One launch of nsteps steps: zero the work counters and the barrier's
// arrival count, then the cooperative kernel.  fill_end: the launch ends
// with the ghost fill of U^n (learned form), which takes the counters of
// one more step.
int enqueue_launch(wenofd_batch *b, int nsteps, bool fill_end = false) {
  const int counted = nsteps + (fill_end ? 1 : 0);
  BATCH_TRY(cudaMemsetAsync(b->d_counters, 0, size_t(counted) * wenofd::kBatchPhases * sizeof(unsigned), b->stream));
  BATCH_TRY(cudaMemsetAsync(b->d_barrier, 0, sizeof(unsigned), b->stream));
  int grid = b->grid;
  BatchArgs a = make_args(b, nsteps);
  a.fill_end = fill_end ? 1 : 0;
  BATCH_TRY(launch_kernel(b, a, &grid));
  return WENOFD_OK;
}

// Learned form: the batched indicator over every member that can step.
int enqueue_indicator(wenofd_batch *b) {
  BATCH_TRY(cudaMemsetAsync(b->d_ind_counter, 0, sizeof(unsigned), b->stream));
  BATCH_TRY(wenofd::launch_indicator_batch(b->d_members, b->d_prefix + 3 * (b->n + 1), b->n, b->d_ind_counter,
                                           b->d_flags + 3, wenofd::guard_record(), std::max(1, b->ind_items),
                                           b->stream));
  return WENOFD_OK;
}

// Learned form: the launch of no steps that opens an advance (gate, then the
// ghost fill of U^n for the first indicator run).
int enqueue_prologue(wenofd_batch *b) { return enqueue_launch(b, 0, true); }

// Learned form: `chunks` pairs of (indicator, `interval` steps).
int enqueue_chunks(wenofd_batch *b, int chunks, int last_steps = 0) {
  for (int k = 0; k < chunks; ++k) {
    if (int rc = enqueue_indicator(b)) return rc;
    const int steps = (k == chunks - 1 && last_steps > 0) ? last_steps : b->interval;
    if (int rc = enqueue_launch(b, steps, true)) return rc;
  }
  return WENOFD_OK;
}

// nsteps steps of every member as the batch runs them: one launch, or for
// the learned form the prologue and indicator/step pairs.
int enqueue_run(wenofd_batch *b, int nsteps) {
  if (!b->learned) return enqueue_launch(b, nsteps);
  if (int rc = enqueue_prologue(b)) return rc;
  const int chunks = (nsteps + b->interval - 1) / b->interval;
  const int rem = nsteps - (chunks - 1) * b->interval;
  return enqueue_chunks(b, chunks, rem);
}

// Work counters for launches of up to nsteps steps (and the end-of-launch
// ghost fill of the learned form).
int ensure_counters(wenofd_batch *b, int nsteps) {
  nsteps += 1;
  if (nsteps <= b->counter_steps) return WENOFD_OK;
  if (b->d_counters) cudaFree(b->d_counters);
  b->d_counters = nullptr;
  b->counter_steps = 0;
  BATCH_TRY(cudaMalloc(&b->d_counters, size_t(nsteps) * wenofd::kBatchPhases * sizeof(unsigned)));
  b->counter_steps = nsteps;
  return WENOFD_OK;
}

void drop_graph(wenofd_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_tried = false;
}

// Work plan for a tile height: per-member tile counts and the three prefix
// sums, uploaded with the member table.
int plan(wenofd_batch *b, int tile_i) {
  const int TI = tile_i == 0 ? 15 : tile_i;
  std::vector<BatchMember> host(b->n);
  std::vector<int> prefix(4 * size_t(b->n + 1), 0);
  int *tp = prefix.data(), *bp = tp + (b->n + 1), *pp = bp + (b->n + 1), *ip = pp + (b->n + 1);
  b->ind_plan.assign(b->n, {nullptr, 0.0f});
  for (int m = 0; m < b->n; ++m) {
    const wenofd_solver *s = b->members[m];
    BatchMember &M = host[m];
    M.g = s->g;
    M.S = s->S;
    M.A = s->A;
    M.B = s->B;
    M.special = s->special;
    M.ctrl = s->ctrl;
    M.tiles_j = int(ceil_div(s->ny, 32));
    // learned form: indicator tiles are 4 x 32 nodes; each strip of them is
    // cut into bands of about kIndBandTiles tiles
    const bool ind = b->learned && s->ind_ready;
    M.flags = b->learned ? s->flags : nullptr;
    M.ind_weights = ind ? s->ind_weights : nullptr;
    M.ind_logit_threshold = s->ind_logit_threshold;
    M.ind_guard = s->ind_guard;
    M.ind_bands = int(ceil_div(ceil_div(s->nx, 4), wenofd::kIndBandTiles));
    M.tile_bounds = s->tile_bounds;
    b->ind_plan[m] = {M.ind_weights, M.ind_logit_threshold};
    const long long tiles = ceil_div(s->nx, TI) * M.tiles_j;
    const long long bc = ceil_div(8LL * s->nx + 8LL * s->ny + 64, wenofd::kBcChunk);  // ghost entries
    const long long pts = ceil_div((long long)s->nx * s->ny, wenofd::kPtChunk);
    const long long runs = b->learned ? (long long)M.ind_bands * M.tiles_j : 0;
    if (tp[m] + tiles > 0x7fffffffLL || bp[m] + bc > 0x7fffffffLL || pp[m] + pts > 0x7fffffffLL ||
        ip[m] + runs > 0x7fffffffLL)
      return fail(WENOFD_BAD_ARG, "batch too large: more than 2^31 work items in a phase");
    tp[m + 1] = int(tp[m] + tiles);
    bp[m + 1] = int(bp[m] + bc);
    pp[m + 1] = int(pp[m] + pts);
    ip[m + 1] = int(ip[m] + runs);
  }
  b->ind_items = ip[b->n];
  BATCH_TRY(cudaMemcpyAsync(b->d_members, host.data(), host.size() * sizeof(BatchMember), cudaMemcpyHostToDevice,
                            b->stream));
  BATCH_TRY(cudaMemcpyAsync(b->d_prefix, prefix.data(), prefix.size() * sizeof(int), cudaMemcpyHostToDevice,
                            b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return WENOFD_OK;
}

int configure(wenofd_batch *b, int tile_i, int blocks_per_sm, int steps_per_launch) {
  if (!tile_allowed(b->precision, tile_i))
    return fail(WENOFD_BAD_ARG, b->precision == WENOFD_FP64 ? "tile_i must be 0, 7 or 15 for FP64 batches"
                                                            : "tile_i must be 0, 15 or 31 for FP32 batches");
  if (blocks_per_sm < 0 || steps_per_launch < 0 || steps_per_launch > 4096)
    return fail(WENOFD_BAD_ARG, "blocks_per_sm must be >= 0 and steps_per_launch in [0, 4096]");
  drop_graph(b);
  b->tile_i = tile_i == 0 ? 15 : tile_i;
  b->blocks_per_sm = blocks_per_sm;
  b->steps_setting = steps_per_launch;
  // Steps per launch: enough that launch and host-check latency are
  // amortised on small batches, one step on large ones.
  b->steps_per_launch = steps_per_launch > 0
                            ? steps_per_launch
                            : int(std::max(1LL, std::min(64LL, (4LL << 20) / std::max(1LL, b->cells))));
  // learned form: a graph replay runs whole (indicator, interval steps) pairs
  b->chunks = b->learned ? std::max(1, (b->steps_per_launch + b->interval - 1) / b->interval) : 1;
  if (b->learned) b->steps_per_launch = b->chunks * b->interval;
  if (int rc = plan(b, b->tile_i)) return rc;
  if (int rc = ensure_counters(b, b->learned ? b->interval : b->steps_per_launch)) return rc;
  BatchArgs q{};
  b->grid = 0;
  BATCH_TRY(launch_kernel(b, q, &b->grid));  // attributes + grid (members null)
  return WENOFD_OK;
}

// Capture one launch of steps_per_launch steps in a graph (learned form: its
// indicator/step pairs).  If the driver cannot capture a cooperative launch
// the batch launches directly instead (graph = 0 in wenofd_batch_info); the
// kernels are the same.
int ensure_graph(wenofd_batch *b) {
  if (b->graph_tried) return WENOFD_OK;
  b->graph_tried = true;
  cudaStream_t cap = nullptr;
  BATCH_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaStream_t keep = b->stream;
  b->stream = cap;
  cudaGraph_t g = nullptr;
  bool ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  int rc = ok ? (b->learned ? enqueue_chunks(b, b->chunks) : enqueue_launch(b, b->steps_per_launch)) : WENOFD_OK;
  if (ok) ok = cudaStreamEndCapture(cap, &g) == cudaSuccess && rc == WENOFD_OK;
  b->stream = keep;
  cudaStreamDestroy(cap);
  if (ok) ok = cudaGraphInstantiate(&b->graph, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return WENOFD_OK;
}

int launch_step_block(wenofd_batch *b) {
  if (b->graph) {
    BATCH_TRY(cudaGraphLaunch(b->graph, b->stream));
  } else if (int rc = b->learned ? enqueue_chunks(b, b->chunks) : enqueue_launch(b, b->steps_per_launch)) {
    return rc;
  }
  b->launches += b->learned ? 2 * b->chunks : 1;
  return WENOFD_OK;
}

// Learned form: the members' indicator weights or thresholds changed since
// the work plan was made (wenofd_set_indicator on a member).
bool indicator_plan_stale(const wenofd_batch *b) {
  if (!b->learned) return false;
  for (int m = 0; m < b->n; ++m) {
    const wenofd_solver *s = b->members[m];
    const void *w = s->ind_ready ? s->ind_weights : nullptr;
    if (b->ind_plan[m].first != w || b->ind_plan[m].second != s->ind_logit_threshold) return true;
  }
  return false;
}

int gather(wenofd_batch *b) {
  BATCH_TRY(wenofd::launch_batch_gather(b->d_members, b->n, b->d_gather, b->stream));
  b->launches += 1;
  BATCH_TRY(cudaMemcpyAsync(b->h_gather, b->d_gather, size_t(b->n) * sizeof(BatchMemberStatus),
                            cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return WENOFD_OK;
}

int sync_members(wenofd_batch *b) {
  for (wenofd_solver *s : b->members) BATCH_TRY(cudaStreamSynchronize(s->stream));
  return WENOFD_OK;
}

void release(wenofd_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  drop_graph(b);
  cudaFree(b->d_members);
  cudaFree(b->d_prefix);
  cudaFree(b->d_counters);
  cudaFree(b->d_ind_counter);
  cudaFree(b->d_barrier);
  cudaFree(b->d_flags);
  cudaFree(b->d_gather);
  cudaFreeHost(b->h_flags);
  cudaFreeHost(b->h_gather);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace

extern "C" {

int wenofd_batch_create(wenofd_solver *const *members, int n, wenofd_batch **out) {
  WENOFD_TRACE("wenofd_batch_create");
  if (!out) return fail(WENOFD_BAD_ARG, "null output pointer");
  *out = nullptr;
  if (!members || n < 1) return fail(WENOFD_BAD_ARG, "a batch needs at least one member");
  for (int m = 0; m < n; ++m) {
    const wenofd_solver *s = members[m];
    if (!s) return fail(WENOFD_BAD_ARG, "null member handle at index " + std::to_string(m));
    if (s->precision != members[0]->precision || s->scheme != members[0]->scheme || s->rk != members[0]->rk ||
        s->device != members[0]->device)
      return fail(WENOFD_BAD_ARG,
                  "member " + std::to_string(m) + ": PRECISION, SCHEME, RKMETH and DEVICE must match member 0");
    if (s->precision == WENOFD_LEARNED && s->ind_interval != members[0]->ind_interval)
      return fail(WENOFD_BAD_ARG, "member " + std::to_string(m) + ": INDICATOR_INTERVAL must match member 0");
    for (int k = 0; k < m; ++k)
      if (members[k] == s) return fail(WENOFD_BAD_ARG, "member " + std::to_string(m) + " repeats member " + std::to_string(k));
  }
  wenofd_batch *b = new wenofd_batch();
  b->device = members[0]->device;
  b->n = n;
  b->precision = members[0]->precision;
  b->scheme = members[0]->scheme;
  b->rk = members[0]->rk;
  b->learned = b->precision == WENOFD_LEARNED;
  b->interval = b->learned ? members[0]->ind_interval : 1;
  b->members.assign(members, members + n);
  for (const wenofd_solver *s : b->members) b->cells += (long long)s->nx * s->ny;
  auto bail = [&](int rc) {
    release(b);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(b->device)) != cudaSuccess)
    return bail(fail(WENOFD_CUDA_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e)));
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&b->d_members, size_t(n) * sizeof(BatchMember)) == cudaSuccess &&
            cudaMalloc(&b->d_prefix, 4 * size_t(n + 1) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&b->d_ind_counter, sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&b->d_barrier, 2 * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&b->d_flags, 8 * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&b->d_gather, size_t(n) * sizeof(BatchMemberStatus)) == cudaSuccess &&
            cudaMallocHost(&b->h_flags, 4 * sizeof(int)) == cudaSuccess &&
            cudaMallocHost(&b->h_gather, size_t(n) * sizeof(BatchMemberStatus)) == cudaSuccess;
  ok = ok && cudaMemsetAsync(b->d_barrier, 0, 2 * sizeof(unsigned), b->stream) == cudaSuccess &&
       cudaMemsetAsync(b->d_flags, 0, 8 * sizeof(int), b->stream) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return bail(fail(WENOFD_CUDA_ERROR, "batch allocation failed"));
  }
  if (int rc = configure(b, 0, 0, 0)) return bail(rc);
  *out = b;
  return WENOFD_OK;
}

int wenofd_batch_destroy(wenofd_batch *b) {
  release(b);
  return WENOFD_OK;
}

int wenofd_batch_configure(wenofd_batch *b, int tile_i, int blocks_per_sm, int steps_per_launch) {
  if (!b) return fail(WENOFD_BAD_ARG, "null batch handle");
  BATCH_TRY(cudaSetDevice(b->device));
  return configure(b, tile_i, blocks_per_sm, steps_per_launch);
}

int wenofd_batch_get_info(const wenofd_batch *b, wenofd_batch_info *info) {
  if (!b || !info) return fail(WENOFD_BAD_ARG, "null batch handle or output");
  info->members = b->n;
  info->precision = b->precision;
  info->tile_i = b->tile_i;
  info->blocks_per_sm = b->blocks_per_sm;
  info->grid = b->grid;
  info->steps_per_launch = b->steps_per_launch;
  info->graph = b->graph ? 1 : 0;
  info->cells = b->cells;
  info->launches = b->launches;
  info->tuned_ms_per_step = b->tuned_ms;
  return WENOFD_OK;
}

int wenofd_batch_advance(wenofd_batch *b, long long max_steps, long long *steps_done) {
  WENOFD_TRACE("wenofd_batch_advance");
  if (!b) return fail(WENOFD_BAD_ARG, "null batch handle");
  BATCH_TRY(cudaSetDevice(b->device));
  if (int rc = sync_members(b)) return rc;
  if (indicator_plan_stale(b))
    if (int rc = plan(b, b->tile_i)) return rc;
  if (int rc = ensure_graph(b)) return rc;
  BATCH_TRY(cudaMemsetAsync(b->d_flags, 0, 4 * sizeof(int), b->stream));
  BATCH_TRY(wenofd::launch_batch_setup(b->d_members, b->n, max_steps, b->stream));
  b->launches += 1;
  if (int rc = gather(b)) return rc;
  if (b->learned) {
    if (int rc = enqueue_prologue(b)) return rc;
    b->launches += 1;
  }
  std::vector<long long> before(b->n);
  for (int m = 0; m < b->n; ++m) before[m] = b->h_gather[m].steps;
  bool any_error = false;
  for (;;) {
    if (b->hold_block >= 0) {
      // armed by wenofd_batch_test_withhold: one direct launch of the test
      // instance, whose grid comes from its own occupancy
      BatchArgs a = make_args(b, b->steps_per_launch);
      a.hold_block = b->hold_block;
      a.hold_barrier = b->hold_barrier;
      b->hold_block = b->hold_barrier = -1;
      BatchArgs q{};
      int grid = 0;
      BATCH_TRY(wenofd::launch_batch_fp64_withhold(q, b->stream, &grid));
      BATCH_TRY(cudaMemsetAsync(b->d_counters, 0, size_t(b->steps_per_launch) * wenofd::kBatchPhases * sizeof(unsigned),
                                b->stream));
      BATCH_TRY(cudaMemsetAsync(b->d_barrier, 0, sizeof(unsigned), b->stream));
      BATCH_TRY(wenofd::launch_batch_fp64_withhold(a, b->stream, &grid));
      b->launches += 1;
    } else if (int rc = launch_step_block(b)) {
      return rc;
    }
    BATCH_TRY(cudaMemcpyAsync(b->h_flags, b->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BATCH_TRY(cudaStreamSynchronize(b->stream));
    if (b->h_flags[0]) {
      // arrival counts are unknown after a give-up: start the barrier afresh
      BATCH_TRY(cudaMemsetAsync(b->d_barrier, 0, 2 * sizeof(unsigned), b->stream));
      BATCH_TRY(cudaStreamSynchronize(b->stream));
      return fail(WENOFD_TIMEOUT, "batched kernel: a grid barrier wait gave up");
    }
    if (b->h_flags[3]) return fail(WENOFD_TIMEOUT, "batched indicator: a tensor-core completion wait gave up");
    any_error = any_error || b->h_flags[2] != 0;
    if (b->h_flags[1] == 0) break;
  }
  if (int rc = gather(b)) return rc;
  long long most = 0;
  int first_err = -1;
  for (int m = 0; m < b->n; ++m) {
    most = std::max(most, b->h_gather[m].steps - before[m]);
    if (first_err < 0 && b->h_gather[m].error) first_err = m;
  }
  if (steps_done) *steps_done = most;
  if (any_error || first_err >= 0)
    return fail(WENOFD_NAN_DT, "Error: Timestep is not a number... (batch member " +
                                   std::to_string(first_err < 0 ? 0 : first_err) + ")");
  return WENOFD_OK;
}

int wenofd_batch_test_withhold(wenofd_batch *b, int block, int barrier) {
  if (!b) return fail(WENOFD_BAD_ARG, "null batch handle");
  if (b->precision != WENOFD_FP64 || b->scheme != 1 || b->tile_i != 15)
    return fail(WENOFD_BAD_ARG, "the withholding test instance is the FP64 WENO-Z batch kernel with tile 15");
  if (block < 0 || barrier < 0) return fail(WENOFD_BAD_ARG, "block and barrier must be >= 0");
  BATCH_TRY(cudaSetDevice(b->device));
  BatchArgs q{};
  int grid = 0;
  BATCH_TRY(wenofd::launch_batch_fp64_withhold(q, b->stream, &grid));  // its grid (outside any capture)
  if (block >= grid) return fail(WENOFD_BAD_ARG, "block must be below the test instance's grid of " +
                                                     std::to_string(grid) + " blocks");
  b->hold_block = block;
  b->hold_barrier = barrier;
  return WENOFD_OK;
}

int wenofd_batch_autotune(wenofd_batch *b, int steps, double *ms_per_step) {
  WENOFD_TRACE("wenofd_batch_autotune");
  if (!b) return fail(WENOFD_BAD_ARG, "null batch handle");
  if (steps < 1 || steps > 4096) return fail(WENOFD_BAD_ARG, "steps must be in [1, 4096]");
  BATCH_TRY(cudaSetDevice(b->device));
  if (int rc = sync_members(b)) return rc;
  if (indicator_plan_stale(b))
    if (int rc = plan(b, b->tile_i)) return rc;
  const int keep_steps = b->steps_setting;
  // snapshot of every member's U^n (with ghosts) and control block
  size_t total = 0;
  for (const wenofd_solver *s : b->members) total += s->state_bytes + sizeof(Ctrl);
  char *snap = nullptr;
  BATCH_TRY(cudaMalloc(&snap, total));
  auto copy_all = [&](bool save) -> int {
    size_t off = 0;
    for (wenofd_solver *s : b->members) {
      char *st = snap + off, *ct = snap + off + s->state_bytes;
      BATCH_TRY(cudaMemcpyAsync(save ? (void *)st : (void *)s->S, save ? (void *)s->S : (void *)st, s->state_bytes,
                                cudaMemcpyDeviceToDevice, b->stream));
      BATCH_TRY(cudaMemcpyAsync(save ? (void *)ct : (void *)s->ctrl, save ? (void *)s->ctrl : (void *)ct, sizeof(Ctrl),
                                cudaMemcpyDeviceToDevice, b->stream));
      off += s->state_bytes + sizeof(Ctrl);
    }
    return WENOFD_OK;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = WENOFD_OK;
  double best_ms = -1.0;
  int best_tile = b->tile_i, best_bps = 0;
  const int tiles[2] = {15, b->precision == WENOFD_FP64 ? 7 : 31};
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = fail(WENOFD_CUDA_ERROR, "cudaEventCreate failed");
  }
  if (!rc) rc = copy_all(true);
  for (int ti = 0; ti < 2 && !rc; ++ti) {
    // resident blocks per SM the kernel can take at this tile height
    if ((rc = configure(b, tiles[ti], 0, steps))) break;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int occ = sms > 0 ? std::max(1, b->grid / sms) : 1;
    for (int bps = occ; bps >= 1 && !rc; --bps) {
      if ((rc = configure(b, tiles[ti], bps, steps))) break;
      float ms = 0.0f;
      // warm-up of one step, then the timed launch; state restored after each
      for (int pass = 0; pass < 2 && !rc; ++pass) {
        if (cudaMemsetAsync(b->d_flags, 0, 4 * sizeof(int), b->stream) != cudaSuccess ||
            wenofd::launch_batch_setup(b->d_members, b->n, -1, b->stream) != cudaSuccess) {
          rc = fail(WENOFD_CUDA_ERROR, "batch setup launch failed");
          break;
        }
        if (pass == 1 && cudaEventRecord(e0, b->stream) != cudaSuccess) rc = fail(WENOFD_CUDA_ERROR, "event record");
        if (!rc) rc = enqueue_run(b, pass == 0 ? 1 : steps);
        if (!rc && pass == 1 && cudaEventRecord(e1, b->stream) != cudaSuccess)
          rc = fail(WENOFD_CUDA_ERROR, "event record");
        b->launches += 2;
        if (!rc && cudaStreamSynchronize(b->stream) != cudaSuccess)
          rc = fail(WENOFD_CUDA_ERROR, std::string("batched kernel: ") + cudaGetErrorString(cudaGetLastError()));
        if (!rc && cudaMemcpy(b->h_flags, b->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess &&
            (b->h_flags[0] || b->h_flags[3]))
          rc = fail(WENOFD_TIMEOUT, b->h_flags[0] ? "batched kernel: a grid barrier wait gave up"
                                                  : "batched indicator: a tensor-core completion wait gave up");
        if (!rc) rc = copy_all(false);
      }
      if (!rc && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && (best_ms < 0 || ms < best_ms)) {
        best_ms = ms;
        best_tile = tiles[ti];
        best_bps = bps;
      }
    }
  }
  if (!rc) rc = copy_all(false);
  cudaStreamSynchronize(b->stream);
  cudaFree(snap);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc) return rc;
  if ((rc = configure(b, best_tile, best_bps, keep_steps))) return rc;
  b->tuned_ms = best_ms / steps;
  if (ms_per_step) *ms_per_step = b->tuned_ms;
  return WENOFD_OK;
}

}  // extern "C"
