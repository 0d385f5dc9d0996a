// The solver handle behind the C ABI's wenofd_solver, shared by the
// translation units that implement the ABI (capi.cpp, batch.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/wenofd.h"
#include "cases.h"
#include "wenofd_internal.h"

struct wenofd_solver {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // created by the handle
  int testcase = 0, nx = 0, ny = 0, rk = 2, scheme = 1, precision = 0, tile_i = 0;
  double cfl = 0.5;
  wenofd::CaseSpec cs;
  wenofd::Geom g{};
  double *S = nullptr, *A = nullptr, *B = nullptr;  // U^n, stage buffers
  size_t state_bytes = 0;
  double *special = nullptr;
  double *partials = nullptr, *red_out = nullptr;
  wenofd::Ctrl *ctrl = nullptr;
  wenofd::Ctrl *ctrl_host = nullptr;    // pinned mirror
  double *red_host = nullptr;   // pinned, 4 doubles
  float2 *tile_bounds = nullptr;  // FP32 forms: per-stage-tile time-step screen bounds
  // learned form (PRECISION 2)
  unsigned char *flags = nullptr;  // [nxt][pitch], ghosts 1
  void *ind_weights = nullptr;     // packed BF16 indicator weights
  int *wait_error = nullptr;       // FP32 forms: set when a device wait (TMA load, tensor-core completion) gave up
  wenofd::StageTma tma[3];         // FP32 forms: TMA maps of the stage inputs S, A, B (and the flags)
  float ind_logit_threshold = 0.0f;
  double label_deviation = 1e-2;  // LABEL_DEVIATION: training-label threshold
  int ind_interval = 1;            // INDICATOR_INTERVAL: steps per indicator run in the time loop
  float ind_guard = 0.0f;          // INDICATOR_GUARD: relative window range that flags a node (0: off)
  bool ind_ready = false;
  cudaGraphExec_t graph = nullptr;   // graph_steps steps of the time loop
  cudaGraphExec_t graph1 = nullptr;  // one step, for the tail of a capped advance
  int graph_steps = 0;
  long long graph_kernels = 0;   // kernel nodes in the graph
  long long graph1_kernels = 0;  // kernel nodes in graph1
  long long launches = 0;       // kernels enqueued so far (graph replays included)
};

namespace wenofd {
// Reports through wenofd_last_error() (defined in capi.cpp).
void set_last_error(const std::string &msg);
}  // namespace wenofd
