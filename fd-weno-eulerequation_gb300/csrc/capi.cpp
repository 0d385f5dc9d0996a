// Implementation of the C ABI declared in include/wenofd.h.
//
// One handle = one whole-domain solve resident on one GPU: three FP64
// state arrays (U^n and two stage buffers; the reference's m_Uh / m_Un /
// m_rhs, include/WENOFD.hpp:73-75), a SPECIAL boundary table, and a device
// control block that carries dt, the time and the loop flags so the time
// loop never waits on the host.
#include "../../include/wenofd.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "cases.h"
#include "guard.cuh"
#include "solver.h"
#include "trace.h"
#include "wenofd_internal.h"

using wenofd::Ctrl;
using wenofd::Geom;
using wenofd::StageArgs;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string &msg) {
  g_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(WENOFD_CUDA_ERROR, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// trim of utils/readConfig.hpp:12-28: strip ' ' at both ends and one
// trailing '\r'.
std::string trim(const std::string &s) {
  const size_t first = s.find_first_not_of(' ');
  if (first == std::string::npos) return std::string();
  size_t last = s.find_last_not_of(' ');
  if (s[last] == '\r') {
    if (last == first) return std::string();
    --last;
  }
  return s.substr(first, last - first + 1);
}

// CConfig::read, utils/readConfig.hpp:39-80.
int read_config(const char *path, std::map<std::string, std::string> &opt) {
  std::ifstream in(path);
  if (!in.is_open()) return fail(WENOFD_BAD_CONFIG, std::string("Failed to open file ") + path);
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#' || line[0] == '\r') continue;
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;  // the reference prints "Invalid line" and skips it
    opt[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
  }
  return WENOFD_OK;
}

// std::stoi / std::stod semantics: leading number, rest ignored.
bool get_int(const std::map<std::string, std::string> &o, const char *k, int &v, bool required) {
  auto it = o.find(k);
  if (it == o.end()) return !required;
  try {
    v = std::stoi(it->second);
  } catch (...) {
    return false;
  }
  return true;
}

bool get_double(const std::map<std::string, std::string> &o, const char *k, double &v, bool required) {
  auto it = o.find(k);
  if (it == o.end()) return !required;
  try {
    v = std::stod(it->second);
  } catch (...) {
    return false;
  }
  return true;
}

int check_handle(const wenofd_solver *s) {
  if (!s) return fail(WENOFD_BAD_ARG, "null solver handle");
  return WENOFD_OK;
}

// Index of a state array in s->tma: 0 = S, 1 = A, 2 = B.
int stage_buffer(const wenofd_solver *s, const double *in) { return in == s->A ? 1 : (in == s->B ? 2 : 0); }

// After the stream has drained: TIMEOUT if a device wait gave up.
int check_wait(wenofd_solver *s) {
  if (!s->wait_error) return WENOFD_OK;
  int err = 0;
  CUDA_TRY(cudaMemcpy(&err, s->wait_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return fail(WENOFD_TIMEOUT, "a bounded device wait gave up (stage TMA load or tensor-core completion)");
  return WENOFD_OK;
}

int sync(wenofd_solver *s) {
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return WENOFD_OK;
}

// bounds: this stage writes U^{n+1} at the end of a graph-driven step; its
// epilogue also screens the next time step (FP32 forms).
// timeloop: launched by the graph-driven step of wenofd_advance.
int launch_stage(wenofd_solver *s, const double *in, const double *un, double *out, double a, double b,
                 double c, int mode, bool bounds = false, bool timeloop = false) {
  StageArgs args;
  args.uin = in;
  args.un = un;
  args.uout = out;
  args.a = a;
  args.b = b;
  args.c = c;
  args.dt = &s->ctrl->dt;
  args.active = &s->ctrl->active;
  args.mode = mode;
  args.form = wenofd::rk_form(a, b, c, in, un);
  args.flags = s->precision == WENOFD_LEARNED ? s->flags : nullptr;
  if (bounds && s->tile_bounds) {
    args.bounds = s->tile_bounds;
    args.screen = &s->ctrl->screen_bits;
  }
  CUDA_TRY(wenofd::launch_bc_fill(s->g, const_cast<double *>(in), s->special, &s->ctrl->active, s->stream));
  s->launches += 2;
  // The learned form classifies the nodes once per step, on the stage-1
  // input (ghosts just filled); all stages of the step route with those flags.
  if (s->precision == WENOFD_LEARNED && in == s->S && un == s->S && s->ind_ready) {
    CUDA_TRY(wenofd::launch_indicator(s->g, in, s->ind_weights, s->ind_logit_threshold, s->ind_guard, s->flags,
                                      s->wait_error,
                                      &s->ctrl->active, timeloop ? s->ctrl : nullptr, s->ind_interval,
                                      s->stream));
    s->launches += 1;
  }
  args.wait_error = s->wait_error;
  if (s->precision != WENOFD_FP64) {
    CUDA_TRY(wenofd::launch_stage_fp32(s->g, args, s->tma[stage_buffer(s, in)], s->scheme, s->tile_i, s->stream));
  } else {
    CUDA_TRY(wenofd::launch_stage_fp64(s->g, args, s->tma[stage_buffer(s, in)], s->scheme, s->tile_i, s->stream));
  }
  return WENOFD_OK;
}

// RunRK1/2/3 (src/WENOFD.cpp:301-396), dt from the control block.  Stage k
// reads its input with a halo and writes a different buffer; the last stage
// writes U^{n+1} over U^n, which it reads only at the node itself.
// fused: the last stage also screens the next time step (RK2, RK3).
int enqueue_rk(wenofd_solver *s, bool fused = false, bool timeloop = false) {
  int rc;
  double *S = s->S, *A = s->A, *B = s->B;
  switch (s->rk) {
    case 0:  // U += dt * rhs, as (1*U + 0*U) + (1*dt)*rhs (same rounding)
      if ((rc = launch_stage(s, S, S, A, 1.0, 0.0, 1.0, wenofd::kModeRK, false, timeloop))) return rc;
      CUDA_TRY(wenofd::launch_copy_interior(s->g, A, S, &s->ctrl->active, s->stream));
      s->launches += 1;
      return WENOFD_OK;
    case 1:
      if ((rc = launch_stage(s, S, S, A, 1.0, 0.0, 1.0, wenofd::kModeRK, false, timeloop))) return rc;
      return launch_stage(s, A, S, S, 0.5, 0.5, 0.5, wenofd::kModeRK, fused);
    case 2:
      if ((rc = launch_stage(s, S, S, A, 1.0, 0.0, 1.0, wenofd::kModeRK, false, timeloop))) return rc;
      if ((rc = launch_stage(s, A, S, B, 3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0, wenofd::kModeRK))) return rc;
      return launch_stage(s, B, S, S, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, wenofd::kModeRK, fused);
  }
  return fail(WENOFD_BAD_CONFIG, "Error: Invalid Runge-Kutta method");
}

// The time-step reduction: FP64 form one FP64 pass; FP32 forms the two-pass
// reduction (same result bit for bit, FP32 screen + FP64 refine).
int enqueue_dt_reduce(wenofd_solver *s) {
  if (s->precision == WENOFD_FP64) {
    CUDA_TRY(wenofd::launch_dt_reduce(s->g, s->S, s->ctrl, s->stream));
    s->launches += 1;
  } else {
    CUDA_TRY(wenofd::launch_dt_reduce_two_pass(s->g, s->S, s->ctrl, s->tile_bounds, s->tile_i, s->stream));
    s->launches += 2;
  }
  return WENOFD_OK;
}

// One graph-driven step: gate, dt reduction, dt, stages, time update.
int enqueue_step(wenofd_solver *s) {
  CUDA_TRY(wenofd::launch_step_begin(s->ctrl, s->stream));
  if (int rc = enqueue_dt_reduce(s)) return rc;
  CUDA_TRY(wenofd::launch_dt_finalize(s->ctrl, s->stream));
  const bool fused = s->tile_bounds && s->rk != 0;
  int rc = enqueue_rk(s, fused, true);
  if (rc) return rc;
  CUDA_TRY(wenofd::launch_step_end(s->ctrl, fused ? 1 : 0, s->stream));
  s->launches += 3;
  return WENOFD_OK;
}

int read_ctrl(wenofd_solver *s) {
  CUDA_TRY(cudaMemcpyAsync(s->ctrl_host, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

int copy_interior(wenofd_solver *s, double *dst_base, const double *src_base, size_t dst_pitch_b,
                  size_t src_pitch_b, bool to_device, cudaMemcpyKind kind) {
  const size_t plane_host = size_t(s->nx) * s->ny;
  for (int r = 0; r < 4; ++r) {
    const size_t dev_off = size_t(r) * s->g.plane + size_t(wenofd::kGhost) * s->g.pitch + wenofd::kGhost;
    double *dst = to_device ? dst_base + dev_off : dst_base + r * plane_host;
    const double *src = to_device ? src_base + r * plane_host : src_base + dev_off;
    CUDA_TRY(cudaMemcpy2DAsync(dst, dst_pitch_b, src, src_pitch_b, size_t(s->ny) * sizeof(double), s->nx, kind,
                               s->stream));
  }
  return WENOFD_OK;
}

int upload(wenofd_solver *s, const double *src, cudaMemcpyKind kind) {
  return copy_interior(s, s->S, src, s->g.pitch * sizeof(double), s->ny * sizeof(double), true, kind);
}

int download(wenofd_solver *s, const double *dev_full, double *dst, cudaMemcpyKind kind) {
  return copy_interior(s, dst, dev_full, s->ny * sizeof(double), s->g.pitch * sizeof(double), false, kind);
}

void release(wenofd_solver *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph1) cudaGraphExecDestroy(s->graph1);
  cudaFree(s->S);
  cudaFree(s->A);
  cudaFree(s->B);
  cudaFree(s->special);
  cudaFree(s->partials);
  cudaFree(s->red_out);
  cudaFree(s->ctrl);
  cudaFree(s->flags);
  cudaFree(s->ind_weights);
  cudaFree(s->wait_error);
  cudaFree(s->tile_bounds);
  cudaFreeHost(s->ctrl_host);
  cudaFreeHost(s->red_host);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
}

int create_from_map(const std::map<std::string, std::string> &opt, wenofd_solver **out) {
  if (!out) return fail(WENOFD_BAD_ARG, "null output pointer");
  *out = nullptr;
  int testcase, nx, ny, rk, scheme, precision = 0, device = 0, tile_i = 0;
  double cfl, t_end = -1.0;
  long long seed_ll = 0;
  // src/WENOFD.cpp:24-40
  if (!get_int(opt, "TESTCASE", testcase, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing TESTCASE");
  if (!get_int(opt, "RKMETH", rk, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing RKMETH");
  if (!get_int(opt, "SCHEME", scheme, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing SCHEME");
  if (!get_double(opt, "CFL", cfl, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing CFL");
  if (!get_int(opt, "ELEMNUMX", nx, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing ELEMNUMX");
  if (!get_int(opt, "ELEMNUMY", ny, true)) return fail(WENOFD_BAD_CONFIG, "bad or missing ELEMNUMY");
  if (!get_int(opt, "PRECISION", precision, false)) return fail(WENOFD_BAD_CONFIG, "bad PRECISION");
  if (!get_int(opt, "DEVICE", device, false)) return fail(WENOFD_BAD_CONFIG, "bad DEVICE");
  if (!get_int(opt, "TILE_I", tile_i, false)) return fail(WENOFD_BAD_CONFIG, "bad TILE_I");
  if (!get_double(opt, "TEND", t_end, false)) return fail(WENOFD_BAD_CONFIG, "bad TEND");
  double label_deviation = 1e-2;
  if (!get_double(opt, "LABEL_DEVIATION", label_deviation, false) || !(label_deviation > 0.0))
    return fail(WENOFD_BAD_CONFIG, "bad LABEL_DEVIATION");
  int ind_interval = 1;
  if (!get_int(opt, "INDICATOR_INTERVAL", ind_interval, false) || ind_interval < 1 || ind_interval > 1000)
    return fail(WENOFD_BAD_CONFIG, "bad INDICATOR_INTERVAL");
  double ind_guard = 0.0;
  if (!get_double(opt, "INDICATOR_GUARD", ind_guard, false) || !(ind_guard >= 0.0) || ind_guard > 1e6)
    return fail(WENOFD_BAD_CONFIG, "bad INDICATOR_GUARD");
  {
    auto it = opt.find("SEED");
    if (it != opt.end()) {
      try {
        seed_ll = std::stoll(it->second);
      } catch (...) {
        return fail(WENOFD_BAD_CONFIG, "bad SEED");
      }
    }
  }
  if (rk < 0 || rk > 2) return fail(WENOFD_BAD_CONFIG, "Error: Invalid Runge-Kutta method");
  if (scheme < 0 || scheme > 3) return fail(WENOFD_BAD_CONFIG, "the scheme is not supported");
  if (precision < 0 || precision > 2)
    return fail(WENOFD_BAD_CONFIG, "PRECISION must be 0 (FP64), 1 (FP32) or 2 (learned + FP32)");
  if (nx < 6 || ny < 6) return fail(WENOFD_BAD_CONFIG, "ELEMNUMX and ELEMNUMY must be at least 6");
  if (nx > 65536 || ny > 65536) return fail(WENOFD_BAD_CONFIG, "ELEMNUMX and ELEMNUMY must be at most 65536");
  if (!(cfl > 0.0)) return fail(WENOFD_BAD_CONFIG, "CFL must be positive");

  wenofd::CaseSpec cs;
  try {
    cs = wenofd::make_case(testcase, (uint64_t)seed_ll);
  } catch (const std::exception &e) {
    return fail(WENOFD_BAD_CONFIG, e.what());
  }
  if (t_end > 0) cs.t_end = t_end;
  // Overrides of the EulerEquation parameters (utils/equations.hpp:58-70):
  // a caller that sets xL..yR, euler_gamma or the boundary types on its
  // equation object passes them here.
  int bcs[4] = {cs.bc_left, cs.bc_right, cs.bc_bottom, cs.bc_top};
  const char *bc_keys[4] = {"BC_LEFT", "BC_RIGHT", "BC_BOTTOM", "BC_TOP"};
  for (int k = 0; k < 4; ++k) {
    if (!get_int(opt, bc_keys[k], bcs[k], false) || bcs[k] < 0 || bcs[k] > 3)
      return fail(WENOFD_BAD_CONFIG, std::string("bad ") + bc_keys[k]);
  }
  cs.bc_left = bcs[0];
  cs.bc_right = bcs[1];
  cs.bc_bottom = bcs[2];
  cs.bc_top = bcs[3];
  if (!get_double(opt, "XL", cs.xl, false) || !get_double(opt, "XR", cs.xr, false) ||
      !get_double(opt, "YL", cs.yl, false) || !get_double(opt, "YR", cs.yr, false) ||
      !get_double(opt, "GAMMA", cs.gamma, false) || !get_int(opt, "GRAVITY", cs.gravity, false))
    return fail(WENOFD_BAD_CONFIG, "bad domain, GAMMA or GRAVITY value");
  if (!(cs.xr > cs.xl) || !(cs.yr > cs.yl) || !(cs.gamma > 1.0))
    return fail(WENOFD_BAD_CONFIG, "domain must have XR > XL, YR > YL and GAMMA > 1");

  wenofd_solver *s = new wenofd_solver();
  s->device = device;
  s->testcase = testcase;
  s->nx = nx;
  s->ny = ny;
  s->rk = rk;
  s->scheme = scheme;
  s->precision = precision;
  s->tile_i = tile_i;
  s->cfl = cfl;
  s->label_deviation = label_deviation;
  s->ind_interval = ind_interval;
  s->ind_guard = float(ind_guard);
  s->cs = cs;
  const double dx = (cs.xr - cs.xl) / (nx - 1);  // src/WENOFD.cpp:73-74
  const double dy = (cs.yr - cs.yl) / (ny - 1);
  s->g = wenofd::make_geom(nx, ny, dx, dy, cs.gamma, std::pow(dx, 2.0 / 3.0), cs.bc_left, cs.bc_right,
                           cs.bc_bottom, cs.gravity);

  auto bail = [&](int rc) {
    release(s);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess)
    return bail(fail(WENOFD_CUDA_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e)));
  s->g.guard = wenofd::guard_record();  // the handle's device's (bounds-checked build)
  if ((e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(fail(WENOFD_CUDA_ERROR, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)));
  s->stream = s->own_stream;
  s->state_bytes = size_t(4) * s->g.plane * sizeof(double);
  const std::vector<double> tab = wenofd::special_table(cs, nx, ny, dx, dy);
  const int nblk = wenofd::reduce_blocks();
  bool ok = cudaMalloc(&s->S, s->state_bytes) == cudaSuccess && cudaMalloc(&s->A, s->state_bytes) == cudaSuccess &&
            cudaMalloc(&s->B, s->state_bytes) == cudaSuccess &&
            cudaMalloc(&s->special, tab.size() * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&s->partials, size_t(nblk) * 4 * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&s->red_out, 4 * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&s->ctrl, sizeof(Ctrl)) == cudaSuccess &&
            cudaMallocHost(&s->ctrl_host, sizeof(Ctrl)) == cudaSuccess &&
            cudaMallocHost(&s->red_host, 4 * sizeof(double)) == cudaSuccess;
  if (ok && precision != WENOFD_FP64) {  // stage tiles of 15 (or 31) x 32 nodes
    const size_t tiles = size_t((nx + 14) / 15) * size_t((ny + 31) / 32);
    ok = cudaMalloc(&s->tile_bounds, tiles * sizeof(float2)) == cudaSuccess;
  }
  if (ok)  // the stage tiles' TMA waits (and the indicator's) report here
    ok = cudaMalloc(&s->wait_error, sizeof(int)) == cudaSuccess &&
         cudaMemsetAsync(s->wait_error, 0, sizeof(int), s->stream) == cudaSuccess;
  if (ok && precision == WENOFD_LEARNED) {
    const size_t fb = size_t(s->g.nxt) * s->g.pitch;
    ok = cudaMalloc(&s->flags, fb) == cudaSuccess &&
         cudaMalloc(&s->ind_weights, wenofd::indicator_weights_bytes()) == cudaSuccess &&
         cudaMemsetAsync(s->flags, 1, fb, s->stream) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    return bail(fail(WENOFD_CUDA_ERROR, "device allocation failed"));
  }
  {  // TMA maps of the three stage inputs
    double *bufs[3] = {s->S, s->A, s->B};
    for (int k = 0; k < 3; ++k)
      if ((e = wenofd::make_stage_tma(s->g, bufs[k], s->flags, tile_i, &s->tma[k])) != cudaSuccess)
        return bail(fail(WENOFD_CUDA_ERROR, "cuTensorMapEncodeTiled failed for the stage tiles' TMA maps"));
  }
  ok = cudaMemsetAsync(s->S, 0, s->state_bytes, s->stream) == cudaSuccess &&
       cudaMemsetAsync(s->A, 0, s->state_bytes, s->stream) == cudaSuccess &&
       cudaMemsetAsync(s->B, 0, s->state_bytes, s->stream) == cudaSuccess &&
       cudaMemcpyAsync(s->special, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream) ==
           cudaSuccess;
  Ctrl c0{};
  c0.now = 0.0;
  c0.t_end = cs.t_end;
  c0.cfl = cfl;
  c0.max_steps = 0x7fffffffffffffffLL;
  c0.done = !(std::fabs(0.0 - cs.t_end) > 1e-9);
  *s->ctrl_host = c0;
  ok = ok && cudaMemcpyAsync(s->ctrl, s->ctrl_host, sizeof(Ctrl), cudaMemcpyHostToDevice, s->stream) == cudaSuccess &&
       cudaStreamSynchronize(s->stream) == cudaSuccess;
  if (!ok) return bail(fail(WENOFD_CUDA_ERROR, "device initialisation failed"));
  *out = s;
  return WENOFD_OK;
}

}  // namespace

namespace wenofd {
// Lets other translation units of the library report through
// wenofd_last_error().
void set_last_error(const std::string &msg) { g_error = msg; }
}  // namespace wenofd

namespace {

// Guard record -> the public report, with the site's file name looked up
// among the sources that hold guards.
void guard_fill_report(const unsigned long long h[wenofd::kGuardWords], long long report[4], char *where,
                       int where_len) {
  static const char *const kFiles[] = {"aux_device.cuh", "aux_kernels.cu",   "batch_kernel.cuh", "learned.cu",
                                       "learned_data.cu", "noalloc.cu",      "stage_f32.cuh",    "stage_kernel.cuh",
                                       "guard.cuh",       "physics.cuh",     "tma.cuh"};
  report[0] = (long long)h[wenofd::kGuardCount];
  report[1] = h[wenofd::kGuardCount] ? (long long)(h[wenofd::kGuardSite] & 0xffffffffull) : 0;
  report[2] = h[wenofd::kGuardCount] ? (long long)h[wenofd::kGuardIndex] : 0;
  report[3] = h[wenofd::kGuardCount] ? (long long)h[wenofd::kGuardExtent] : 0;
  if (!where || where_len <= 0 || !h[wenofd::kGuardCount]) return;
  const unsigned hash = unsigned(h[wenofd::kGuardSite] >> 32);
  const char *name = "?";
  for (const char *f : kFiles)
    if (wenofd::guard_file_hash(f) == hash) name = f;
  std::snprintf(where, size_t(where_len), "%s:%lld", name, report[1]);
}

}  // namespace

extern "C" {

const char *wenofd_last_error(void) { return g_error.c_str(); }

const char *wenofd_version(void) { return "wenofd-gb300 0.1 (sm_103a)"; }

int wenofd_create(const char *const *keys, const char *const *values, int n, wenofd_solver **out) {
  WENOFD_TRACE("wenofd_create");
  if (n < 0 || (n > 0 && (!keys || !values))) return fail(WENOFD_BAD_ARG, "bad key/value arrays");
  std::map<std::string, std::string> opt;
  for (int i = 0; i < n; ++i) {
    if (!keys[i] || !values[i]) return fail(WENOFD_BAD_ARG, "null key or value");
    opt[trim(keys[i])] = trim(values[i]);
  }
  return create_from_map(opt, out);
}

int wenofd_create_from_file(const char *config_path, wenofd_solver **out) {
  if (!config_path) return fail(WENOFD_BAD_ARG, "null config path");
  std::map<std::string, std::string> opt;
  int rc = read_config(config_path, opt);
  if (rc) return rc;
  return create_from_map(opt, out);
}

int wenofd_destroy(wenofd_solver *s) {
  if (!s) return WENOFD_OK;
  release(s);
  return WENOFD_OK;
}

int wenofd_set_stream(wenofd_solver *s, void *cuda_stream) {
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : s->own_stream;
  return WENOFD_OK;
}

int wenofd_get_info(const wenofd_solver *s, wenofd_info *info) {
  if (int rc = check_handle(s)) return rc;
  if (!info) return fail(WENOFD_BAD_ARG, "null info");
  wenofd_solver *m = const_cast<wenofd_solver *>(s);
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = read_ctrl(m)) return rc;
  info->nx = s->nx;
  info->ny = s->ny;
  info->testcase = s->testcase;
  info->scheme = s->scheme;
  info->rk = s->rk;
  info->precision = s->precision;
  info->bc_left = s->cs.bc_left;
  info->bc_right = s->cs.bc_right;
  info->bc_bottom = s->cs.bc_bottom;
  info->bc_top = s->cs.bc_top;
  info->has_exact = s->cs.exact;
  info->pitch = s->g.pitch;
  info->dx = s->g.dx;
  info->dy = s->g.dy;
  info->cfl = s->cfl;
  info->t_end = s->cs.t_end;
  info->now = s->ctrl_host->now;
  info->gamma = s->cs.gamma;
  info->xl = s->cs.xl;
  info->xr = s->cs.xr;
  info->yl = s->cs.yl;
  info->yr = s->cs.yr;
  info->steps = s->ctrl_host->steps;
  info->launches = s->launches;
  info->graph_steps = s->graph_steps;
  info->dt = s->ctrl_host->dt;
  return WENOFD_OK;
}

int wenofd_initialize(wenofd_solver *s) {
  WENOFD_TRACE("wenofd_initialize");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  std::vector<double> host(size_t(4) * s->nx * s->ny);
  wenofd::initial_state(s->cs, s->nx, s->ny, s->g.dx, s->g.dy, host.data());
  if (int rc = upload(s, host.data(), cudaMemcpyHostToDevice)) return rc;
  CUDA_TRY(wenofd::launch_set_time(s->ctrl, 0.0, s->stream));
  if (int rc = sync(s)) return rc;
  if (int rc = read_ctrl(s)) return rc;
  s->ctrl_host->steps = 0;
  CUDA_TRY(cudaMemcpyAsync(s->ctrl, s->ctrl_host, sizeof(Ctrl), cudaMemcpyHostToDevice, s->stream));
  return sync(s);
}

int wenofd_set_state(wenofd_solver *s, const double *host_state) {
  WENOFD_TRACE("wenofd_set_state");
  if (int rc = check_handle(s)) return rc;
  if (!host_state) return fail(WENOFD_BAD_ARG, "null state");
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = upload(s, host_state, cudaMemcpyHostToDevice)) return rc;
  return sync(s);
}

int wenofd_get_state(wenofd_solver *s, double *host_state) {
  WENOFD_TRACE("wenofd_get_state");
  if (int rc = check_handle(s)) return rc;
  if (!host_state) return fail(WENOFD_BAD_ARG, "null state");
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = download(s, s->S, host_state, cudaMemcpyDeviceToHost)) return rc;
  return sync(s);
}

int wenofd_set_state_device(wenofd_solver *s, const double *dev_state) {
  if (int rc = check_handle(s)) return rc;
  if (!dev_state) return fail(WENOFD_BAD_ARG, "null state");
  CUDA_TRY(cudaSetDevice(s->device));
  return upload(s, dev_state, cudaMemcpyDeviceToDevice);
}

int wenofd_get_state_device(wenofd_solver *s, double *dev_state) {
  if (int rc = check_handle(s)) return rc;
  if (!dev_state) return fail(WENOFD_BAD_ARG, "null state");
  CUDA_TRY(cudaSetDevice(s->device));
  return download(s, s->S, dev_state, cudaMemcpyDeviceToDevice);
}

int wenofd_get_state_ghosted(wenofd_solver *s, double *host_full) {
  if (int rc = check_handle(s)) return rc;
  if (!host_full) return fail(WENOFD_BAD_ARG, "null state");
  CUDA_TRY(cudaSetDevice(s->device));
  const size_t hp = size_t(s->g.nxt) * s->g.nyt;
  for (int r = 0; r < 4; ++r)
    CUDA_TRY(cudaMemcpy2DAsync(host_full + r * hp, s->g.nyt * sizeof(double), s->S + r * s->g.plane,
                               s->g.pitch * sizeof(double), s->g.nyt * sizeof(double), s->g.nxt,
                               cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

int wenofd_set_time(wenofd_solver *s, double now) {
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_set_time(s->ctrl, now, s->stream));
  return sync(s);
}

int wenofd_set_boundary_values(wenofd_solver *s, const double *host_table) {
  if (int rc = check_handle(s)) return rc;
  if (!host_table) return fail(WENOFD_BAD_ARG, "null table");
  CUDA_TRY(cudaSetDevice(s->device));
  const size_t n = 8 * size_t(s->g.nxt) + 8 * size_t(s->g.nyt);
  CUDA_TRY(cudaMemcpyAsync(s->special, host_table, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  return sync(s);
}

int wenofd_fill_boundary(wenofd_solver *s) {
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_bc_fill(s->g, s->S, s->special, nullptr, s->stream));
  return sync(s);
}

int wenofd_get_flux(wenofd_solver *s, double *host_rhs) {
  WENOFD_TRACE("wenofd_get_flux");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_ctrl_open(s->ctrl, s->stream));
  if (int rc = launch_stage(s, s->S, s->S, s->A, 0.0, 0.0, 0.0, wenofd::kModeRHS)) return rc;
  if (host_rhs)
    if (int rc = download(s, s->A, host_rhs, cudaMemcpyDeviceToHost)) return rc;
  if (int rc = sync(s)) return rc;
  return check_wait(s);
}

int wenofd_calc_dt(wenofd_solver *s, double *dt) {
  WENOFD_TRACE("wenofd_calc_dt");
  if (int rc = check_handle(s)) return rc;
  if (!dt) return fail(WENOFD_BAD_ARG, "null dt");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_ctrl_open(s->ctrl, s->stream));
  if (int rc = enqueue_dt_reduce(s)) return rc;
  CUDA_TRY(wenofd::launch_dt_finalize(s->ctrl, s->stream));
  s->launches += 2;
  if (int rc = read_ctrl(s)) return rc;
  if (s->ctrl_host->error) return fail(WENOFD_NAN_DT, "Error: Timestep is not a number...");
  *dt = s->ctrl_host->dt;
  return WENOFD_OK;
}

int wenofd_rk_step(wenofd_solver *s, double dt) {
  WENOFD_TRACE("wenofd_rk_step");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_set_dt(s->ctrl, dt, s->stream));
  if (int rc = enqueue_rk(s)) return rc;
  if (int rc = sync(s)) return rc;
  return check_wait(s);
}

int wenofd_step(wenofd_solver *s, double *dt_out) {
  WENOFD_TRACE("wenofd_step");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_ctrl_open(s->ctrl, s->stream));
  if (int rc = enqueue_dt_reduce(s)) return rc;
  CUDA_TRY(wenofd::launch_dt_finalize(s->ctrl, s->stream));
  if (int rc = enqueue_rk(s)) return rc;
  CUDA_TRY(wenofd::launch_step_end(s->ctrl, 0, s->stream));
  s->launches += 3;
  if (int rc = read_ctrl(s)) return rc;
  if (int rc = check_wait(s)) return rc;
  if (s->ctrl_host->error) return fail(WENOFD_NAN_DT, "Error: Timestep is not a number...");
  if (dt_out) *dt_out = s->ctrl_host->dt;
  return WENOFD_OK;
}

namespace {

// Captures `nsteps` graph-driven steps into an executable graph on a private
// stream; *kernels receives the kernel nodes it holds.
int capture_steps(wenofd_solver *s, int nsteps, cudaGraphExec_t *exec, long long *kernels) {
  cudaStream_t cap = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaStream_t keep = s->stream;
  s->stream = cap;
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int rc = WENOFD_OK;
  const long long before = s->launches;
  if (ce == cudaSuccess) {
    for (int k = 0; k < nsteps && rc == WENOFD_OK; ++k) rc = enqueue_step(s);
    ce = cudaStreamEndCapture(cap, &graph);
  }
  *kernels = s->launches - before;
  s->launches = before;
  s->stream = keep;
  cudaStreamDestroy(cap);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  CUDA_TRY(ce);
  ce = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  CUDA_TRY(ce);
  return WENOFD_OK;
}

void drop_graphs(wenofd_solver *s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph1) cudaGraphExecDestroy(s->graph1);
  s->graph = nullptr;
  s->graph1 = nullptr;
}

}  // namespace

int wenofd_advance(wenofd_solver *s, long long max_steps, long long *steps_done) {
  WENOFD_TRACE("wenofd_advance");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = read_ctrl(s)) return rc;
  const long long start = s->ctrl_host->steps;
  if (!s->graph) {
    // One gated-off pass outside capture configures the kernels' shared
    // memory limits on this device: the gate is closed (max_steps = steps),
    // so every kernel returns at once.
    CUDA_TRY(wenofd::launch_advance_setup(s->ctrl, 0, s->stream));
    if (int rc = enqueue_step(s)) return rc;
    if (int rc = sync(s)) return rc;
    // Steps per graph launch: enough that launch latency is amortised on
    // small grids, one step on large ones.
    const long long cells = (long long)s->nx * s->ny;
    s->graph_steps = int(std::max(1LL, std::min(64LL, (4LL << 20) / std::max(1LL, cells))));
    if (int rc = capture_steps(s, s->graph_steps, &s->graph, &s->graph_kernels)) return rc;
  }
  CUDA_TRY(wenofd::launch_advance_setup(s->ctrl, max_steps, s->stream));
  s->launches += 1;
  // Steps this call may still take (-1: no cap).  A chunk past the cap runs
  // gated-off launches that return at once; when fewer steps than a chunk
  // remain, one-step graphs are replayed instead.
  long long left = max_steps < 0 ? -1 : max_steps;
  for (;;) {
    if (left >= 0 && left < s->graph_steps) {
      if (!s->graph1) {
        if (int rc = capture_steps(s, 1, &s->graph1, &s->graph1_kernels)) return rc;
      }
      for (long long k = 0; k < left; ++k) {
        CUDA_TRY(cudaGraphLaunch(s->graph1, s->stream));
        s->launches += s->graph1_kernels;
      }
    } else {
      CUDA_TRY(cudaGraphLaunch(s->graph, s->stream));
      s->launches += s->graph_kernels;
    }
    if (int rc = read_ctrl(s)) return rc;
    const Ctrl &c = *s->ctrl_host;
    if (int rc = check_wait(s)) return rc;
    if (c.error) {
      if (steps_done) *steps_done = c.steps - start;
      return fail(WENOFD_NAN_DT, "Error: Timestep is not a number...");
    }
    if (c.done || c.steps >= c.max_steps) break;
    if (left >= 0) left = c.max_steps - c.steps;
  }
  if (steps_done) *steps_done = s->ctrl_host->steps - start;
  return WENOFD_OK;
}

int wenofd_error_norms(wenofd_solver *s, double out[3]) {
  WENOFD_TRACE("wenofd_error_norms");
  if (int rc = check_handle(s)) return rc;
  if (!out) return fail(WENOFD_BAD_ARG, "null output");
  if (!s->cs.exact) return fail(WENOFD_NO_EXACT, "this case has no exact solution");
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = read_ctrl(s)) return rc;
  CUDA_TRY(wenofd::launch_reduce(s->g, s->S, 0, s->ctrl_host->now, s->cs.xl, s->cs.yl, s->partials, s->red_out,
                                 s->stream));
  CUDA_TRY(cudaMemcpyAsync(s->red_host, s->red_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (int rc = sync(s)) return rc;
  std::memcpy(out, s->red_host, 3 * sizeof(double));
  return WENOFD_OK;
}

int wenofd_time_stages(wenofd_solver *s, int reps, double *ms_per_launch) {
  WENOFD_TRACE("wenofd_time_stages");
  if (int rc = check_handle(s)) return rc;
  if (!ms_per_launch || reps < 1) return fail(WENOFD_BAD_ARG, "bad arguments");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_ctrl_open(s->ctrl, s->stream));
  s->launches += 1;
  struct St { const double *in, *un; double *out; double a, b, c; };
  std::vector<St> st;
  st.push_back({s->S, s->S, s->A, 1.0, 0.0, 1.0});
  if (s->rk == 2) {
    st.push_back({s->A, s->S, s->B, 3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0});
    st.push_back({s->B, s->S, s->S, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0});
  } else if (s->rk == 1) {
    st.push_back({s->A, s->S, s->S, 0.5, 0.5, 0.5});
  }
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaEventRecord(e0, s->stream));
  for (int r = 0; r < reps; ++r)
    for (const St &x : st) {
      StageArgs a{x.in, x.un, x.out, x.a, x.b, x.c, &s->ctrl->dt, &s->ctrl->active, wenofd::kModeRK,
                  s->precision == WENOFD_LEARNED ? s->flags : nullptr};
      a.form = wenofd::rk_form(x.a, x.b, x.c, x.in, x.un);
      a.wait_error = s->wait_error;
      cudaError_t e = s->precision != WENOFD_FP64
                          ? wenofd::launch_stage_fp32(s->g, a, s->tma[stage_buffer(s, x.in)], s->scheme, s->tile_i,
                                                      s->stream)
                          : wenofd::launch_stage_fp64(s->g, a, s->tma[stage_buffer(s, x.in)], s->scheme, s->tile_i,
                                                      s->stream);
      CUDA_TRY(e);
      s->launches += 1;
    }
  CUDA_TRY(cudaEventRecord(e1, s->stream));
  CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = double(ms) / (double(reps) * st.size());
  return check_wait(s);
}

int wenofd_set_indicator(wenofd_solver *s, const float *host_params, float threshold) {
  if (int rc = check_handle(s)) return rc;
  if (s->precision != WENOFD_LEARNED) return fail(WENOFD_BAD_CONFIG, "the indicator needs PRECISION = 2");
  if (!host_params || !(threshold > 0.0f) || !(threshold < 1.0f)) return fail(WENOFD_BAD_ARG, "bad indicator arguments");
  CUDA_TRY(cudaSetDevice(s->device));
  std::vector<unsigned char> packed(wenofd::indicator_weights_bytes());
  wenofd::pack_indicator_weights(host_params, packed.data());
  CUDA_TRY(cudaMemcpyAsync(s->ind_weights, packed.data(), packed.size(), cudaMemcpyHostToDevice, s->stream));
  s->ind_logit_threshold = std::log(threshold / (1.0f - threshold));
  if (int rc = sync(s)) return rc;
  s->ind_ready = true;
  // the time-loop graphs hold the indicator launch and its threshold: capture
  // them again on the next advance
  drop_graphs(s);
  return WENOFD_OK;
}

int wenofd_routing_flags(wenofd_solver *s, unsigned char *host_flags) {
  if (int rc = check_handle(s)) return rc;
  if (!host_flags) return fail(WENOFD_BAD_ARG, "null flags");
  if (s->precision != WENOFD_LEARNED) return fail(WENOFD_BAD_CONFIG, "routing flags need PRECISION = 2");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(cudaMemcpy2DAsync(host_flags, s->ny, s->flags + size_t(wenofd::kGhost) * s->g.pitch + wenofd::kGhost,
                             s->g.pitch, s->ny, s->nx, cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

int wenofd_indicator_flags(wenofd_solver *s, unsigned char *host_flags) {
  WENOFD_TRACE("wenofd_indicator_flags");
  if (int rc = check_handle(s)) return rc;
  if (!host_flags) return fail(WENOFD_BAD_ARG, "null flags");
  if (s->precision != WENOFD_LEARNED || !s->ind_ready)
    return fail(WENOFD_BAD_CONFIG, "no indicator loaded (PRECISION = 2 and wenofd_set_indicator)");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_ctrl_open(s->ctrl, s->stream));
  CUDA_TRY(wenofd::launch_bc_fill(s->g, s->S, s->special, nullptr, s->stream));
  CUDA_TRY(wenofd::launch_indicator(s->g, s->S, s->ind_weights, s->ind_logit_threshold, s->ind_guard, s->flags,
                                    s->wait_error,
                                    nullptr, nullptr, 1, s->stream));
  s->launches += 3;
  CUDA_TRY(cudaMemcpy2DAsync(host_flags, s->ny, s->flags + size_t(wenofd::kGhost) * s->g.pitch + wenofd::kGhost,
                             s->g.pitch, s->ny, s->nx, cudaMemcpyDeviceToHost, s->stream));
  int err = 0;
  CUDA_TRY(cudaMemcpyAsync(&err, s->wait_error, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  if (int rc = sync(s)) return rc;
  if (err) return fail(WENOFD_TIMEOUT, "indicator kernel: a tensor-core completion wait gave up");
  return WENOFD_OK;
}

int wenofd_indicator_data(wenofd_solver *s, float *dev_features, unsigned char *dev_labels) {
  WENOFD_TRACE("wenofd_indicator_data");
  if (int rc = check_handle(s)) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_bc_fill(s->g, s->S, s->special, nullptr, s->stream));
  if (dev_features) CUDA_TRY(wenofd::launch_features(s->g, s->S, dev_features, s->stream));
  if (dev_labels) CUDA_TRY(wenofd::launch_labels(s->g, s->S, dev_labels, s->label_deviation, s->stream));
  return sync(s);
}

int wenofd_output_variables(wenofd_solver *s, double *host_out) {
  WENOFD_TRACE("wenofd_output_variables");
  if (int rc = check_handle(s)) return rc;
  if (!host_out) return fail(WENOFD_BAD_ARG, "null output");
  CUDA_TRY(cudaSetDevice(s->device));
  // The stage buffers are free between steps: planes 0-3 of the result go
  // to A, planes 4-5 to B (each holds >= 4 * nx * ny doubles).
  const size_t n = size_t(s->nx) * s->ny;
  CUDA_TRY(wenofd::launch_output_vars(s->g, s->S, s->A, s->B, s->stream));
  s->launches += 1;
  CUDA_TRY(cudaMemcpyAsync(host_out, s->A, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(host_out + 4 * n, s->B, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

namespace {

// Restart file: this header, then the interior state [4][NX][NY] float64
// (the host layout of wenofd_set_state), all little-endian.
struct StateFileHeader {
  char magic[8];  // "WENOFDS1"
  int32_t version;
  int32_t nx, ny, testcase, scheme, rk, precision;
  int32_t reserved;
  int64_t steps;
  double now, t_end, dx, dy, gamma, cfl;
};
constexpr char kStateMagic[8] = {'W', 'E', 'N', 'O', 'F', 'D', 'S', '1'};

// Sets the loop clock (time and step count) of the control block.
int set_clock(wenofd_solver *s, double now, long long steps) {
  CUDA_TRY(wenofd::launch_set_time(s->ctrl, now, s->stream));
  if (int rc = read_ctrl(s)) return rc;
  s->ctrl_host->steps = steps;
  CUDA_TRY(cudaMemcpyAsync(s->ctrl, s->ctrl_host, sizeof(Ctrl), cudaMemcpyHostToDevice, s->stream));
  return sync(s);
}

}  // namespace

int wenofd_save_state(wenofd_solver *s, const char *path) {
  WENOFD_TRACE("wenofd_save_state");
  if (int rc = check_handle(s)) return rc;
  if (!path) return fail(WENOFD_BAD_ARG, "null path");
  CUDA_TRY(cudaSetDevice(s->device));
  if (int rc = read_ctrl(s)) return rc;
  StateFileHeader h{};
  std::memcpy(h.magic, kStateMagic, 8);
  h.version = 1;
  h.nx = s->nx;
  h.ny = s->ny;
  h.testcase = s->testcase;
  h.scheme = s->scheme;
  h.rk = s->rk;
  h.precision = s->precision;
  h.steps = s->ctrl_host->steps;
  h.now = s->ctrl_host->now;
  h.t_end = s->ctrl_host->t_end;
  h.dx = s->g.dx;
  h.dy = s->g.dy;
  h.gamma = s->g.gamma;
  h.cfl = s->cfl;
  std::vector<double> host(size_t(4) * s->nx * s->ny);
  if (int rc = download(s, s->S, host.data(), cudaMemcpyDeviceToHost)) return rc;
  if (int rc = sync(s)) return rc;
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(WENOFD_BAD_ARG, std::string("cannot write ") + path);
  const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                  std::fwrite(host.data(), sizeof(double), host.size(), f) == host.size();
  if (std::fclose(f) != 0 || !ok) return fail(WENOFD_BAD_ARG, std::string("write failed: ") + path);
  return WENOFD_OK;
}

int wenofd_load_state(wenofd_solver *s, const char *path) {
  WENOFD_TRACE("wenofd_load_state");
  if (int rc = check_handle(s)) return rc;
  if (!path) return fail(WENOFD_BAD_ARG, "null path");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(WENOFD_BAD_ARG, std::string("cannot read ") + path);
  StateFileHeader h{};
  std::vector<double> host;
  int rc = WENOFD_OK;
  if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1) {
    rc = fail(WENOFD_BAD_ARG, std::string("not a wenofd state file (version 1): ") + path);
  } else if (h.nx != s->nx || h.ny != s->ny || h.testcase != s->testcase || h.dx != s->g.dx || h.dy != s->g.dy) {
    rc = fail(WENOFD_BAD_CONFIG, "state file " + std::string(path) + " is for another grid or test case (" +
                                     std::to_string(h.nx) + "x" + std::to_string(h.ny) + ", TESTCASE " +
                                     std::to_string(h.testcase) + ")");
  } else {
    host.resize(size_t(4) * s->nx * s->ny);
    if (std::fread(host.data(), sizeof(double), host.size(), f) != host.size())
      rc = fail(WENOFD_BAD_ARG, std::string("state file is truncated: ") + path);
  }
  std::fclose(f);
  if (rc) return rc;
  CUDA_TRY(cudaSetDevice(s->device));
  if ((rc = upload(s, host.data(), cudaMemcpyHostToDevice))) return rc;
  return set_clock(s, h.now, h.steps);
}

int wenofd_indicator_sample(wenofd_solver *s, long long per_snapshot, unsigned long long seed, float *dev_x,
                            float *dev_y, long long capacity, long long *rows_out) {
  WENOFD_TRACE("wenofd_indicator_sample");
  if (int rc = check_handle(s)) return rc;
  if (!dev_x || !dev_y || !rows_out) return fail(WENOFD_BAD_ARG, "null output");
  if (per_snapshot < 2 || capacity < 0) return fail(WENOFD_BAD_ARG, "per_snapshot must be >= 2, capacity >= 0");
  CUDA_TRY(cudaSetDevice(s->device));
  const long long n = (long long)s->nx * s->ny;
  const int G = wenofd::sample_blocks();
  // scratch in the stage buffer A (free between steps): labels, per-block
  // counts and row offsets, the kept nodes' indices
  const long long rows_cap = std::min(capacity, n);
  auto align8 = [](size_t b) { return (b + 7) & ~size_t(7); };
  const size_t off_counts = align8(size_t(n));
  const size_t off_offsets = align8(off_counts + size_t(G) * sizeof(unsigned));
  const size_t off_cells = off_offsets + size_t(G) * sizeof(long long);
  if (off_cells + size_t(rows_cap) * sizeof(long long) > s->state_bytes)
    return fail(WENOFD_BAD_ARG, "grid too small for the sampler's scratch");
  unsigned char *scratch = reinterpret_cast<unsigned char *>(s->A);
  unsigned char *labels = scratch;
  unsigned *counts = reinterpret_cast<unsigned *>(scratch + off_counts);
  long long *offsets = reinterpret_cast<long long *>(scratch + off_offsets);
  long long *cells = reinterpret_cast<long long *>(scratch + off_cells);
  unsigned long long *npos_dev = reinterpret_cast<unsigned long long *>(s->red_out);
  CUDA_TRY(wenofd::launch_bc_fill(s->g, s->S, s->special, nullptr, s->stream));
  CUDA_TRY(wenofd::launch_labels(s->g, s->S, labels, s->label_deviation, s->stream));
  CUDA_TRY(wenofd::launch_count_positive(labels, n, npos_dev, s->stream));
  unsigned long long npos = 0;
  CUDA_TRY(cudaMemcpyAsync(s->red_host, npos_dev, sizeof(npos), cudaMemcpyDeviceToHost, s->stream));
  if (int rc = sync(s)) return rc;
  std::memcpy(&npos, s->red_host, sizeof(npos));
  const unsigned long long nneg = (unsigned long long)n - npos;
  // half positives, half negatives where possible (the other class fills in)
  const unsigned long long k_pos = std::min<unsigned long long>(npos, (unsigned long long)per_snapshot / 2);
  const unsigned long long k_neg = std::min<unsigned long long>(nneg, (unsigned long long)per_snapshot - k_pos);
  auto thr = [](unsigned long long k, unsigned long long count) -> unsigned long long {
    if (count == 0 || k == 0) return 0ull;
    if (k >= count) return 1ull << 32;
    return (k << 32) / count;
  };
  const unsigned long long thr0 = thr(k_neg, nneg), thr1 = thr(k_pos, npos);
  CUDA_TRY(wenofd::launch_sample_count(labels, n, seed, thr0, thr1, counts, s->stream));
  std::vector<unsigned> hc(G);
  CUDA_TRY(cudaMemcpyAsync(hc.data(), counts, size_t(G) * sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
  if (int rc = sync(s)) return rc;
  std::vector<long long> ho(G);
  long long total = 0;
  for (int b = 0; b < G; ++b) {
    ho[b] = total;
    total += hc[b];
  }
  CUDA_TRY(cudaMemcpyAsync(offsets, ho.data(), size_t(G) * sizeof(long long), cudaMemcpyHostToDevice, s->stream));
  const long long rows = std::min(total, rows_cap);
  CUDA_TRY(wenofd::launch_sample_write(s->g, s->S, labels, seed, thr0, thr1, offsets, rows_cap, rows, cells, dev_x,
                                       dev_y, s->stream));
  s->launches += 6;
  if (int rc = sync(s)) return rc;
  *rows_out = rows;
  return WENOFD_OK;
}

int wenofd_conservation_sums(wenofd_solver *s, double out[4]) {
  WENOFD_TRACE("wenofd_conservation_sums");
  if (int rc = check_handle(s)) return rc;
  if (!out) return fail(WENOFD_BAD_ARG, "null output");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(wenofd::launch_reduce(s->g, s->S, 1, 0.0, 0.0, 0.0, s->partials, s->red_out, s->stream));
  CUDA_TRY(cudaMemcpyAsync(s->red_host, s->red_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (int rc = sync(s)) return rc;
  std::memcpy(out, s->red_host, 4 * sizeof(double));
  return WENOFD_OK;
}

int wenofd_bounds_report(long long report[4], char *where, int where_len, int reset) {
  if (!report) return fail(WENOFD_BAD_ARG, "null report");
  if (where && where_len > 0) where[0] = '\0';
  unsigned long long *rec = wenofd::guard_record();
  if (!rec) {
    report[0] = -1;
    report[1] = report[2] = report[3] = 0;
    return WENOFD_OK;
  }
  unsigned long long h[wenofd::kGuardWords] = {};
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(h, rec, sizeof(h), cudaMemcpyDeviceToHost));
  if (reset) CUDA_TRY(cudaMemset(rec, 0, sizeof(h)));
  guard_fill_report(h, report, where, where_len);
  return WENOFD_OK;
}

int wenofd_bounds_selftest(long long report[4], char *where, int where_len) {
  if (!report) return fail(WENOFD_BAD_ARG, "null report");
  if (where && where_len > 0) where[0] = '\0';
  // a private record and the 4-element array, one allocation
  unsigned long long *buf = nullptr;
  CUDA_TRY(cudaMalloc(&buf, sizeof(unsigned long long) * wenofd::kGuardWords + 4 * sizeof(int)));
  unsigned long long h[wenofd::kGuardWords] = {}, site = 0;
  cudaError_t e = cudaMemset(buf, 0, sizeof(unsigned long long) * wenofd::kGuardWords + 4 * sizeof(int));
  if (e == cudaSuccess)
    e = wenofd::launch_guard_selftest(buf, reinterpret_cast<int *>(buf + wenofd::kGuardWords), &site, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(h, buf, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return fail(WENOFD_CUDA_ERROR, std::string("bounds self-test: ") + cudaGetErrorString(e));
  guard_fill_report(h, report, where, where_len);
  return WENOFD_OK;
}

}  // extern "C"
