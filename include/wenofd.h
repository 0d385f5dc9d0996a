/*
 * wenofd.h — C ABI of the GB300-native WENO finite-difference Euler solver.
 *
 * The entry points replace the per-step hot path of the reference solver
 * class CWENOFD (infinity-07/FD-WENO-EulerEquation, include/WENOFD.hpp:28-124,
 * src/WENOFD.cpp).  Each declaration names the reference member it stands
 * in for.  One solver handle owns one whole-domain, device-resident state on
 * one GPU; the reference's 1-D MPI slab decomposition and halo exchange
 * (src/WENOFD.cpp:47-70, 850-929) become an in-place device ghost fill.
 *
 * Conventions
 *  - Every function returns an int status (enum wenofd_status).  On failure
 *    wenofd_last_error() returns a message for the calling thread.  Where the
 *    reference aborts (MPI_Abort, exit) or throws, these return a status.
 *  - Host-side state arrays are float64, interior nodes only, structure of
 *    arrays [4][ELEMNUMX][ELEMNUMY] with ej (y) fastest: element (r, ei, ej)
 *    is m_Uh[ei+4][ej+4].vector[r] of the reference.  r = rho, rho*u, rho*v, E.
 *  - A handle is used by one host thread at a time.  Its work runs on one
 *    CUDA stream (its own, or the caller's via wenofd_set_stream).
 *  - No torch or other framework types cross this boundary.
 */
#ifndef WENOFD_H
#define WENOFD_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wenofd_solver wenofd_solver;

enum wenofd_status {
  WENOFD_OK = 0,
  WENOFD_BAD_CONFIG = 1, /* bad or missing config key (reference: std::stoi throws, invalid_argument) */
  WENOFD_CUDA_ERROR = 2, /* a CUDA call failed */
  WENOFD_NAN_DT = 3,     /* time step is NaN (reference: src/WENOFD.cpp:437-442 aborts) */
  WENOFD_TIMEOUT = 4,    /* a bounded device-side wait gave up */
  WENOFD_BAD_ARG = 5,    /* null pointer, size or mode out of range */
  WENOFD_NO_EXACT = 6    /* error norms asked for a case without an exact solution */
};

/* Arithmetic of the flux / reconstruction kernels.  FP64 reproduces the
 * reference bit for bit.  FP32 keeps state, RK sums, the time-step reduction
 * and all norms in FP64 and evaluates fluxes and reconstruction in FP32.
 * LEARNED is FP32 plus the learned troubled-cell indicator: each step a
 * tensor-core MLP flags nodes, and only faces near flagged nodes take
 * characteristic WENO; the others take the linear fifth-order upwind flux. */
enum wenofd_precision { WENOFD_FP64 = 0, WENOFD_FP32 = 1, WENOFD_LEARNED = 2 };

/* Test cases: TESTCASETYPE (utils/equations.hpp:30-36) plus two seeded ones. */
enum wenofd_testcase {
  WENOFD_SMOOTH = 0, WENOFD_RIEMANN1 = 1, WENOFD_RIEMANN2 = 2, WENOFD_RTI = 3,
  WENOFD_RIEMANN_SEEDED = 4, /* four-quadrant Riemann problem, quadrant states from SEED */
  WENOFD_SHEAR = 5           /* periodic shear layer on [0,1]^2 with seeded noise */
};

typedef struct wenofd_info {
  int nx, ny;             /* ELEMNUMX, ELEMNUMY (nodes incl. both boundary nodes) */
  int testcase, scheme, rk, precision;
  int bc_left, bc_right, bc_bottom, bc_top; /* BOUNDARYTYPE values */
  int has_exact;          /* equation->u_exact_exist */
  int pitch;              /* device row pitch, in elements */
  double dx, dy, cfl, t_end, now, gamma;
  double xl, xr, yl, yr;
  long long steps;        /* completed time steps */
  long long launches;     /* kernels this handle has enqueued (graph nodes counted per replay) */
  int graph_steps;        /* time steps per CUDA-graph replay in wenofd_advance (0: not built yet) */
  double dt;              /* the last time step (calculateDeltaT's deltaT); 0 before the first */
} wenofd_info;

/* Message describing the last failure on the calling thread ("" if none). */
const char *wenofd_last_error(void);
const char *wenofd_version(void);

/* CConfig::read + CWENOFD::initializeSolver (utils/readConfig.hpp:39-80,
 * src/WENOFD.cpp:10-164).  keys/values are the config.cfg pairs; required:
 * TESTCASE, ELEMNUMX, ELEMNUMY, RKMETH, CFL, SCHEME (src/WENOFD.cpp:24-40).
 * Optional keys the reference does not have: PRECISION (0 FP64, 1 FP32,
 * 2 learned + FP32), SEED (seeded cases), TEND (overrides
 * equation->outputtime), DEVICE, TILE_I (stage-kernel tile height; 0 =
 * default), LABEL_DEVIATION (training labels of wenofd_indicator_data;
 * default 1e-2), INDICATOR_INTERVAL (time steps per indicator run, see
 * wenofd_routing_flags; default 1), INDICATOR_GUARD (learned form: a node
 * is also flagged when the range of its 5x5 density or pressure window
 * exceeds this fraction of the centre value, so strong jumps take WENO-Z
 * whatever the network says; default 0 = off), and overrides of the
 * EulerEquation members the reference's callers may set on their equation
 * object (utils/equations.hpp:58-70): XL, XR, YL, YR, GAMMA, BC_LEFT,
 * BC_RIGHT, BC_BOTTOM, BC_TOP (BOUNDARYTYPE values), GRAVITY (0/1). */
int wenofd_create(const char *const *keys, const char *const *values, int n, wenofd_solver **out);
/* Same, reading a config.cfg file with the reference's parser semantics
 * (`key = value` lines, `#` comments, trimmed spaces and '\r'). */
int wenofd_create_from_file(const char *config_path, wenofd_solver **out);
int wenofd_destroy(wenofd_solver *s);
/* Run this handle's work on the caller's cudaStream_t (NULL: back to the
 * handle's own stream). */
int wenofd_set_stream(wenofd_solver *s, void *cuda_stream);
int wenofd_get_info(const wenofd_solver *s, wenofd_info *info);

/* CWENOFD::initializeAve (src/WENOFD.cpp:165-188): initial condition of the
 * configured case at every interior node; time and step count reset to 0. */
int wenofd_initialize(wenofd_solver *s);
/* Upload / download the interior state (host pointers, [4][NX][NY]). */
int wenofd_set_state(wenofd_solver *s, const double *host_state);
int wenofd_get_state(wenofd_solver *s, double *host_state);
/* Same with device pointers (no host round trip; stream-ordered). */
int wenofd_set_state_device(wenofd_solver *s, const double *dev_state);
int wenofd_get_state_device(wenofd_solver *s, double *dev_state);
/* Full state including the 4 ghost layers, [4][NX+8][NY+8] (host). */
int wenofd_get_state_ghosted(wenofd_solver *s, double *host_full);
int wenofd_set_time(wenofd_solver *s, double now);

/* Values of SPECIAL boundaries (getU0 at fixed boundary nodes,
 * src/WENOFD.cpp:1045-1058, 1092-1102, 1138-1149) for callers with their own
 * initial condition.  Table of 8*(NX+8) + 8*(NY+8) doubles, each block
 * r-major: bottom per ei at node (ei, 4); top per ei at (ei, NY+3); left per
 * ej at (4, ej); right per ej at (NX+4, ej) -- the first ghost column, as the
 * reference uses (line 1144).  ei, ej count the 4 ghost nodes. */
int wenofd_set_boundary_values(wenofd_solver *s, const double *host_table);

/* exchangeGhostCellsValue + setBoundary (src/WENOFD.cpp:850-929, 998-1159)
 * on the current state, in place. */
int wenofd_fill_boundary(wenofd_solver *s);
/* CWENOFD::assembleRHS (src/WENOFD.cpp:454-465; assembleBoundaryTerm
 * 481-798 is the "getFlux" of the reference README) of the current state:
 * boundary fill, x and y characteristic WENO sweeps, source term.  The
 * interior RHS [4][NX][NY] is written to host_rhs (may be NULL: kept on the
 * device only). */
int wenofd_get_flux(wenofd_solver *s, double *host_rhs);
/* CWENOFD::calculateDeltaT (src/WENOFD.cpp:398-452) of the current state. */
int wenofd_calc_dt(wenofd_solver *s, double *dt);
/* CWENOFD::RunRK1/2/3 (src/WENOFD.cpp:301-396) with the given step, per
 * RKMETH.  Does not advance the time. */
int wenofd_rk_step(wenofd_solver *s, double dt);
/* One iteration of the CWENOFD::run loop (src/WENOFD.cpp:213-239):
 * calculateDeltaT, RunRK, m_now += dt.  dt_out may be NULL. */
int wenofd_step(wenofd_solver *s, double *dt_out);
/* The CWENOFD::run time loop (src/WENOFD.cpp:213-284) until |now - t_end|
 * <= 1e-9 or max_steps more steps (max_steps < 0: no cap).  The time step
 * never leaves the device; steps run in CUDA-graph chunks.  steps_done may
 * be NULL. */
int wenofd_advance(wenofd_solver *s, long long max_steps, long long *steps_done);
/* CWENOFD::outputAccuracy norms (src/WENOFD.cpp:1308-1382) of density
 * against the exact solution at the current time: out = {Linf, L1, L2},
 * L1/L2 normalised by NX*NY.  FP64 device reduction. */
int wenofd_error_norms(wenofd_solver *s, double out[3]);
/* Interior sums of rho, rho*u, rho*v, E over all NX*NY nodes (FP64 device
 * reduction).  The grid is node-based: in a periodic direction the last node
 * duplicates the first, so these sums move by the duplicate row's change;
 * the conserved totals run over the unique nodes (drop the last row and
 * column of the state). */
int wenofd_conservation_sums(wenofd_solver *s, double out[4]);

/* CWENOFD::outputAve's variables (utils/equations.hpp:666-698,
 * src/WENOFD.cpp:1161-1238) of the current state, computed on the device in
 * FP64 with the reference's operation order: host_out receives
 * [6][NX][NY] doubles, planes rho, u, v, pre, c, E (the Tecplot VARIABLES
 * after X and Y).  Uses the stage buffers as scratch (between steps). */
int wenofd_output_variables(wenofd_solver *s, double *host_out);
/* Binary restart, no counterpart in the reference (its outputs are Tecplot
 * text).  wenofd_save_state writes a 96-byte header -- magic "WENOFDS1",
 * version 1, NX, NY, TESTCASE, SCHEME, RKMETH, PRECISION, step count, time,
 * TEND, dx, dy, gamma, CFL -- and the interior state [4][NX][NY] float64,
 * all little-endian.  wenofd_load_state reads such a file into a handle of
 * the same grid and TESTCASE (else WENOFD_BAD_CONFIG) and sets its state,
 * time and step count; a run continued from it is bit for bit the run that
 * wrote it. */
int wenofd_save_state(wenofd_solver *s, const char *path);
int wenofd_load_state(wenofd_solver *s, const char *path);

/* Measurement aid, no reference counterpart: replays the RK stage kernels of
 * one step (RKMETH's stages, boundary fills excluded, dt as last set) `reps`
 * times on the handle's stream between two CUDA events and returns the mean
 * duration of one stage-kernel launch in milliseconds.  It advances the
 * state; callers re-upload a state afterwards. */
int wenofd_time_stages(wenofd_solver *s, int reps, double *ms_per_launch);

/* ---- Learned troubled-cell indicator (no counterpart in the reference) ----
 * Network: 50 inputs (5x5 windows of density and pressure, each normalised
 * as (v - v_centre) / max|v - v_centre|, zero when that range is <= 1e-4 of
 * |v_centre|) -> 32 -> 32 -> 1, GELU (tanh form) hidden layers, sigmoid
 * output.  Parameters are WENOFD_MLP_PARAMS floats: W1[32][50], b1[32],
 * W2[32][32], b2[32], w3[32], b3. */
#define WENOFD_MLP_INPUTS 50
#define WENOFD_MLP_PARAMS 2721

/* Load trained parameters (host, FP32; converted to BF16 for the tensor
 * cores) into a PRECISION = 2 solver; nodes whose predicted probability
 * exceeds `threshold` are flagged.  Without it every face takes WENO. */
int wenofd_set_indicator(wenofd_solver *s, const float *host_params, float threshold);
/* Run the indicator on the current state; flags [NX][NY] bytes to the host
 * (they also become the stored routing flags). */
int wenofd_indicator_flags(wenofd_solver *s, unsigned char *host_flags);
/* The stored routing flags [NX][NY] as they are (no indicator run): those of
 * the indicator's last run, which routed the last step.  In the time loop
 * the indicator runs on the first step of every wenofd_advance call and then
 * on every INDICATOR_INTERVAL-th step (config key, default 1); the steps in
 * between route with the flags of its last run. */
int wenofd_routing_flags(wenofd_solver *s, unsigned char *host_flags);
/* Training data of the current state: features [NX*NY][50] float and labels
 * [NX*NY] bytes (1 where WENO-Z's nonlinear weights differ from the linear
 * ones by more than LABEL_DEVIATION, default 1e-2, on a non-flat stencil at
 * any of the node's four faces), device pointers; either may be NULL. */
int wenofd_indicator_data(wenofd_solver *s, float *dev_features, unsigned char *dev_labels);
/* Balanced training sample of the current state, formed on the device:
 * labels of every node as wenofd_indicator_data forms them, then about
 * per_snapshot / 2 flagged and per_snapshot / 2 unflagged nodes (fewer of a
 * class that has fewer; the other class fills in), each node of a class kept
 * independently when a hash of (seed, node index) falls below that class's
 * rate; the same state and seed keep the same nodes.  The kept nodes'
 * features go to dev_x[row][50] and their labels (0.0 / 1.0) to dev_y[row],
 * rows in node order, at most `capacity` rows; *rows_out receives the count
 * (it varies around per_snapshot by the sampling).  Synchronous.  Replaces
 * the host-side sampling a training driver would otherwise need. */
int wenofd_indicator_sample(wenofd_solver *s, long long per_snapshot, unsigned long long seed, float *dev_x,
                            float *dev_y, long long capacity, long long *rows_out);
/* FP32 training kernels on device buffers (stream-ordered):
 *   forward: logits[n] of samples x[n][50];
 *   backward: mean binary cross-entropy of logits vs y[n] (0/1) into *loss and
 *             its gradient into grad[WENOFD_MLP_PARAMS] (both overwritten);
 *   adam: one Adam step (beta 0.9 / 0.999, eps 1e-8), step counts from 1;
 *   train: per epoch a seeded random permutation of the n samples, cut
 *          into mini-batches of backward + adam (the samples may come in
 *          any order), the mean loss of each epoch to host_epoch_loss[epochs]
 *          (may be NULL); each mini-batch's gradient is summed in a fixed
 *          order, so the same data and seed give the same parameters bit for
 *          bit (the standalone backward accumulates with atomics).  It
 *          allocates its optimiser state and an 8-byte index per sample. */
int wenofd_mlp_forward(const float *dev_params, const float *dev_x, long long n, float *dev_logits, void *stream);
int wenofd_mlp_backward(const float *dev_params, const float *dev_x, const float *dev_y, long long n,
                        float *dev_grad, float *dev_loss, void *stream);
int wenofd_mlp_adam(float *dev_params, const float *dev_grad, float *dev_m, float *dev_v, int step, float lr,
                    void *stream);
int wenofd_mlp_train(float *dev_params, const float *dev_x, const float *dev_y, long long n, int epochs, int batch,
                     float lr, unsigned long long seed, float *host_epoch_loss, void *stream);
/* Initial parameters for training (host buffer of WENOFD_MLP_PARAMS floats,
 * host-only, no GPU needed): W1 uniform in +-sqrt(6/50), W2 and w3 uniform
 * in +-sqrt(6/32), biases zero, from a seeded splitmix64 sequence; the same
 * seed gives the same parameters everywhere. */
int wenofd_mlp_init(float *host_params, unsigned long long seed);

/* ---- Batches: many independent solves in one persistent launch ----------
 * No counterpart in the reference, which runs one solve per program
 * (src/main.cpp:8-30); a batch replaces N runs of the time loop of
 * CWENOFD::run (src/WENOFD.cpp:213-224, calculateDeltaT + RunRK3 + m_now += dt)
 * by one kernel launch per few steps that advances every member.
 *
 * Members are existing handles: same device, same SCHEME, same RKMETH (RK1,
 * SSP-RK2 or SSP-RK3) and the same PRECISION (FP64, FP32 or LEARNED; learned
 * members also the same INDICATOR_INTERVAL); sizes, test cases, boundary
 * conditions, CFL, TEND and the learned members' indicator weights and
 * thresholds may differ.  The
 * batch works on the members' own device state: a member stepped by a
 * batch is read (wenofd_get_state, wenofd_get_info, wenofd_routing_flags,
 * ...) through its own handle; members must outlive the batch and must not
 * be advanced through their own handles while a batch call runs.  Each
 * member's steps are those of wenofd_advance on its own: FP64 members bit
 * for bit.  Learned members: one tensor-core indicator launch over all of
 * them runs on the first step of every wenofd_batch_advance call and then
 * every INDICATOR_INTERVAL steps (between launches of the batched kernel,
 * which routes each member's faces with its flags), as in wenofd_advance;
 * a member without weights (no wenofd_set_indicator) routes every face to
 * WENO.  Weights loaded on a member reach the batch's next call.
 *
 * wenofd_batch_configure: tile rows per stage tile (FP64: 7 or 15, FP32 and
 *   learned: 15 or 31; 0 = default 15), resident blocks per SM (0 = as many
 *   as fit) and steps per launch (0 = chosen from the batch's size; learned
 *   batches round it up to whole INDICATOR_INTERVAL runs of steps, each its
 *   own launch after an indicator launch).
 * wenofd_batch_autotune: times each (tile, blocks per SM) candidate over
 *   `steps` steps, keeps the fastest and returns its milliseconds per step;
 *   the members' states and times are restored after every trial.
 * wenofd_batch_advance: like wenofd_advance for every member: each member
 *   steps until its TEND or `max_steps` more steps (-1: no limit).
 *   *steps_done receives the largest number of steps a member took.
 *   WENOFD_NAN_DT if a member's time step became NaN (that member stops,
 *   the others finish the call; the message names the member index);
 *   WENOFD_TIMEOUT if a grid barrier wait or a tensor-core completion wait
 *   of the batched indicator gave up. */
typedef struct wenofd_batch wenofd_batch;

typedef struct wenofd_batch_info {
  int members;
  int precision;
  int tile_i;            /* tile rows of the stage tiles */
  int blocks_per_sm;     /* resident blocks per SM of the persistent kernel */
  int grid;              /* blocks per launch */
  int steps_per_launch;  /* time steps one launch (learned: one graph replay) runs */
  int graph;             /* 1: launches are replays of a captured CUDA graph */
  long long cells;       /* interior nodes over all members */
  long long launches;    /* kernels launched by this batch so far */
  double tuned_ms_per_step; /* from wenofd_batch_autotune, else 0 */
} wenofd_batch_info;

int wenofd_batch_create(wenofd_solver *const *members, int n, wenofd_batch **out);
int wenofd_batch_destroy(wenofd_batch *b);
int wenofd_batch_configure(wenofd_batch *b, int tile_i, int blocks_per_sm, int steps_per_launch);
int wenofd_batch_autotune(wenofd_batch *b, int steps, double *ms_per_step);
int wenofd_batch_advance(wenofd_batch *b, long long max_steps, long long *steps_done);
int wenofd_batch_get_info(const wenofd_batch *b, wenofd_batch_info *info);
/* Test hook, no counterpart in the reference (whose failures abort,
 * src/WENOFD.cpp:437-442): arms the next wenofd_batch_advance to run its
 * first launch on a separately compiled instance of the batched kernel
 * (FP64 WENO-Z batches, tile 15 only) whose grid barrier polls at most 4096
 * times, and in which block `block` does not arrive at the launch's barrier
 * number `barrier` (0 = the first).  Every wait at that barrier gives up,
 * every later wait ends within 1024 polls, and the advance returns
 * WENOFD_TIMEOUT; the members' states are then undefined and the batch can
 * be advanced again after the members are re-initialised.  The kernels of
 * the normal path carry no part of this hook. */
int wenofd_batch_test_withhold(wenofd_batch *b, int block, int barrier);

/* No counterpart in the reference.  calculateDeltaT (src/WENOFD.cpp:398-452
 * arithmetic, bit for bit) of a caller-owned device state, for callers that
 * must not allocate: an application whose GPU memory belongs to its own pool
 * and that lends this library only its state buffers, or a time loop that
 * cannot absorb cudaMalloc/cudaFree, which synchronise the whole device.
 * Needs no handle and allocates nothing; it only enqueues two kernels.
 *   dev_state  interior state, device memory, float64 [4][nx][ny] (ej fastest)
 *   dev_dt     device double that receives dt, or NaN if any node's wave speed
 *              is NaN.  This is stricter than the reference, whose loop
 *              (src/WENOFD.cpp:426-442) lets a later finite node overwrite a
 *              NaN candidate and aborts only when the last candidate is NaN.
 *   stream     cudaStream_t (NULL: the default stream); the call returns
 *              without waiting for the result.
 * Limit: nx*ny <= 2^28 nodes (16384 x 16384); larger grids are rejected with
 * WENOFD_BAD_ARG and a message.  Scratch: a fixed 8 KiB __device__ array in
 * the library (per-block maxima), held by every GPU that loads the library
 * until exit.  The first call on a device looks up that array's address
 * (with the device current), so make it before any stream capture on that
 * device; so is the first call after a device reset (cudaDeviceReset), which
 * looks the address up again.  All calls share the array: calls that
 * overlap on the GPU race. */
int wenofd_calc_dt_noalloc(const double *dev_state, int nx, int ny, double dx, double dy, double gamma,
                           double cfl, double now, double t_end, double *dev_dt, void *stream);

/* Index guards of the bounds-checked debug library (built with
 * `python fd-weno-eulerequation_gb300/build.py --bounds-check`, i.e. with
 * -DWENOFD_BOUNDS_CHECK, into fd-weno-eulerequation_gb300/_build_check/).  It
 * stands in for the reference's assert-checked Array1D/Array2D indexing
 * (utils/array.h:273-303, 552-583): every kernel tests its state, flag, table,
 * work-item and shared-memory indices, and the TMA boxes' first coordinates,
 * against their extents; an index out of range is counted in the current
 * device's guard record and not used (the access goes to element 0 of the
 * same array).  report[0] = violations since the last reset, report[1] = the
 * first one's source line, report[2] = its index, report[3] = the extent (or
 * alignment) it broke; `where` (if not null, where_len bytes) receives the
 * first one's "file:line".  Waits for the device to finish its work first;
 * reset != 0 zeroes the record afterwards.  In the release library
 * report[0] = -1 (no guards compiled) and report[1..3] = 0. */
int wenofd_bounds_report(long long report[4], char *where, int where_len, int reset);

/* The guard mechanism itself, in either library: one kernel makes one guarded
 * access one past the end of a 4-element array (the guard sends it to
 * element 0) against a private record, returned as in wenofd_bounds_report:
 * report = {1, line, 4, 4}, `where` naming the self-test's source line. */
int wenofd_bounds_selftest(long long report[4], char *where, int where_len);

#ifdef __cplusplus
}
#endif

#endif
