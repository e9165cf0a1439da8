/*
 * gbde.h -- C ABI of the GB300 ensemble ODE/SDE solver (libgbde.so).
 *
 * This is the drop-in boundary for the data-parallel hot path of
 * DifferentialEquations.jl:
 *
 *     solve(EnsembleProblem(prob; prob_func), alg, ensemblealg;
 *           trajectories, saveat, reltol, abstol)
 *
 * The reference re-exports that surface from SciMLBase / OrdinaryDiffEq
 * (src/DifferentialEquations.jl:8-9); the names it allow-lists are
 * EnsembleProblem (test/qa/qa.jl:50), EnsembleThreads (qa.jl:56),
 * solve (qa.jl:192), remake (qa.jl:183), ReturnCode (qa.jl:213),
 * Tsit5 (qa.jl:119), Vern7 (qa.jl:126), Rosenbrock23 (qa.jl:98),
 * Rodas5P (qa.jl:97), SDEProblem (qa.jl:103).  The per-trajectory solve
 * that EnsembleThreads maps over trajectories lives in OrdinaryDiffEq v7 /
 * SciMLBase v3 (Project.toml:13,18), which the reference does not vendor.
 *
 * gbde_ensemble_solve() replaces the whole
 *     SciMLBase.__solve(::EnsembleProblem, alg, ::EnsembleAlgorithm)
 * branch: the host evaluates prob_func into structure-of-arrays inputs,
 * makes ONE call, and wraps the returned arrays as per-trajectory solutions.
 *
 * Conventions
 *   - Every function returns an int status: GBDE_OK (0) or a negative
 *     GBDE_ERR_* code; gbde_last_error() describes the last failure.
 *   - No call aborts the process; per-trajectory outcomes are written to
 *     outputs.retcode[] (GBDE_RET_*), never raised.
 *   - Arrays are C-order ("row-major"); the trajectory index is the slowest
 *     dimension of every per-trajectory array, which is Julia's column-major
 *     Array{Float64}(n, N) / Array{Float64,3}(n_state, n_save, N).
 *   - A context is bound to one device and one CUDA stream; calls on one
 *     context are serialised by an internal mutex.
 */
#ifndef GBDE_H
#define GBDE_H

#ifndef __CUDACC_RTC__ /* runtime-compiled device code (rtc.cu) defines these types */
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBDE_ABI_VERSION 4

#if defined(__GNUC__)
#define GBDE_API __attribute__((visibility("default")))
#else
#define GBDE_API
#endif

/* ---- status codes ------------------------------------------------------ */
#define GBDE_OK 0
#define GBDE_ERR_INVALID (-1)     /* bad argument (sizes, pointers, enums) */
#define GBDE_ERR_CUDA (-2)        /* a CUDA runtime call failed           */
#define GBDE_ERR_UNSUPPORTED (-3) /* valid but not implemented combination */
#define GBDE_ERR_TIMEOUT (-4)     /* device work gave up after its deadline */
#define GBDE_ERR_NOMEM (-5)       /* device or pinned allocation failed    */
#define GBDE_ERR_STATE (-6)       /* e.g. learned=1 without a loaded MLP   */

/* ---- per-trajectory return codes (SciMLBase ReturnCode, qa.jl:213) ---- */
#define GBDE_RET_DEFAULT 0        /* not solved                            */
#define GBDE_RET_SUCCESS 1        /* ReturnCode.Success                    */
#define GBDE_RET_MAXITERS 2       /* ReturnCode.MaxIters                   */
#define GBDE_RET_DTLESSTHANMIN 3  /* ReturnCode.DtLessThanMin              */
#define GBDE_RET_UNSTABLE 4       /* ReturnCode.Unstable (non-finite state)*/
#define GBDE_RET_INITIALFAILURE 5 /* ReturnCode.InitialFailure (bad input) */
#define GBDE_RET_TIMEOUT 6        /* device deadline hit (no Julia analog) */
#define GBDE_RET_TERMINATED 7     /* ReturnCode.Terminated (a callback ended it) */

/* callback kinds (gbde_callback.kind) */
#define GBDE_CB_CONTINUOUS 1      /* ContinuousCallback (qa.jl:24)         */
#define GBDE_CB_DISCRETE 2        /* DiscreteCallback (qa.jl:36)           */
#define GBDE_CB_VECTOR 3          /* VectorContinuousCallback (qa.jl:124)  */
/* most continuous conditions one solve's callback (set) may carry */
#define GBDE_MAX_CB_CONDITIONS 64

/* ---- built-in right-hand sides (ODEFunction f!(du,u,p,t), qa.jl:84) ---- */
#define GBDE_MODEL_LINEAR 1    /* n=1, p=[a]:           du = a*u (test/core.jl:10) */
#define GBDE_MODEL_LORENZ 2    /* n=3, p=[sigma,rho,beta]          (test/core.jl:22-27) */
#define GBDE_MODEL_ROBERTSON 3 /* n=3, p=[k1,k2,k3]                (test/core.jl:39-45) */
#define GBDE_MODEL_VDP_RING8 4 /* n=16, p=[mu,kappa]: 8 Van der Pol oscillators on a ring;
                                  Tsit5 / Rodas5 / Rodas5P run 16 lanes per trajectory */
#define GBDE_MODEL_LOTKA_VOLTERRA 5 /* n=2, p=[alpha,beta,gamma,delta,sigma]:
                                       drift [a x - b x y, d x y - g y],
                                       diagonal noise sigma*u (SDE)            */
/* User models (gbde_model_register) get ids from GBDE_MODEL_USER_BASE up. */
#define GBDE_MODEL_USER_BASE 1000
#define GBDE_USER_MAX_STATE 8
#define GBDE_USER_MAX_PARAM 32

/* ---- algorithms ------------------------------------------------------- */
#define GBDE_ALG_TSIT5 1        /* Tsitouras 5(4), FSAL, free 4th-order interpolant */
#define GBDE_ALG_VERN7 2        /* Verner 7(6)                                      */
#define GBDE_ALG_ROSENBROCK23 3 /* Shampine-Reichelt 2(3) W-method                  */
#define GBDE_ALG_RODAS5 4       /* Di Marzo 5(4) Rosenbrock, stiffly accurate       */
#define GBDE_ALG_RODAS5P 5      /* Steinebach 5(4) Rosenbrock                       */
#define GBDE_ALG_EM 6           /* Euler-Maruyama, fixed step                       */
#define GBDE_ALG_SOSRI 7        /* SOSRI (Rackauckas & Nie 2018): stability-optimised
                                   SRI of strong order 1.5, adaptive with rejection
                                   sampling with memory (SOSRI, SDEProblem qa.jl:103) */
#define GBDE_ALG_AUTO 8         /* per-trajectory Tsit5 / Rodas5 choice, made once
                                   before integration: stiff iff p[0] >
                                   stiff_threshold (or the learned predictor's label);
                                   stands in for AutoTsit5(Rosenbrock23()),
                                   test/qa/qa.jl:15.  Stiff trajectories always run
                                   Rodas5 in FP64; with GBDE_PREC_MIXED the others run
                                   Tsit5 with FP32 state.                             */

#define GBDE_ALG_SRIW1 9        /* SRIW1 (Roessler 2010): SRI of strong order 1.5,
                                   adaptive with rejection sampling with memory      */
/* AutoTsit5(Rosenbrock23()) / AutoTsit5(Rodas5()) (test/qa/qa.jl:15): per
 * trajectory, run-time switching.  Tsit5 estimates the Jacobian's spectral
 * radius from its last two stages, the stiff method takes ||J||_inf; before
 * every attempt after the first, stiffness = |eig dt / 3.5068| > 0.9 counts
 * towards a switch: more than 10 successive stiff estimates switch Tsit5 to
 * the stiff method (dt * 2), more than 3 successive non-stiff ones switch
 * back (dt / 2) -- OrdinaryDiffEq's AutoSwitch with its defaults.  Each method
 * steps with its own PI exponents (Tsit5's are the options', the stiff
 * method's its defaults).  outputs.method: the method of the last step.
 * Built-in models with n <= 3 and user models; FP64 or GBDE_PREC_MIXED. */
#define GBDE_ALG_AUTOTSIT5_ROSENBROCK23 10
#define GBDE_ALG_AUTOTSIT5_RODAS5 11

/* ---- precision -------------------------------------------------------- */
#define GBDE_PREC_FP64 0  /* everything in FP64                                  */
#define GBDE_PREC_MIXED 1 /* FP32 state and stages; FP64 compensated time, FP64
                             error norm, FP64 W-matrix LU                         */
#define GBDE_PREC_F32X2 2 /* state, stages and right-hand sides as unevaluated
                             pairs of FP32 (~48-bit significand) on the FP32 pipe;
                             FP64 W-matrix LU (solves on its pair-rounded factors),
                             FP64 error norm and compensated time.  One thread per
                             trajectory ODE kernels (not SDE, not the 16-state
                             ring, not AUTO)                                       */

/* ---- batching --------------------------------------------------------- */
#define GBDE_BATCH_PLAIN 0      /* one thread per trajectory, one launch      */
#define GBDE_BATCH_PERSISTENT 1 /* persistent CTAs refill finished threads from a
                                   device work queue (longest trajectories first) */

/* ---- save-time layout ------------------------------------------------- */
#define GBDE_SAVE_GRID 0     /* saveat[n_save] shared by all trajectories   */
#define GBDE_SAVE_PER_TRAJ 1 /* saveat[N][n_save]                             */

/* ---- memory space of the problem / output pointers -------------------- */
#define GBDE_MEM_HOST 0   /* host pointers: the call copies H2D and D2H; a
                             page-locked, device-mapped outputs.u
                             (cudaHostAlloc / cudaHostRegister) is written
                             by the kernels directly, without a copy      */
#define GBDE_MEM_DEVICE 1 /* device pointers on the context's device: no copies */

/* ---- output element type ---------------------------------------------- */
#define GBDE_F64 0
#define GBDE_F32 1

typedef struct gbde_ctx gbde_ctx;

/* One ensemble: N trajectories of the same model with per-trajectory
 * parameters, initial states and time spans (the result of prob_func /
 * remake over i = 1..N).  Save times must be non-decreasing and lie in
 * [t0_i, tf_i]; a save time equal to t0_i stores u0_i exactly (the
 * reference pins sol.u[1] == u0 at test/core.jl:34), one equal to tf_i
 * stores the final state.  The host layer decides whether t0 / tf are in
 * the list (save_start / save_end; test/core.jl:90-96 expects 11 points
 * for saveat=0.1 on (0,1)). */
typedef struct {
  int32_t model;       /* GBDE_MODEL_*                                     */
  int32_t n_state;     /* must equal the model's state size               */
  int32_t n_param;     /* must equal the model's parameter count          */
  int32_t mem;         /* GBDE_MEM_HOST or GBDE_MEM_DEVICE                */
  int64_t n_traj;      /* N >= 0                                          */
  const double* p;     /* [N][n_param]                                    */
  const double* u0;    /* [N][n_state]                                    */
  const double* t0;    /* [N]                                             */
  const double* tf;    /* [N], tf_i >= t0_i                               */
  int32_t save_kind;   /* GBDE_SAVE_GRID or GBDE_SAVE_PER_TRAJ            */
  int32_t n_save;      /* >= 0 save times per trajectory                  */
  const double* saveat;/* [n_save] or [N][n_save]                         */
} gbde_problem;

/* Solver options: the solve() keyword arguments of the reference
 * (reltol, abstol, dt, adaptive, maxiters, dtmin, dtmax, qmin, qmax, gamma,
 * beta1, beta2, qsteady_min, qsteady_max, qoldinit; seed for the noise).
 * Fill with gbde_opts_default() and override. */
typedef struct {
  int32_t alg;         /* GBDE_ALG_*                                      */
  int32_t precision;   /* GBDE_PREC_*                                     */
  int32_t batching;    /* GBDE_BATCH_*                                    */
  int32_t adaptive;    /* 1 = error-controlled steps; 0 = fixed dt        */
  double reltol, abstol;
  double dt;           /* initial dt (0 = automatic), or the fixed step   */
  double dtmin;        /* a step below dtmin ends with DtLessThanMin      */
  double dtmax;        /* 0 = unlimited                                   */
  int64_t maxiters;    /* attempted steps per trajectory                  */
  double qmin, qmax, gamma, beta1, beta2, qsteady_min, qsteady_max, qoldinit;
  uint64_t seed;       /* Philox key for SDE noise                        */
  int32_t learned;     /* GBDE_LEARN_* flags (0 = no learned predictor)   */
  int32_t block_size;  /* threads per CTA (0 = tuned default)             */
  int32_t chunk;       /* persistent-queue trajectories per fetch (0 = default) */
  int32_t ctas_per_sm; /* persistent CTAs per SM (0 = tuned default)      */
  double stiff_threshold; /* GBDE_ALG_AUTO without MLP: stiff iff p[0] > this */
  double timeout_s;    /* device deadline per call (0 = none)             */
  int32_t threads_per_traj; /* 0 = model default; 1 = one thread per trajectory;
                          16 = a 16-lane team (16-state models)            */
  int32_t callback;    /* 0, or an id from gbde_callback_register          */
} gbde_opts;

/* Results.  u is [N][n_save][n_state] of u_dtype; retcode [N]; the step
 * statistics may be NULL. */
typedef struct {
  void* u;             /* [N][n_save][n_state]                            */
  int32_t u_dtype;     /* GBDE_F64 or GBDE_F32                            */
  int32_t* retcode;    /* [N] GBDE_RET_*                                  */
  int32_t* naccept;    /* [N] or NULL: accepted steps                     */
  int32_t* nreject;    /* [N] or NULL: rejected steps                     */
  int32_t* nf;         /* [N] or NULL: right-hand-side evaluations        */
  double* t_end;       /* [N] or NULL: time reached                       */
  int32_t* method;     /* [N] or NULL: GBDE_ALG_* actually used (AUTO)    */
  float device_ms;     /* out: device time of the solve kernels           */
  float total_ms;      /* out: wall time of the whole call                */
  double* dt_first;    /* [N] or NULL: size of the first accepted step (the
                          step log the learned predictor is trained on)   */
  double* reduce;      /* [2][n_save][n_state] or NULL: the sums over
                          trajectories of each saved state and of its
                          square, accumulated inside the step kernels
                          (EnsembleProblem's reduction, qa.jl:50: moments
                          without storing the ensemble).  With u = NULL
                          the ensemble is not stored at all.  Additions
                          run in no fixed order (FP64 atomics).          */
  /* Saves at callback events (the callbacks' save_positions; solves with
   * opts.callback only, ignored otherwise).  Trajectory i's k-th event save
   * is (ev_t[i][k], ev_u[i][k][:]) for k < min(ev_count[i], ev_capacity), in
   * the order made; ev_u has u_dtype.  ev_count[i] counts every save the
   * trajectory made, also those beyond ev_capacity (not stored): a caller
   * that finds ev_count[i] > ev_capacity solves again with a larger one.
   * ev_count NULL: no event saves.                                        */
  double* ev_t;        /* [N][ev_capacity] or NULL                          */
  void* ev_u;          /* [N][ev_capacity][n_state] or NULL                 */
  int32_t* ev_count;   /* [N] or NULL                                       */
  int32_t ev_capacity; /* event saves per trajectory the buffers hold       */
} gbde_outputs;

/* ABI version of the loaded library (GBDE_ABI_VERSION). */
GBDE_API int gbde_version(void);

/* Create a context on CUDA device `device`; allocates nothing large. */
GBDE_API int gbde_ctx_create(int device, gbde_ctx** out);
/* Destroy a context and release its device/pinned buffers. NULL is a no-op. */
GBDE_API int gbde_ctx_destroy(gbde_ctx* ctx);
/* Description of the last error on ctx (valid until the next call on it);
 * with ctx == NULL, the last context-less error of this thread. */
GBDE_API const char* gbde_last_error(const gbde_ctx* ctx);
/* Use `stream` (a cudaStream_t on the context's device, or NULL for the
 * context's own stream) for all following launches and copies. */
GBDE_API int gbde_ctx_set_stream(gbde_ctx* ctx, void* stream);

/* Fill `out` with this library's defaults for algorithm `alg`. */
GBDE_API int gbde_opts_default(int32_t alg, gbde_opts* out);

/* Solve the ensemble.  Blocks until the results are in `out` (host mode) or
 * the kernels have finished (device mode). */
GBDE_API int gbde_ensemble_solve(gbde_ctx* ctx, const gbde_problem* prob,
                        const gbde_opts* opts, gbde_outputs* out);

/* ---- CUDA graphs ---------------------------------------------------------
 * Capture the whole device work of one solve of a device-memory problem
 * (queue and status words, learned predictions, queue order, step kernels)
 * as a CUDA graph; gbde_graph_launch replays it on the context's stream.
 * The graph keeps the problem's and outputs' device pointers: refill the
 * input arrays in place between launches.  No counterpart in the reference
 * (batching of repeated ensembles at launch-free cost).
 * GBDE_ALG_AUTO cannot be captured (it sizes its launches on the host). */
typedef struct gbde_graph gbde_graph;
GBDE_API int gbde_graph_create(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                      gbde_outputs* out, gbde_graph** graph);
/* Replays and waits; device_ms (may be NULL) receives the replay's time. */
GBDE_API int gbde_graph_launch(gbde_graph* graph, float* device_ms);
GBDE_API int gbde_graph_destroy(gbde_graph* graph);

/* ---- autotuner -----------------------------------------------------------
 * Times the solve of `prob` under each launch configuration -- batching,
 * block size, resident CTAs per SM, persistent-queue chunk and (16-state
 * ring, Tsit5) threads per trajectory -- `reps` times each, writes the
 * fastest options to *best and the timing table to table[0..*n_entries),
 * and leaves the results of a final run with *best in `out`.  No
 * counterpart in the reference. */
typedef struct {
  int32_t batching, block_size, ctas_per_sm, chunk, threads_per_traj;
  float device_ms;     /* best of reps; 1e30 if the configuration failed  */
} gbde_tune_entry;
GBDE_API int gbde_autotune(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                  gbde_outputs* out, int32_t reps, gbde_opts* best,
                  gbde_tune_entry* table, int32_t table_cap, int32_t* n_entries);

/* Model metadata: state and parameter counts of a built-in model. */
GBDE_API int gbde_model_info(int32_t model, int32_t* n_state, int32_t* n_param);

/* Host regeneration of the noise stream: the standard normals the SDE
 * kernels draw for trajectory `traj` at draw indices counter..counter+n-1
 * (two normals per Philox4x32-10 block in FP64).  Bit-identical to the
 * device stream; lets a caller reproduce any trajectory's Brownian path. */
GBDE_API int gbde_philox_normals(uint64_t seed, uint64_t traj, uint64_t counter,
                        int64_t n, double* out);
/* Raw Philox4x32-10 block: out[4] = philox(ctr[4], key[2]). */
GBDE_API int gbde_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);

/* ---- solve without device allocation -------------------------------------
 * No counterpart in the reference: this entry point exists for callers of
 * this library that must not allocate device memory -- code inside a
 * real-time loop where cudaMalloc's implicit device synchronisation is not
 * allowed, a process whose device memory is owned by one allocator (a
 * framework's caching pool, the array pool of a garbage-collected host
 * language), or an embedding with a fixed device-memory budget.
 *
 * Same problem, options and outputs as gbde_ensemble_solve(), with these
 * differences:
 *   - every problem and output pointer is device memory on the calling
 *     thread's current device (prob->mem must be GBDE_MEM_DEVICE);
 *   - no context: the work runs on `stream` (NULL = the legacy default
 *     stream) and errors are read with gbde_last_error(NULL);
 *   - it calls no cudaMalloc / cudaFree / allocating library routine.  The
 *     solve's scratch (the persistent work-queue counter and the status word
 *     of the device deadline, 16 bytes whatever the ensemble size) lives in a
 *     static device array of GBDE_NOALLOC_SCRATCH_BYTES inside libgbde.so,
 *     which every GPU that loads the library holds until the process exits.
 *     A solve whose scratch would exceed that array is rejected with
 *     GBDE_ERR_INVALID;
 *   - the first call on a device looks up that array's device address
 *     (cudaGetSymbolAddress, with the device current); make that first call
 *     before any stream capture;
 *   - every call on a device shares the one array, which keeps the last
 *     call's contents (each call clears what it needs in stream order).
 *     Calls that overlap on the GPU race: serialise them on one stream or
 *     with events;
 *   - options and sizes are checked as gbde_ensemble_solve checks them; in
 *     addition these are rejected: learned != 0 (GBDE_ERR_STATE: no
 *     predictor), GBDE_ALG_AUTO (GBDE_ERR_UNSUPPORTED: its per-trajectory lists
 *     grow with n_traj), callback != 0 and user models (GBDE_ERR_UNSUPPORTED:
 *     their kernels are compiled and loaded by gbde_ensemble_solve),
 *     out->reduce (GBDE_ERR_UNSUPPORTED), GBDE_PREC_F32X2 on the 16-state ring
 *     (GBDE_ERR_UNSUPPORTED);
 *   - the device deadline (timeout_s) works as in gbde_ensemble_solve: the
 *     status word in the static array reports it (GBDE_ERR_TIMEOUT);
 *   - device_ms is not measured (0);
 *   - the device address of the array is looked up once per device and kept
 *     for the process: after a cudaDeviceReset the entry point must not be
 *     called again in that process.
 * Blocks until the kernels have finished. */
#define GBDE_NOALLOC_SCRATCH_BYTES 256
GBDE_API int gbde_ensemble_solve_noalloc(const gbde_problem* prob, const gbde_opts* opts,
                                gbde_outputs* out, void* stream);

/* Measure the device's FP64 / FP32 FMA throughput (TFLOP/s, FMA = 2 flops)
 * with a dependent-chain-free FMA loop; kind 0 = FP64, 1 = FP32.  kind 2
 * measures the rate of the SDE kernels' FP32 normal stream (Philox4x32-10 and
 * Box-Muller, as gbde_philox_normals defines it) in 10^12 normals/s.  No
 * counterpart in the reference (roofline denominators for this library). */
GBDE_API int gbde_measure_fma_peak(gbde_ctx* ctx, int32_t kind, double* tflops);

/* ---- learned step-size / stiffness / cost predictor ----------------------
 * No counterpart in the reference (its nearest relative is the runtime
 * stiffness switching of AutoTsit5(Rosenbrock23()), test/qa/qa.jl:15).
 * A 4-layer MLP 8 -> 64 -> 64 -> 64 -> 3 with GELU, BF16 weights and FP32
 * accumulation maps 8 features of a trajectory (its parameters, initial state
 * and time span; gbde_mlp_features) to (log10 of the first accepted dt,
 * logit of "stiff", log2 of the attempted steps).  A solve with opts.learned
 * != 0 runs the loaded network first:
 *   GBDE_LEARN_START: the predicted dt replaces the Hairer-Wanner starting
 *     step, and GBDE_ALG_AUTO uses the stiff label instead of the threshold;
 *   GBDE_LEARN_STIFF: GBDE_ALG_AUTO uses the stiff label; every trajectory
 *     starts from the Hairer-Wanner step, so it takes the steps the method
 *     takes without the predictor;
 *   GBDE_LEARN_ORDER: the persistent queue hands out trajectories by
 *     predicted cost, highest first, instead of longest span first -- the
 *     lanes of a warp then carry trajectories of similar step counts.  Each
 *     trajectory's result does not depend on the order.
 * The error controller still accepts or rejects every step.
 * Network blob: GBDE_MLP_NET_FLOATS floats, FP32:
 *   W1[8][64] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64][3] b4[3]
 *   x_mean[8] x_scale[8] y_mean y_scale c_mean c_scale                    */
#define GBDE_MLP_IN 8
#define GBDE_MLP_OUT 3
#define GBDE_MLP_PARAMS 9091
#define GBDE_MLP_NET_FLOATS 9111
#define GBDE_LEARN_START 1 /* learned first dt and AUTO method choice          */
#define GBDE_LEARN_ORDER 2 /* persistent queue ordered by the learned cost     */
#define GBDE_LEARN_STIFF 4 /* AUTO method choice only (Hairer-Wanner start)    */

typedef struct {
  int32_t epochs;      /* passes over the data                              */
  int32_t batch;       /* minibatch size                                    */
  float lr;            /* AdamW learning rate                               */
  float weight_decay;  /* decoupled weight decay (matrices only)            */
  uint64_t seed;       /* minibatch shuffling                               */
} gbde_mlp_train_opts;

/* He-uniform initial weights (seeded), identity normalisation. */
GBDE_API int gbde_mlp_init(uint64_t seed, float* net);
/* features[N][8] (device memory) of every trajectory of a device-memory
 * problem. */
GBDE_API int gbde_mlp_features(gbde_ctx* ctx, const gbde_problem* prob, float* features);
/* Train on the GPU: x[n][8] features, y[n][3] targets (log10 first accepted
 * dt, stiff label 0/1, log2 attempted steps; NaN = no label), host memory.  `net` holds the initial
 * weights on entry and the trained network on return (the normalisation
 * fields are set from the data); loss_history[epochs] may be NULL. */
GBDE_API int gbde_mlp_train(gbde_ctx* ctx, const float* x, const float* y, int64_t n,
                   const gbde_mlp_train_opts* opts, float* net, float* loss_history);
/* Raw outputs y[n][3] (normalised log10 dt, stiff logit, normalised log2
 * steps) for x[n][8]; host memory. */
GBDE_API int gbde_mlp_forward(gbde_ctx* ctx, const float* net, const float* x, int64_t n,
                     float* y);
/* Gradient of the mean training loss over (x, y) w.r.t. the GBDE_MLP_PARAMS
 * weights, and the loss; host memory. */
GBDE_API int gbde_mlp_grad(gbde_ctx* ctx, const float* net, const float* x, const float* y,
                  int64_t n, float* grad, float* loss);
/* Make `net` (host) the network that learned solves of `model` use. */
GBDE_API int gbde_mlp_load(gbde_ctx* ctx, int32_t model, const float* net);

/* ---- ensemble statistics on the device -----------------------------------
 * Replaces EnsembleSummary / EnsembleAnalysis (timepoint_meanvar,
 * timepoint_quantile; qa.jl:54,211): per save point and state component,
 * across the N trajectories of u[N][n_save][n_state] (a solve's output),
 *   mean, variance (N - 1 in the denominator; NaN for N = 1) and the
 *   quantiles q_j by linear interpolation between order statistics
 *   ((N-1) q_j, the default of Julia's Statistics.quantile and numpy).
 * A column holding a NaN (the unreached save slots of a failed trajectory)
 * gives NaN statistics.  Quantiles are exact (radix selection on the
 * values' bits).  mem = GBDE_MEM_DEVICE: u and the outputs are device memory
 * of the context's device, and the kernels run on its stream;
 * GBDE_MEM_HOST: host memory, staged by the call.  Outputs may be NULL. */
#define GBDE_SUMMARY_MAX_Q 8
typedef struct {
  int32_t n_quantiles;                     /* 0 .. GBDE_SUMMARY_MAX_Q     */
  double quantiles[GBDE_SUMMARY_MAX_Q];    /* each in [0, 1]              */
  double* mean;                            /* [n_save][n_state] or NULL   */
  double* var;                             /* [n_save][n_state] or NULL   */
  double* qvals;                           /* [n_quantiles][n_save][n_state] or NULL */
} gbde_summary;
GBDE_API int gbde_ensemble_summary(gbde_ctx* ctx, const void* u, int32_t u_dtype, int32_t mem,
                                   int64_t n_traj, int32_t n_save, int32_t n_state,
                                   gbde_summary* out);

/* ---- user right-hand sides, compiled at run time ------------------------
 * Replaces passing a Julia function to ODEFunction (ODEFunction, qa.jl:84;
 * the problem's f!(du, u, p, t), test/core.jl:22-31,39-46).  f_body is the body
 * of a CUDA C++ function template
 *     template <class T> void f(T* du, const T* u, const T* p)
 * that fills du[0..n_state) from u and the parameters p (autonomous: a
 * time-dependent system carries t as an extra state with dt/dt = 1).  T is
 * double, float (GBDE_PREC_MIXED) or the FP32-pair type (GBDE_PREC_F32X2,
 * which has +, - and * only).  jac_body, if not NULL, is the body of
 *     template <class T> void jac(T (*J)[n_state], const T* u, const T* p)
 * filling J[r][c] = d du_r / d u_c; if NULL, Rosenbrock methods take the
 * Jacobian from forward-mode dual numbers over f_body (the reference's
 * AutoForwardDiff default, qa.jl:12), which also needs T(x) constructions and
 * the operators +, -, *, / and exp, log, sqrt, sin, cos, tanh, fabs, pow.
 * The first solve (or gbde_model_compile) of a model with an algorithm and a
 * precision compiles the library's step kernels around f with NVRTC for
 * sm_103a (seconds); later solves reuse the cached cubin.  User models run
 * Tsit5, Vern7, Rosenbrock23, Rodas5 and Rodas5P, one thread per trajectory,
 * in every batching mode; models registered with a noise term
 * (gbde_sde_model_register) also run EM, SOSRI and SRIW1 in FP64 or mixed
 * precision; not GBDE_ALG_AUTO or learned=1.                               */
typedef struct {
  const char* name;     /* label used in compile messages (may be NULL)    */
  int32_t n_state;      /* 1 .. GBDE_USER_MAX_STATE                        */
  int32_t n_param;      /* 1 .. GBDE_USER_MAX_PARAM                        */
  const char* f_body;   /* CUDA C++ statements: du[i] = ... (required)     */
  const char* jac_body; /* CUDA C++ statements: J[r][c] = ..., or NULL     */
} gbde_user_model;

/* Register a user model; *model_id receives its id (>= GBDE_MODEL_USER_BASE).
 * Source is copied; nothing is compiled yet.  Process-wide, thread-safe. */
GBDE_API int gbde_model_register(const gbde_user_model* def, int32_t* model_id);
/* Register a user SDE model (replaces SDEFunction(f, g), qa.jl:102, with
 * diagonal noise): def as for gbde_model_register (f is the drift), and
 * g_body the body of
 *     template <class T> void g(T* g, const T* u, const T* p)
 * filling g[0..n_state), the diagonal noise: du_i = f_i dt + g_i dW_i.  The
 * SDE methods draw the same counter-based normal stream as for built-in models
 * (gbde_philox_normals regenerates it).  The id also runs the ODE methods on f. */
GBDE_API int gbde_sde_model_register(const gbde_user_model* def, const char* g_body,
                                     int32_t* model_id);
/* Compile (and cache) a user model's kernels for one algorithm and precision
 * without a GPU; GBDE_ERR_INVALID with NVRTC's log in gbde_last_error(NULL)
 * when the source does not compile, GBDE_ERR_UNSUPPORTED without NVRTC. */
GBDE_API int gbde_model_compile(int32_t model_id, int32_t alg, int32_t precision);

/* ---- callbacks ----------------------------------------------------------
 * Replace ContinuousCallback / DiscreteCallback / VectorContinuousCallback /
 * CallbackSet (qa.jl:24,36,124,26; the reference's own tests solve with the
 * first two, test/core.jl:60-79).  condition is CUDA C++ statements that set
 * `double g` from `const double* u` (the state), `double t` and `const
 * double* p` (GBDE_CB_VECTOR: that set `out[0..len-1]`, `double* out`);
 * affect (may be NULL) modifies `double* u` and may set `bool terminate`
 * (GBDE_CB_VECTOR: `int idx` in [0, len) names the condition that fired).
 *   GBDE_CB_CONTINUOUS / GBDE_CB_VECTOR: a sign change of a condition over an
 *     accepted step is located on the method's dense output (Illinois regula
 *     falsi to ~1 ulp of t); of several, the earliest root (the first
 *     condition on a tie) is the event.  The trajectory moves to the left
 *     side of the root (LeftRootFind), applies that affect and restarts the
 *     method there.  Save points up to the event use the step's dense output;
 *     the next step ignores crossings in its first 1% (repeat_nudge), so a
 *     root is found once.
 *   GBDE_CB_DISCRETE: g != 0 after an accepted step (or an event) applies
 *     affect.
 * A set (gbde_callback_set_register) holds earlier ids, sets included, in
 * order: its continuous conditions compete for the earliest root; after each
 * accepted step or event its discrete callbacks run in order.
 * terminate ends the trajectory with GBDE_RET_TERMINATED (later save slots
 * hold NaN; t_end is the event time).  A solve with opts.callback compiles
 * its kernels at run time (NVRTC, as user models), for built-in one-thread
 * models and user models; not GBDE_ALG_AUTO, SDE methods or learned=1.
 * save_positions (the reference's keyword of every callback kind, default
 * (true, true): GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER) adds saves at the
 * callback's events to gbde_outputs.ev_*, beside the saveat points:
 *   GBDE_SAVE_BEFORE: (t, u) before the affect, unless a saveat point at
 *     exactly t was stored at that moment (the first discrete callback to
 *     fire after a step that ends on a saveat time, or an event on one);
 *   GBDE_SAVE_AFTER: (t, u) after the affect (continuous callbacks only
 *     when they have an affect, as the reference saves only a modified u).
 * At one time, saveat points come first, then the event saves in the order
 * made: the continuous event's, then each discrete callback's that fired. */
#define GBDE_SAVE_BEFORE 1
#define GBDE_SAVE_AFTER 2
typedef struct {
  int32_t kind;          /* GBDE_CB_CONTINUOUS, GBDE_CB_DISCRETE, _VECTOR  */
  const char* condition; /* statements: g = ...   (required)               */
  const char* affect;    /* statements on u[] / terminate, or NULL         */
  int32_t terminate;     /* 1: terminate after affect at every event       */
  int32_t save_positions;/* GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER bits (0: no
                            event saves; the reference's default is both) */
} gbde_callback;
/* Register a callback; *callback_id (>= 1) goes into gbde_opts.callback. */
GBDE_API int gbde_callback_register(const gbde_callback* def, int32_t* callback_id);
/* Register a VectorContinuousCallback of len conditions (def->kind ==
 * GBDE_CB_VECTOR, 1 <= len <= GBDE_MAX_CB_CONDITIONS). */
GBDE_API int gbde_vector_callback_register(const gbde_callback* def, int32_t len,
                                           int32_t* callback_id);
/* Register a CallbackSet of n earlier callback ids (leaves or sets); a solve
 * with it carries at most GBDE_MAX_CB_CONDITIONS continuous conditions. */
GBDE_API int gbde_callback_set_register(const int32_t* ids, int32_t n, int32_t* set_id);
/* Compile (and cache) the kernels of a model with a callback for one
 * algorithm and precision, without a GPU; errors as gbde_model_compile. */
GBDE_API int gbde_callback_compile(int32_t model, int32_t alg, int32_t precision,
                                   int32_t callback_id);

/* Self-check (no counterpart in the reference): the largest relative
 * difference, over n pseudo-random x with |x| in [2^-60, 2^61), between the
 * Newton-refined reciprocal the kernels use and the IEEE division 1/x on the
 * device (one Newton step: about 2^-40). */
GBDE_API int gbde_check_rcp64(gbde_ctx* ctx, int64_t n, double* max_rel_err);

#ifdef __cplusplus
}
#endif
#endif /* GBDE_H */
