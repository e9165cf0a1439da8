// capi.cu -- the extern "C" boundary (include/gbde.h): context, argument
// validation, device buffers, host<->device staging, launch dispatch.
//
// gbde_ensemble_solve() stands in for
//   SciMLBase.__solve(::EnsembleProblem, alg, ::EnsembleThreads; trajectories, ...)
// (EnsembleProblem qa.jl:50, EnsembleThreads qa.jl:56, solve qa.jl:192):
// one call solves every trajectory and fills the solution arrays.
#include <chrono>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbde.h"
#include "launch.h"
#include "philox.h"

using namespace gbde;

namespace {

thread_local std::string g_thread_err;

struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

// Device scratch of one ensemble solve: [0] queue counter, [1] status word,
// [2] second queue (AUTO), [3] AUTO list sizes; the persistent order; the
// AUTO lists; the learned predictions.  A context keeps one set for its
// solves; a captured graph keeps its own.
struct Scratch {
  DevBuf work, order, part, pred_dt, pred_stiff, pred_cost, dt_init;
  void release() {
    for (DevBuf* b : {&work, &order, &part, &pred_dt, &pred_stiff, &pred_cost, &dt_init})
      b->release();
  }
};

}  // namespace

struct gbde_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;       // GBDE_ALG_AUTO's second partition
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_join = nullptr;    // aux -> stream
  std::mutex mu;
  std::string err;
  // staging for GBDE_MEM_HOST calls
  DevBuf p, u0, t0, tf, saveat, u, ret, nacc, nrej, nf, tend, method;
  Scratch scratch;    // device scratch of ensemble solves (queue, order, lists, predictions)
  DevBuf dt1;         // staging of the first-accepted-step log (host calls)
  DevBuf mlp_net;     // learned predictor (GBDE_MLP_NET_FLOATS floats)
  DevBuf summary, summary_io;  // gbde_ensemble_summary: scratch; staged outputs (host mode)
  DevBuf red;         // staged in-kernel reduction (host mode)
  DevBuf evt, evu, evn;  // staged event saves (host mode)
  int mlp_model = 0;  // model the loaded predictor belongs to (0 = none)
};

static int set_err(gbde_ctx* ctx, int code, const char* fmt, ...) {
  char buf[4096];  // room for a user model's compile log
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  else g_thread_err = buf;
  return code;
}

#define GBDE_CUDA(ctx, call)                                                               \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return set_err(ctx, e_ == cudaErrorMemoryAllocation ? GBDE_ERR_NOMEM : GBDE_ERR_CUDA, \
                     "%s failed: %s", #call, cudaGetErrorString(e_));                      \
  } while (0)

namespace gbde {
// Records the calling thread's context-less error (gbde_last_error(NULL)) for
// entry points that take no context.
int set_thread_error(int code, const char* msg) {
  g_thread_err = msg;
  return code;
}

// One algorithm over a (sub)ensemble: team kernels for the 16-state ring,
// one thread per trajectory otherwise.
cudaError_t launch_alg(int alg, LaunchCfg cfg, const KArgs& a, cudaStream_t s) {
  cfg.alg = alg;
  if (cfg.model >= GBDE_MODEL_USER_BASE || cfg.callback) return launch_rtc(cfg, a, s);
  if (cfg.model == GBDE_MODEL_VDP_RING8 &&
      (alg == GBDE_ALG_RODAS5 || alg == GBDE_ALG_RODAS5P ||
       (alg == GBDE_ALG_TSIT5 && cfg.tpt != 1)))
    return launch_team(cfg, a, s);
  if (alg == GBDE_ALG_TSIT5 || alg == GBDE_ALG_VERN7) return launch_explicit(cfg, a, s);
  if (alg == GBDE_ALG_AUTOTSIT5_ROSENBROCK23 || alg == GBDE_ALG_AUTOTSIT5_RODAS5)
    return launch_autoswitch(cfg, a, s);
  if (alg == GBDE_ALG_EM || alg == GBDE_ALG_SOSRI || alg == GBDE_ALG_SRIW1)
    return launch_sde(cfg, a, s);
  return launch_rosenbrock(cfg, a, s);
}

int ctx_device(const gbde_ctx* ctx, int* device, int* num_sms, cudaStream_t* stream) {
  if (!ctx) return GBDE_ERR_INVALID;
  *device = ctx->device;
  *num_sms = ctx->num_sms;
  *stream = ctx->stream;
  return GBDE_OK;
}
}  // namespace gbde

extern "C" {

int gbde_version(void) { return GBDE_ABI_VERSION; }

const char* gbde_last_error(const gbde_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_thread_err.c_str();
}

int gbde_model_info(int32_t model, int32_t* n_state, int32_t* n_param) {
  int ns = 0, np = 0;
  switch (model) {
    case GBDE_MODEL_LINEAR: ns = Linear::N; np = Linear::NP; break;
    case GBDE_MODEL_LORENZ: ns = Lorenz::N; np = Lorenz::NP; break;
    case GBDE_MODEL_ROBERTSON: ns = Robertson::N; np = Robertson::NP; break;
    case GBDE_MODEL_VDP_RING8: ns = VdpRing8::N; np = VdpRing8::NP; break;
    case GBDE_MODEL_LOTKA_VOLTERRA: ns = LotkaVolterra::N; np = LotkaVolterra::NP; break;
    default:
      if (rtc_model_info(model, &ns, &np)) break;
      return set_err(nullptr, GBDE_ERR_INVALID, "unknown model id %d", model);
  }
  if (n_state) *n_state = ns;
  if (n_param) *n_param = np;
  return GBDE_OK;
}

int gbde_ctx_create(int device, gbde_ctx** out) {
  if (!out) return set_err(nullptr, GBDE_ERR_INVALID, "gbde_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_err(nullptr, GBDE_ERR_CUDA, "no CUDA device available (%s)",
                   cudaGetErrorString(e));
  if (device < 0 || device >= ndev)
    return set_err(nullptr, GBDE_ERR_INVALID, "device %d out of range [0,%d)", device, ndev);
  gbde_ctx* c = new gbde_ctx();
  c->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    int r = set_err(nullptr, GBDE_ERR_CUDA, "context setup failed: %s", cudaGetErrorString(e));
    delete c;
    return r;
  }
  c->stream = c->own;
  *out = c;
  return GBDE_OK;
}

int gbde_ctx_destroy(gbde_ctx* ctx) {
  if (!ctx) return GBDE_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->p, &ctx->u0, &ctx->t0, &ctx->tf, &ctx->saveat, &ctx->u, &ctx->ret,
                    &ctx->nacc, &ctx->nrej, &ctx->nf, &ctx->tend, &ctx->method, &ctx->dt1,
                    &ctx->mlp_net, &ctx->summary, &ctx->summary_io, &ctx->red, &ctx->evt,
                    &ctx->evu, &ctx->evn})
    b->release();
  ctx->scratch.release();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->aux) {
    cudaStreamSynchronize(ctx->aux);
    cudaStreamDestroy(ctx->aux);
  }
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
  return GBDE_OK;
}

int gbde_ctx_set_stream(gbde_ctx* ctx, void* stream) {
  if (!ctx) return set_err(nullptr, GBDE_ERR_INVALID, "ctx is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
  return GBDE_OK;
}

int gbde_opts_default(int32_t alg, gbde_opts* o) {
  if (!o) return set_err(nullptr, GBDE_ERR_INVALID, "gbde_opts_default: out is NULL");
  std::memset(o, 0, sizeof(*o));
  o->alg = alg;
  o->precision = GBDE_PREC_FP64;
  o->batching = GBDE_BATCH_PLAIN;
  o->adaptive = 1;
  o->reltol = 1e-3;
  o->abstol = 1e-6;
  o->dt = 0.0;
  o->dtmin = 0.0;
  o->dtmax = 0.0;
  o->maxiters = 100000;
  o->qmin = 0.2;
  o->qmax = 10.0;
  o->gamma = 0.9;
  o->qsteady_min = 1.0;
  o->qsteady_max = 1.0;
  o->qoldinit = 1e-4;
  o->seed = 0;
  o->stiff_threshold = 0.0;
  switch (alg) {
    case GBDE_ALG_TSIT5:  // Dormand-Prince style PI constants (HNW I, II.4)
      o->beta2 = 0.04;
      o->beta1 = 0.2 - 0.75 * 0.04;
      break;
    case GBDE_ALG_VERN7:
      o->beta2 = 2.0 / (5.0 * 7.0);
      o->beta1 = 7.0 / (10.0 * 7.0);
      break;
    case GBDE_ALG_ROSENBROCK23:  // error ~ h^3: I-controller
      o->beta1 = 1.0 / 3.0;
      o->beta2 = 0.0;
      break;
    case GBDE_ALG_RODAS5:
    case GBDE_ALG_RODAS5P:  // embedded order 4: error ~ h^5
      o->beta1 = 1.0 / 5.0;
      o->beta2 = 0.0;
      break;
    case GBDE_ALG_EM:
      o->adaptive = 0;
      o->beta1 = 0.5;
      break;
    case GBDE_ALG_SOSRI:  // strong order 1.5 pairs: error ~ h^2 (I-controller)
    case GBDE_ALG_SRIW1:
      o->beta1 = 1.0 / 2.0;
      o->beta2 = 0.0;
      o->reltol = 1e-2;
      o->abstol = 1e-2;
      break;
    case GBDE_ALG_AUTO:  // Tsit5's PI constants for both methods
      o->beta2 = 0.04;
      o->beta1 = 0.2 - 0.75 * 0.04;
      o->stiff_threshold = 30.0;
      break;
    case GBDE_ALG_AUTOTSIT5_ROSENBROCK23:  // Tsit5's; the stiff method's own defaults
    case GBDE_ALG_AUTOTSIT5_RODAS5:        // are taken when it steps
      o->beta2 = 0.04;
      o->beta1 = 0.2 - 0.75 * 0.04;
      break;
    default:
      return set_err(nullptr, GBDE_ERR_INVALID, "unknown algorithm id %d", alg);
  }
  return GBDE_OK;
}

// The device address of a page-locked host buffer mapped into the device's
// address space (cudaHostAlloc / cudaHostRegister memory, e.g. torch's
// pinned tensors), or nullptr for any other pointer (pageable memory is
// staged and copied).
static void* mapped_host(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // a pointer the runtime does not know: not mapped
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

static bool is_switch_alg(int a) {
  return a == GBDE_ALG_AUTOTSIT5_ROSENBROCK23 || a == GBDE_ALG_AUTOTSIT5_RODAS5;
}
static bool is_ode_alg(int a) {
  return a == GBDE_ALG_TSIT5 || a == GBDE_ALG_VERN7 || a == GBDE_ALG_ROSENBROCK23 ||
         a == GBDE_ALG_RODAS5 || a == GBDE_ALG_RODAS5P || a == GBDE_ALG_AUTO || is_switch_alg(a);
}
// the stiff method of a switching composite
static int switch_stiff_alg(int a) {
  return a == GBDE_ALG_AUTOTSIT5_RODAS5 ? GBDE_ALG_RODAS5 : GBDE_ALG_ROSENBROCK23;
}
static bool is_sde_alg(int a) {
  return a == GBDE_ALG_EM || a == GBDE_ALG_SOSRI || a == GBDE_ALG_SRIW1;
}

// GBDE_ALG_AUTO: classify every trajectory (stiff iff p[0] > stiff_threshold,
// or the learned predictor's label), then run the non-stiff list with Tsit5
// in the requested precision and the stiff list with Rodas5: FP64 when FP64
// is requested, otherwise FP32-pair stages and solves on an FP64 Jacobian,
// LU and norm (Rodas needs more than FP32 stages for its tolerances).
// The options' controller exponents (Tsit5's by default) drive the Tsit5
// part; the Rodas5 part uses Rodas5's default exponents.
static int solve_auto(gbde_ctx* ctx, Scratch& sc, const LaunchCfg& cfg, const KArgs& a, int np,
                      const gbde_opts* opts, cudaStream_t s) {
  const int64_t N = a.N;
  if (N == 0) return GBDE_OK;
  unsigned long long* work = (unsigned long long*)sc.work.ptr;
  unsigned* counters = reinterpret_cast<unsigned*>(work + 3);
  int32_t *nonstiff = nullptr, *stiff = nullptr;
  const int8_t* pred =
      (opts->learned & (GBDE_LEARN_START | GBDE_LEARN_STIFF)) ? (const int8_t*)sc.pred_stiff.ptr
                                                               : nullptr;
  GBDE_CUDA(ctx, build_partition(a.p, np, opts->stiff_threshold, pred, N, sc.part.ptr,
                                 counters, ctx->num_sms, s, &nonstiff, &stiff));
  unsigned cnt[2] = {0, 0};
  GBDE_CUDA(ctx, cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  GBDE_CUDA(ctx, cudaStreamSynchronize(s));
  // The stiff list first on the solve's stream, the non-stiff one on the
  // auxiliary stream: its CTAs take the SMs the first kernel's tail leaves
  // idle (each kernel alone fills the GPU).  The solve's stream then waits for
  // both.  (Every earlier piece of work on the stream has completed: the
  // list sizes were read back above.)
  const bool two = cnt[0] > 0 && cnt[1] > 0 && ctx->aux != nullptr;
  const struct {
    int alg, precision;
    unsigned n;
    const int32_t* list;
    unsigned long long* queue;
    cudaStream_t st;
  } parts[2] = {{GBDE_ALG_RODAS5, cfg.precision == GBDE_PREC_FP64 ? GBDE_PREC_FP64 : GBDE_PREC_F32X2,
                 cnt[1], stiff, work + 2, s},
                {GBDE_ALG_TSIT5, cfg.precision, cnt[0], nonstiff, work, two ? ctx->aux : s}};
  for (const auto& part : parts) {
    if (part.n == 0) continue;
    KArgs b = a;
    b.N = part.n;
    b.order = part.list;
    b.queue = cfg.persistent ? part.queue : nullptr;
    if (part.alg == GBDE_ALG_RODAS5) {
      // the stiff part runs with Rodas5's own controller exponents
      gbde_opts r;
      gbde_opts_default(GBDE_ALG_RODAS5, &r);
      b.ctl = ctl_consts(r.beta1, r.beta2, opts->gamma, opts->qmin, opts->qmax,
                         opts->qsteady_min, opts->qsteady_max, opts->qoldinit);
    }
    LaunchCfg c = cfg;
    c.precision = part.precision;
    const cudaError_t e = launch_alg(part.alg, c, b, part.st);
    if (e == cudaErrorNotSupported)
      return set_err(ctx, GBDE_ERR_UNSUPPORTED, "GBDE_ALG_AUTO is not built for model %d",
                     cfg.model);
    if (e != cudaSuccess)
      return set_err(ctx, GBDE_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  }
  if (two) {
    GBDE_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->aux));
    GBDE_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));
  }
  return GBDE_OK;
}

// Every argument check of an ensemble solve (shared by gbde_ensemble_solve,
// gbde_graph_create and gbde_autotune).
static int check_solve_args(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                            const gbde_outputs* out, int32_t* ns_out, int32_t* np_out) {
  if (!prob || !opts || !out)
    return set_err(ctx, GBDE_ERR_INVALID, "prob, opts and out must be non-NULL");
  int32_t ns = 0, np = 0;
  if (gbde_model_info(prob->model, &ns, &np) != GBDE_OK)
    return set_err(ctx, GBDE_ERR_INVALID, "unknown model id %d", prob->model);
  if (prob->n_state != ns || prob->n_param != np)
    return set_err(ctx, GBDE_ERR_INVALID,
                   "model %d has n_state=%d n_param=%d; got n_state=%d n_param=%d", prob->model,
                   ns, np, prob->n_state, prob->n_param);
  const int64_t N = prob->n_traj;
  if (N < 0) return set_err(ctx, GBDE_ERR_INVALID, "n_traj must be >= 0 (got %lld)", (long long)N);
  if (prob->mem != GBDE_MEM_HOST && prob->mem != GBDE_MEM_DEVICE)
    return set_err(ctx, GBDE_ERR_INVALID, "mem must be GBDE_MEM_HOST or GBDE_MEM_DEVICE");
  if (prob->save_kind != GBDE_SAVE_GRID && prob->save_kind != GBDE_SAVE_PER_TRAJ)
    return set_err(ctx, GBDE_ERR_INVALID, "unknown save_kind %d", prob->save_kind);
  if (prob->n_save < 0) return set_err(ctx, GBDE_ERR_INVALID, "n_save must be >= 0");
  if (N > 0 && (!prob->p || !prob->u0 || !prob->t0 || !prob->tf))
    return set_err(ctx, GBDE_ERR_INVALID, "p, u0, t0 and tf must be non-NULL");
  if (prob->n_save > 0 && !prob->saveat)
    return set_err(ctx, GBDE_ERR_INVALID, "saveat must be non-NULL when n_save > 0");
  if (N > 0 && (!out->retcode || (prob->n_save > 0 && !out->u && !out->reduce)))
    return set_err(ctx, GBDE_ERR_INVALID,
                   "out->retcode must be non-NULL, and out->u or out->reduce");
  if (out->u_dtype != GBDE_F64 && out->u_dtype != GBDE_F32)
    return set_err(ctx, GBDE_ERR_INVALID, "u_dtype must be GBDE_F64 or GBDE_F32");
  if (opts->callback != 0 && out->ev_count && out->ev_capacity < 0)
    return set_err(ctx, GBDE_ERR_INVALID, "ev_capacity must be >= 0");
  const int alg = opts->alg;
  if (!is_ode_alg(alg) && !is_sde_alg(alg))
    return set_err(ctx, GBDE_ERR_INVALID, "unknown algorithm id %d", alg);
  if (is_sde_alg(alg) && prob->model != GBDE_MODEL_LOTKA_VOLTERRA &&
      !(prob->model >= GBDE_MODEL_USER_BASE && rtc_model_has_noise(prob->model)))
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "SDE algorithms need a model with a noise term (the built-in Lotka-Volterra "
                   "model, or a user model from gbde_sde_model_register)");
  if (opts->precision != GBDE_PREC_FP64 && opts->precision != GBDE_PREC_MIXED &&
      opts->precision != GBDE_PREC_F32X2)
    return set_err(ctx, GBDE_ERR_INVALID, "unknown precision %d", opts->precision);
  if (opts->precision == GBDE_PREC_F32X2 &&
      (is_sde_alg(alg) ||
       (prob->model == GBDE_MODEL_VDP_RING8 && opts->threads_per_traj == 1)))
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "GBDE_PREC_F32X2 is built for the ODE kernels: one thread per trajectory, "
                   "or 16-lane teams on the 16-state ring");
  if (opts->batching != GBDE_BATCH_PLAIN && opts->batching != GBDE_BATCH_PERSISTENT)
    return set_err(ctx, GBDE_ERR_INVALID, "unknown batching %d", opts->batching);
  if (opts->adaptive && !(opts->reltol > 0.0 && opts->abstol > 0.0))
    return set_err(ctx, GBDE_ERR_INVALID, "adaptive stepping needs reltol > 0 and abstol > 0");
  if (!opts->adaptive && !(opts->dt > 0.0))
    return set_err(ctx, GBDE_ERR_INVALID, "fixed-step solving needs dt > 0");
  if (opts->maxiters <= 0) return set_err(ctx, GBDE_ERR_INVALID, "maxiters must be > 0");
  if (opts->adaptive && !(opts->qmin > 0.0 && opts->qmax >= 1.0 && opts->gamma > 0.0))
    return set_err(ctx, GBDE_ERR_INVALID, "controller needs qmin > 0, qmax >= 1, gamma > 0");
  if (opts->learned & ~(GBDE_LEARN_START | GBDE_LEARN_ORDER | GBDE_LEARN_STIFF))
    return set_err(ctx, GBDE_ERR_INVALID, "unknown learned flags %d", opts->learned);
  if (opts->learned && ctx->mlp_model != prob->model)
    return set_err(ctx, GBDE_ERR_STATE,
                   "learned=%d needs a predictor for model %d (gbde_mlp_load)", opts->learned,
                   prob->model);
  if (alg == GBDE_ALG_ROSENBROCK23 && prob->model == GBDE_MODEL_VDP_RING8)
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "Rosenbrock23 is built for n_state <= 3 (use Rodas5 / Rodas5P for the ring)");
  if (alg == GBDE_ALG_AUTO && N > INT32_MAX)
    return set_err(ctx, GBDE_ERR_INVALID, "GBDE_ALG_AUTO supports n_traj < 2^31");

  if (opts->threads_per_traj != 0 && opts->threads_per_traj != 1 && opts->threads_per_traj != 16)
    return set_err(ctx, GBDE_ERR_INVALID, "threads_per_traj must be 0, 1 or 16");
  if (opts->threads_per_traj == 16 && prob->model != GBDE_MODEL_VDP_RING8)
    return set_err(ctx, GBDE_ERR_UNSUPPORTED, "16-lane teams are built for the 16-state ring");
  if (opts->threads_per_traj == 1 && prob->model == GBDE_MODEL_VDP_RING8 &&
      alg != GBDE_ALG_TSIT5 && alg != GBDE_ALG_VERN7)
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "Rosenbrock methods on the 16-state ring run as 16-lane teams only");
  if (opts->chunk < 0) return set_err(ctx, GBDE_ERR_INVALID, "chunk must be >= 0");
  if (prob->model >= GBDE_MODEL_USER_BASE || opts->callback != 0) {
    // a user model or a callback: compile (once per model, algorithm,
    // precision and callback) and load the kernels now, before anything is
    // enqueued or captured
    if (alg == GBDE_ALG_AUTO || opts->learned || (is_sde_alg(alg) && opts->callback != 0) ||
        (is_switch_alg(alg) && opts->callback != 0))
      return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                     "user models run the one-thread ODE and SDE methods and callbacks the ODE "
                     "methods but the AutoTsit5 composites, without GBDE_ALG_AUTO and without "
                     "the learned predictor");
    if (prob->model == GBDE_MODEL_VDP_RING8)
      return set_err(ctx, GBDE_ERR_UNSUPPORTED, "callbacks are not built for the 16-lane ring");
    std::string why;
    GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
    const int rc = rtc_prepare(prob->model, alg, opts->precision, opts->callback, &why);
    if (rc != GBDE_OK) return set_err(ctx, rc, "%s", why.c_str());
  }
  if (is_switch_alg(alg) && (opts->precision == GBDE_PREC_F32X2 || opts->learned))
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "the AutoTsit5 composites run in FP64 or GBDE_PREC_MIXED, without the "
                   "learned predictor");
  if (is_switch_alg(alg) && prob->model == GBDE_MODEL_VDP_RING8)
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "the AutoTsit5 composites are built for one-thread models (n <= 3) and "
                   "user models; the 16-state ring has GBDE_ALG_AUTO");
  if (opts->block_size != 0 && (opts->block_size > 128 || opts->block_size < 32 ||
                                (opts->block_size & 31)))
    return set_err(ctx, GBDE_ERR_INVALID, "block_size must be a multiple of 32 and <= 128");
  *ns_out = ns;
  *np_out = np;
  return GBDE_OK;
}

// Scalar solver arguments.
static void fill_common(KArgs& a, const gbde_problem* prob, const gbde_opts* opts,
                        const gbde_outputs* out) {
  std::memset(&a, 0, sizeof(a));
  a.N = prob->n_traj;
  a.n_save = prob->n_save;
  a.save_kind = prob->save_kind;
  a.out_f32 = out->u_dtype == GBDE_F32;
  a.reltol = opts->reltol;
  a.abstol = opts->abstol;
  a.dt0 = opts->dt;
  a.dtmin = opts->dtmin;
  a.dtmax = opts->dtmax;
  a.maxiters = opts->maxiters;
  a.adaptive = opts->adaptive;
  a.qmin = opts->qmin;
  a.qmax = opts->qmax;
  a.gamma = opts->gamma;
  a.beta1 = opts->beta1;
  a.beta2 = opts->beta2;
  a.qsteady_min = opts->qsteady_min;
  a.qsteady_max = opts->qsteady_max;
  a.qoldinit = opts->qoldinit;
  a.seed = opts->seed;
  a.timeout_ns = opts->timeout_s > 0 ? (uint64_t)(opts->timeout_s * 1e9) : 0;
  a.ctl = ctl_consts(opts->beta1, opts->beta2, opts->gamma, opts->qmin, opts->qmax,
                     opts->qsteady_min, opts->qsteady_max, opts->qoldinit);
  a.ctl_stiff = a.ctl;
  if (is_switch_alg(opts->alg)) {  // the stiff method steps with its own exponents
    gbde_opts r;
    gbde_opts_default(switch_stiff_alg(opts->alg), &r);
    a.ctl_stiff = ctl_consts(r.beta1, r.beta2, opts->gamma, opts->qmin, opts->qmax,
                             opts->qsteady_min, opts->qsteady_max, opts->qoldinit);
  }
  a.chunk = opts->chunk > 0 ? opts->chunk : 1;
}

// the event-save outputs are in use (the kernels take them only with a callback)
static bool event_saves(const gbde_outputs* out) { return out->ev_count != nullptr; }

static void fill_device_ptrs(KArgs& a, const gbde_problem* prob, const gbde_outputs* out) {
  a.p = prob->p;
  a.u0 = prob->u0;
  a.t0 = prob->t0;
  a.tf = prob->tf;
  a.saveat = prob->saveat;
  a.u_out = out->u;
  a.retcode = out->retcode;
  a.naccept = out->naccept;
  a.nreject = out->nreject;
  a.nf = out->nf;
  a.t_end = out->t_end;
  a.method_out = out->method;
  a.dt_first = out->dt_first;
  a.red = out->reduce;
  if (event_saves(out)) {
    a.ev_t = out->ev_t;
    a.ev_u = out->ev_u;
    a.ev_n = out->ev_count;
    a.ev_cap = out->ev_capacity;
  }
}

static LaunchCfg make_cfg(const gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts) {
  LaunchCfg cfg;
  cfg.alg = opts->alg;
  cfg.model = prob->model;
  cfg.precision = opts->precision;
  cfg.persistent = opts->batching == GBDE_BATCH_PERSISTENT;
  cfg.block = opts->block_size > 0 ? opts->block_size : 128;
  cfg.grid = 0;
  cfg.ctas_per_sm = opts->ctas_per_sm;
  cfg.num_sms = ctx->num_sms;
  cfg.tpt = opts->threads_per_traj;
  cfg.callback = opts->callback;
  return cfg;
}

// Allocate every scratch buffer a solve of N trajectories with these options
// uses, before any work is enqueued (a stream capture must not meet a
// cudaMalloc).
// Adaptive one-thread-per-trajectory ODE solves start from the Hairer-Wanner
// step computed by a converged pre-pass kernel (k_init_dt) instead of inside
// the step kernel, where each refill would run it for one lane of a warp.
static bool uses_dt_prepass(const gbde_opts* o, int model) {
  const int a = o->alg;
  const bool ode = a == GBDE_ALG_TSIT5 || a == GBDE_ALG_VERN7 || a == GBDE_ALG_ROSENBROCK23 ||
                   a == GBDE_ALG_RODAS5 || a == GBDE_ALG_RODAS5P || is_switch_alg(a);
  const bool team = model == GBDE_MODEL_VDP_RING8 &&
                    (a == GBDE_ALG_RODAS5 || a == GBDE_ALG_RODAS5P ||
                     (a == GBDE_ALG_TSIT5 && o->threads_per_traj != 1));
  return ode && !team && o->adaptive && !(o->dt > 0.0) && !(o->learned & GBDE_LEARN_START);
}

static int reserve_scratch(gbde_ctx* ctx, Scratch& sc, int64_t N, const gbde_opts* opts,
                           int model) {
  GBDE_CUDA(ctx, sc.work.ensure(256));
  if (opts->learned && N > 0) {
    GBDE_CUDA(ctx, sc.pred_dt.ensure((size_t)N * sizeof(float)));
    GBDE_CUDA(ctx, sc.pred_stiff.ensure((size_t)N));
    GBDE_CUDA(ctx, sc.pred_cost.ensure((size_t)N * sizeof(float)));
  }
  if (opts->alg == GBDE_ALG_AUTO && N > 0)
    GBDE_CUDA(ctx, sc.part.ensure(partition_scratch_bytes(N)));
  else if (opts->batching == GBDE_BATCH_PERSISTENT && N > 1 && N <= INT32_MAX)
    GBDE_CUDA(ctx, sc.order.ensure(span_order_scratch_bytes(N)));
  if (uses_dt_prepass(opts, model) && N > 0)
    GBDE_CUDA(ctx, sc.dt_init.ensure((size_t)N * sizeof(double)));
  return GBDE_OK;
}

// Enqueue the device work of one solve on stream s: clear the queue and status
// words, learned predictions, queue order (or AUTO's lists), the step kernels.
// No host synchronisation except GBDE_ALG_AUTO's list sizes.
static int enqueue_solve(gbde_ctx* ctx, Scratch& sc, KArgs& a, const LaunchCfg& cfg,
                         const gbde_opts* opts, int np, int ns, cudaStream_t s) {
  const int64_t N = a.N;
  const int alg = opts->alg;
  unsigned long long* work = (unsigned long long*)sc.work.ptr;
  GBDE_CUDA(ctx, cudaMemsetAsync(work, 0, 256, s));
  if (a.red && a.n_save > 0)  // the in-kernel reduction starts from zero sums
    GBDE_CUDA(ctx, cudaMemsetAsync(a.red, 0, 2 * (size_t)a.n_save * ns * sizeof(double), s));
  a.queue = cfg.persistent ? work : nullptr;
  a.flag = (int32_t*)(work + 1);
  if (opts->learned && N > 0) {
    // learned predictions: first dt (all methods), stiff label (AUTO) and
    // cost (queue order)
    GBDE_CUDA(ctx, mlp_predict(cfg.model, (const float*)ctx->mlp_net.ptr, a,
                               (float*)sc.pred_dt.ptr, (int8_t*)sc.pred_stiff.ptr,
                               (float*)sc.pred_cost.ptr, ctx->num_sms, s));
    if (opts->learned & GBDE_LEARN_START) a.pred_dt = (const float*)sc.pred_dt.ptr;
  }
  if (alg == GBDE_ALG_AUTO) return solve_auto(ctx, sc, cfg, a, np, opts, s);
  if (cfg.persistent && N > 1 && N <= INT32_MAX) {
    // queue order (order.cu): highest learned cost first, else longest span
    // first
    const int32_t* ord = nullptr;
    if (opts->learned & GBDE_LEARN_ORDER)
      GBDE_CUDA(ctx, build_cost_order((const float*)sc.pred_cost.ptr, N, sc.order.ptr,
                                      ctx->num_sms, s, &ord));
    else
      GBDE_CUDA(ctx, build_span_order(a.t0, a.tf, N, sc.order.ptr, ctx->num_sms, s, &ord));
    a.order = ord;
  }
  if (N > 0) {
    LaunchCfg c = cfg;
    if (uses_dt_prepass(opts, cfg.model)) c.dt_init = (double*)sc.dt_init.ptr;
    const cudaError_t e = launch_alg(alg, c, a, s);
    if (e == cudaErrorNotSupported)
      return set_err(ctx, GBDE_ERR_UNSUPPORTED, "algorithm %d is not built for model %d", alg,
                     cfg.model);
    if (e != cudaSuccess)
      return set_err(ctx, GBDE_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  }
  return GBDE_OK;
}

int gbde_ensemble_solve(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                        gbde_outputs* out) {
  if (!ctx) return set_err(nullptr, GBDE_ERR_INVALID, "ctx is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  const auto wall0 = std::chrono::steady_clock::now();
  int32_t ns = 0, np = 0;
  const int rc0 = check_solve_args(ctx, prob, opts, out, &ns, &np);
  if (rc0 != GBDE_OK) return rc0;
  const int64_t N = prob->n_traj;
  GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const size_t n_save = (size_t)prob->n_save;
  const size_t esz = out->u_dtype == GBDE_F32 ? 4 : 8;
  const size_t save_elems = prob->save_kind == GBDE_SAVE_GRID ? n_save : n_save * (size_t)N;
  const size_t u_bytes = (size_t)N * n_save * (size_t)ns * esz;

  KArgs a;
  fill_common(a, prob, opts, out);
  const bool host = prob->mem == GBDE_MEM_HOST;
  const bool ev = opts->callback != 0 && event_saves(out);
  void* u_direct = nullptr;
  if (host) {
    GBDE_CUDA(ctx, ctx->p.ensure((size_t)N * np * 8));
    GBDE_CUDA(ctx, ctx->u0.ensure((size_t)N * ns * 8));
    GBDE_CUDA(ctx, ctx->t0.ensure((size_t)N * 8));
    GBDE_CUDA(ctx, ctx->tf.ensure((size_t)N * 8));
    GBDE_CUDA(ctx, ctx->saveat.ensure(save_elems * 8));
    // saves straight into a page-locked, mapped output buffer: the kernels
    // store them over the host link while they run (GB300's coherent C2C;
    // ~2 GB/s of stores spread over the solve instead of a 1 GB copy after it)
    u_direct = out->u ? mapped_host(out->u) : nullptr;
    if (out->u && !u_direct) GBDE_CUDA(ctx, ctx->u.ensure(u_bytes));
    GBDE_CUDA(ctx, ctx->ret.ensure((size_t)N * 4));
    if (N > 0) {
      GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->p.ptr, prob->p, (size_t)N * np * 8, cudaMemcpyHostToDevice, s));
      GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->u0.ptr, prob->u0, (size_t)N * ns * 8, cudaMemcpyHostToDevice, s));
      GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->t0.ptr, prob->t0, (size_t)N * 8, cudaMemcpyHostToDevice, s));
      GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->tf.ptr, prob->tf, (size_t)N * 8, cudaMemcpyHostToDevice, s));
    }
    if (save_elems > 0)
      GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->saveat.ptr, prob->saveat, save_elems * 8, cudaMemcpyHostToDevice, s));
    a.p = (const double*)ctx->p.ptr;
    a.u0 = (const double*)ctx->u0.ptr;
    a.t0 = (const double*)ctx->t0.ptr;
    a.tf = (const double*)ctx->tf.ptr;
    a.saveat = (const double*)ctx->saveat.ptr;
    a.u_out = out->u ? (u_direct ? u_direct : ctx->u.ptr) : nullptr;
    a.retcode = (int32_t*)ctx->ret.ptr;
    if (out->reduce) {
      GBDE_CUDA(ctx, ctx->red.ensure(2 * n_save * (size_t)ns * 8));
      a.red = (double*)ctx->red.ptr;
    }
    if (out->naccept) { GBDE_CUDA(ctx, ctx->nacc.ensure((size_t)N * 4)); a.naccept = (int32_t*)ctx->nacc.ptr; }
    if (out->nreject) { GBDE_CUDA(ctx, ctx->nrej.ensure((size_t)N * 4)); a.nreject = (int32_t*)ctx->nrej.ptr; }
    if (out->nf) { GBDE_CUDA(ctx, ctx->nf.ensure((size_t)N * 4)); a.nf = (int32_t*)ctx->nf.ptr; }
    if (out->t_end) { GBDE_CUDA(ctx, ctx->tend.ensure((size_t)N * 8)); a.t_end = (double*)ctx->tend.ptr; }
    if (out->method) { GBDE_CUDA(ctx, ctx->method.ensure((size_t)N * 4)); a.method_out = (int32_t*)ctx->method.ptr; }
    if (out->dt_first) { GBDE_CUDA(ctx, ctx->dt1.ensure((size_t)N * 8)); a.dt_first = (double*)ctx->dt1.ptr; }
    if (ev) {
      const size_t slots = (size_t)N * (size_t)out->ev_capacity;
      GBDE_CUDA(ctx, ctx->evn.ensure((size_t)N * 4));
      a.ev_n = (int32_t*)ctx->evn.ptr;
      a.ev_cap = out->ev_capacity;
      if (out->ev_t && slots) { GBDE_CUDA(ctx, ctx->evt.ensure(slots * 8)); a.ev_t = (double*)ctx->evt.ptr; }
      if (out->ev_u && slots) { GBDE_CUDA(ctx, ctx->evu.ensure(slots * ns * esz)); a.ev_u = ctx->evu.ptr; }
    }
  } else {
    fill_device_ptrs(a, prob, out);
  }
  const LaunchCfg cfg = make_cfg(ctx, prob, opts);
  { const int rc = reserve_scratch(ctx, ctx->scratch, N, opts, prob->model); if (rc != GBDE_OK) return rc; }
  GBDE_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  { const int rc = enqueue_solve(ctx, ctx->scratch, a, cfg, opts, np, ns, s); if (rc != GBDE_OK) return rc; }
  GBDE_CUDA(ctx, cudaEventRecord(ctx->ev1, s));

  int32_t flag = 0;
  if (host) {
    if (u_bytes && out->u && !u_direct)
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->u, ctx->u.ptr, u_bytes, cudaMemcpyDeviceToHost, s));
    if (out->reduce && n_save)
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->reduce, a.red, 2 * n_save * (size_t)ns * 8,
                                     cudaMemcpyDeviceToHost, s));
    if (N > 0) {
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->retcode, ctx->ret.ptr, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
      if (out->naccept) GBDE_CUDA(ctx, cudaMemcpyAsync(out->naccept, a.naccept, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
      if (out->nreject) GBDE_CUDA(ctx, cudaMemcpyAsync(out->nreject, a.nreject, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
      if (out->nf) GBDE_CUDA(ctx, cudaMemcpyAsync(out->nf, a.nf, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
      if (out->t_end) GBDE_CUDA(ctx, cudaMemcpyAsync(out->t_end, a.t_end, (size_t)N * 8, cudaMemcpyDeviceToHost, s));
      if (out->method) GBDE_CUDA(ctx, cudaMemcpyAsync(out->method, a.method_out, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
      if (out->dt_first) GBDE_CUDA(ctx, cudaMemcpyAsync(out->dt_first, a.dt_first, (size_t)N * 8, cudaMemcpyDeviceToHost, s));
      if (ev) {
        const size_t slots = (size_t)N * (size_t)out->ev_capacity;
        GBDE_CUDA(ctx, cudaMemcpyAsync(out->ev_count, a.ev_n, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
        if (a.ev_t) GBDE_CUDA(ctx, cudaMemcpyAsync(out->ev_t, a.ev_t, slots * 8, cudaMemcpyDeviceToHost, s));
        if (a.ev_u) GBDE_CUDA(ctx, cudaMemcpyAsync(out->ev_u, a.ev_u, slots * ns * esz, cudaMemcpyDeviceToHost, s));
      }
    }
  }
  GBDE_CUDA(ctx, cudaMemcpyAsync(&flag, a.flag, 4, cudaMemcpyDeviceToHost, s));
  GBDE_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  GBDE_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  out->device_ms = ms;
  out->total_ms = (float)std::chrono::duration<double, std::milli>(
                      std::chrono::steady_clock::now() - wall0).count();
  if (flag & 1)
    return set_err(ctx, GBDE_ERR_TIMEOUT, "device deadline of %.3f s reached; unfinished "
                   "trajectories carry GBDE_RET_TIMEOUT", opts->timeout_s);
  return GBDE_OK;
}

// ---------------------------------------------------------- CUDA graphs
struct gbde_graph {
  gbde_ctx* ctx = nullptr;
  Scratch scratch;  // the graph's own scratch: later solves cannot move it
  cudaGraphExec_t exec = nullptr;
  double timeout_s = 0.0;
};

int gbde_graph_create(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                      gbde_outputs* out, gbde_graph** graph) {
  if (!ctx || !graph) return set_err(ctx, GBDE_ERR_INVALID, "ctx and graph must be non-NULL");
  *graph = nullptr;
  std::lock_guard<std::mutex> lk(ctx->mu);
  int32_t ns = 0, np = 0;
  const int rc0 = check_solve_args(ctx, prob, opts, out, &ns, &np);
  if (rc0 != GBDE_OK) return rc0;
  if (prob->mem != GBDE_MEM_DEVICE)
    return set_err(ctx, GBDE_ERR_INVALID, "a graph captures a device-memory problem (GBDE_MEM_DEVICE)");
  if (opts->alg == GBDE_ALG_AUTO)
    return set_err(ctx, GBDE_ERR_UNSUPPORTED,
                   "GBDE_ALG_AUTO sizes its launches on the host and cannot be captured");
  GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
  KArgs a;
  fill_common(a, prob, opts, out);
  fill_device_ptrs(a, prob, out);
  const LaunchCfg cfg = make_cfg(ctx, prob, opts);
  gbde_graph* G = new gbde_graph();
  G->ctx = ctx;
  G->timeout_s = opts->timeout_s;
  int rc = reserve_scratch(ctx, G->scratch, prob->n_traj, opts, prob->model);
  if (rc != GBDE_OK) {
    delete G;
    return rc;
  }
  cudaStream_t s = ctx->stream;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    rc = enqueue_solve(ctx, G->scratch, a, cfg, opts, np, ns, s);
    e = cudaStreamEndCapture(s, &g);
  }
  if (e == cudaSuccess && rc == GBDE_OK) e = cudaGraphInstantiate(&G->exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess || rc != GBDE_OK) {
    G->scratch.release();
    delete G;
    return rc != GBDE_OK ? rc : set_err(ctx, GBDE_ERR_CUDA, "graph capture failed: %s",
                                        cudaGetErrorString(e));
  }
  *graph = G;
  return GBDE_OK;
}

int gbde_graph_launch(gbde_graph* G, float* device_ms) {
  if (!G) return set_err(nullptr, GBDE_ERR_INVALID, "graph is NULL");
  gbde_ctx* ctx = G->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  int32_t flag = 0;
  GBDE_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  GBDE_CUDA(ctx, cudaGraphLaunch(G->exec, s));
  GBDE_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
  GBDE_CUDA(ctx, cudaMemcpyAsync(&flag, (unsigned long long*)G->scratch.work.ptr + 1, 4,
                                 cudaMemcpyDeviceToHost, s));
  GBDE_CUDA(ctx, cudaStreamSynchronize(s));
  if (device_ms) GBDE_CUDA(ctx, cudaEventElapsedTime(device_ms, ctx->ev0, ctx->ev1));
  if (flag & 1)
    return set_err(ctx, GBDE_ERR_TIMEOUT, "device deadline of %.3f s reached; unfinished "
                   "trajectories carry GBDE_RET_TIMEOUT", G->timeout_s);
  return GBDE_OK;
}

int gbde_graph_destroy(gbde_graph* G) {
  if (!G) return GBDE_OK;
  gbde_ctx* ctx = G->ctx;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (G->exec) cudaGraphExecDestroy(G->exec);
    G->scratch.release();
  }
  delete G;
  return GBDE_OK;
}

// ------------------------------------------------------------ autotuner
// Times the solve under each launch configuration (batching, block size,
// resident CTAs per SM, queue chunk, threads per trajectory) on the caller's
// own problem and returns the fastest in *best.  `out` receives the results
// of a final run with the best configuration.
int gbde_autotune(gbde_ctx* ctx, const gbde_problem* prob, const gbde_opts* opts,
                  gbde_outputs* out, int32_t reps, gbde_opts* best, gbde_tune_entry* table,
                  int32_t table_cap, int32_t* n_entries) {
  if (!ctx || !prob || !opts || !out || !best)
    return set_err(ctx, GBDE_ERR_INVALID, "ctx, prob, opts, out and best must be non-NULL");
  if (reps <= 0) reps = 2;
  std::vector<gbde_opts> cand;
  auto add = [&](int batching, int block, int cps, int chunk, int tpt) {
    gbde_opts o = *opts;
    o.batching = batching;
    o.block_size = block;
    o.ctas_per_sm = cps;
    o.chunk = chunk;
    o.threads_per_traj = tpt;
    cand.push_back(o);
  };
  std::vector<int> tpts = {opts->threads_per_traj};
  if (prob->model == GBDE_MODEL_VDP_RING8 && opts->alg == GBDE_ALG_TSIT5) tpts = {16, 1};
  for (int tpt : tpts) {
    for (int block : {64, 128}) add(GBDE_BATCH_PLAIN, block, 0, 0, tpt);
    for (int block : {64, 128})
      for (int cps : {0, 2, 4})
        for (int chunk : {1, 4}) add(GBDE_BATCH_PERSISTENT, block, cps, chunk, tpt);
  }
  float best_ms = 1e30f;
  int best_i = -1, count = 0;
  for (size_t k = 0; k < cand.size(); ++k) {
    float ms = 1e30f;
    for (int r = 0; r < reps; ++r) {
      const int rc = gbde_ensemble_solve(ctx, prob, &cand[k], out);
      if (rc != GBDE_OK) {
        ms = 1e30f;
        break;
      }
      ms = out->device_ms < ms ? out->device_ms : ms;
    }
    if (table && count < table_cap) {
      table[count] = {cand[k].batching, cand[k].block_size, cand[k].ctas_per_sm, cand[k].chunk,
                      cand[k].threads_per_traj, ms};
    }
    ++count;
    if (ms < best_ms) {
      best_ms = ms;
      best_i = (int)k;
    }
  }
  if (n_entries) *n_entries = count < table_cap ? count : table_cap;
  if (best_i < 0) return set_err(ctx, GBDE_ERR_INVALID, "no launch configuration ran");
  *best = cand[best_i];
  return gbde_ensemble_solve(ctx, prob, best, out);
}

int gbde_ensemble_summary(gbde_ctx* ctx, const void* u, int32_t u_dtype, int32_t mem,
                          int64_t n_traj, int32_t n_save, int32_t n_state, gbde_summary* out) {
  if (!ctx || !out) return set_err(ctx, GBDE_ERR_INVALID, "ctx and out must be non-NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n_traj < 1 || n_save < 1 || n_state < 1 || !u)
    return set_err(ctx, GBDE_ERR_INVALID, "need u, n_traj >= 1, n_save >= 1, n_state >= 1");
  if (u_dtype != GBDE_F64 && u_dtype != GBDE_F32)
    return set_err(ctx, GBDE_ERR_INVALID, "u_dtype must be GBDE_F64 or GBDE_F32");
  if (mem != GBDE_MEM_HOST && mem != GBDE_MEM_DEVICE)
    return set_err(ctx, GBDE_ERR_INVALID, "mem must be GBDE_MEM_HOST or GBDE_MEM_DEVICE");
  const int nq = out->n_quantiles;
  if (nq < 0 || nq > GBDE_SUMMARY_MAX_Q)
    return set_err(ctx, GBDE_ERR_INVALID, "n_quantiles must be in [0, %d]", GBDE_SUMMARY_MAX_Q);
  for (int j = 0; j < nq; ++j)
    if (!(out->quantiles[j] >= 0.0 && out->quantiles[j] <= 1.0))
      return set_err(ctx, GBDE_ERR_INVALID, "quantiles must lie in [0, 1]");
  const int64_t C64 = (int64_t)n_save * n_state;
  if (C64 > 65535) return set_err(ctx, GBDE_ERR_UNSUPPORTED, "n_save * n_state must be <= 65535");
  const int C = (int)C64;
  const int f32 = u_dtype == GBDE_F32;
  const size_t ubytes = (size_t)n_traj * C * (f32 ? 4 : 8);
  GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int qn = out->qvals ? nq : 0;
  GBDE_CUDA(ctx, ctx->summary.ensure(
                     summary_scratch_bytes(n_traj, C, f32, qn, summary_sum_blocks(C, ctx->num_sms))));
  const void* ud = u;
  double *mean = out->mean, *var = out->var, *qv = out->qvals;
  if (mem == GBDE_MEM_HOST) {
    GBDE_CUDA(ctx, ctx->u.ensure(ubytes));
    GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->u.ptr, u, ubytes, cudaMemcpyHostToDevice, s));
    ud = ctx->u.ptr;
    GBDE_CUDA(ctx, ctx->summary_io.ensure((size_t)C * (2 + nq) * sizeof(double)));
    double* io = (double*)ctx->summary_io.ptr;
    mean = out->mean ? io : nullptr;
    var = out->var ? io + C : nullptr;
    qv = out->qvals ? io + 2 * C : nullptr;
  }
  GBDE_CUDA(ctx, enqueue_summary(ud, f32, n_traj, C, qn, out->quantiles, mean, var, qv,
                                 ctx->summary.ptr, ctx->num_sms, s));
  if (mem == GBDE_MEM_HOST) {
    if (out->mean)
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->mean, mean, C * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (out->var)
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->var, var, C * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (out->qvals && nq)
      GBDE_CUDA(ctx, cudaMemcpyAsync(out->qvals, qv, (size_t)nq * C * sizeof(double),
                                     cudaMemcpyDeviceToHost, s));
  }
  GBDE_CUDA(ctx, cudaStreamSynchronize(s));
  return GBDE_OK;
}

int gbde_mlp_load(gbde_ctx* ctx, int32_t model, const float* net) {
  if (!ctx || !net) return set_err(nullptr, GBDE_ERR_INVALID, "ctx and net must be non-NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (gbde_model_info(model, nullptr, nullptr) != GBDE_OK)
    return set_err(ctx, GBDE_ERR_INVALID, "unknown model id %d", model);
  GBDE_CUDA(ctx, cudaSetDevice(ctx->device));
  GBDE_CUDA(ctx, ctx->mlp_net.ensure(sizeof(float) * GBDE_MLP_NET_FLOATS));
  GBDE_CUDA(ctx, cudaMemcpyAsync(ctx->mlp_net.ptr, net, sizeof(float) * GBDE_MLP_NET_FLOATS,
                                 cudaMemcpyHostToDevice, ctx->stream));
  GBDE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->mlp_model = model;
  return GBDE_OK;
}

int gbde_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  if (!ctr || !key || !out) return set_err(nullptr, GBDE_ERR_INVALID, "NULL argument");
  Philox4 r = philox4x32_10(Philox4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
  return GBDE_OK;
}

int gbde_philox_normals(uint64_t seed, uint64_t traj, uint64_t counter, int64_t n, double* out) {
  if (n < 0 || (n > 0 && !out)) return set_err(nullptr, GBDE_ERR_INVALID, "bad n or out");
  for (int64_t k = 0; k < n; ++k) out[k] = philox_normal_f64(seed, traj, counter + (uint64_t)k);
  return GBDE_OK;
}

}  // extern "C"
