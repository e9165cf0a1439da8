// noalloc.cu -- gbde_ensemble_solve_noalloc(): the ensemble solve for callers
// that cannot allocate device memory.
//
// Who needs it: a caller that already holds every input and output in device
// memory but may not call cudaMalloc.  Examples are a real-time loop in which
// cudaMalloc's implicit device-wide synchronisation is not acceptable, a
// process whose device memory belongs to one allocator (a framework's caching
// pool, the array pool of a garbage-collected host language) that must stay
// its only owner, and an embedding with a fixed device-memory budget.
// gbde_ensemble_solve() cannot serve them: its context cudaMallocs a small
// work buffer on first use and staging buffers for host-memory problems.
//
// The only device memory a solve needs beyond the caller's inputs and outputs
// is its scratch: the persistent work-queue counter and the status word that
// reports a device deadline.  Here they live in g_noalloc_scratch, a
// file-scope __device__ array of GBDE_NOALLOC_SCRATCH_BYTES that every GPU
// which loads libgbde.so holds until the process exits.  Nothing in this file
// calls cudaMalloc, cudaFree or any allocating library routine.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/gbde.h"
#include "launch.h"

namespace gbde {
int set_thread_error(int code, const char* msg);  // capi.cu
}  // namespace gbde

using namespace gbde;

namespace {

constexpr int kScratchWords = GBDE_NOALLOC_SCRATCH_BYTES / 8;
// Words of scratch a solve uses: [0] queue counter, [1] status word.  The need
// does not grow with the ensemble.
constexpr int kWordsUsed = 2;
static_assert(kWordsUsed <= kScratchWords, "scratch array too small for one solve");

// The shared scratch.  Host code must not pass this name to a kernel: on the
// host it is a stand-in symbol, not a device address.  The device address of
// each GPU's copy comes from cudaGetSymbolAddress() in device_setup().
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;

struct DeviceSetup {
  bool ready = false;
  unsigned long long* scratch = nullptr;  // device address of g_noalloc_scratch
  int num_sms = 0;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return set_thread_error(code, buf);
}

// Once per device, with that device current: the device address of the
// scratch array and the SM count.  Runs on the first call on each device.
int device_setup(int device, DeviceSetup* out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSetup& d = g_setup[device];
  if (!d.ready) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(GBDE_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed on device %d: %s",
                  device, cudaGetErrorString(e));
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess)
      return fail(GBDE_ERR_CUDA, "cudaDeviceGetAttribute failed on device %d: %s", device,
                  cudaGetErrorString(e));
    d.scratch = static_cast<unsigned long long*>(ptr);
    d.num_sms = sms;
    d.ready = true;
  }
  *out = d;
  return GBDE_OK;
}

bool is_switch(int a) {
  return a == GBDE_ALG_AUTOTSIT5_ROSENBROCK23 || a == GBDE_ALG_AUTOTSIT5_RODAS5;
}
bool is_ode(int a) {
  return a == GBDE_ALG_TSIT5 || a == GBDE_ALG_VERN7 || a == GBDE_ALG_ROSENBROCK23 ||
         a == GBDE_ALG_RODAS5 || a == GBDE_ALG_RODAS5P || is_switch(a);
}
bool is_sde(int a) { return a == GBDE_ALG_EM || a == GBDE_ALG_SOSRI || a == GBDE_ALG_SRIW1; }

#define NOALLOC_CUDA(call)                                                           \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(GBDE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
  } while (0)

}  // namespace

extern "C" int gbde_ensemble_solve_noalloc(const gbde_problem* prob, const gbde_opts* opts,
                                           gbde_outputs* out, void* stream) {
  const auto wall0 = std::chrono::steady_clock::now();
  if (!prob || !opts || !out) return fail(GBDE_ERR_INVALID, "prob, opts and out must be non-NULL");
  if (prob->mem != GBDE_MEM_DEVICE)
    return fail(GBDE_ERR_INVALID,
                "gbde_ensemble_solve_noalloc needs device pointers (mem = GBDE_MEM_DEVICE): "
                "staging host arrays would allocate device memory");
  int32_t ns = 0, np = 0;
  if (gbde_model_info(prob->model, &ns, &np) != GBDE_OK)
    return fail(GBDE_ERR_INVALID, "unknown model id %d", prob->model);
  if (prob->model >= GBDE_MODEL_USER_BASE)
    return fail(GBDE_ERR_UNSUPPORTED,
                "gbde_ensemble_solve_noalloc runs the built-in models only: a user model's "
                "kernels are compiled and loaded by gbde_ensemble_solve");
  if (prob->n_state != ns || prob->n_param != np)
    return fail(GBDE_ERR_INVALID, "model %d has n_state=%d n_param=%d; got n_state=%d n_param=%d",
                prob->model, ns, np, prob->n_state, prob->n_param);
  const int64_t N = prob->n_traj;
  if (N < 0) return fail(GBDE_ERR_INVALID, "n_traj must be >= 0 (got %lld)", (long long)N);
  if (prob->save_kind != GBDE_SAVE_GRID && prob->save_kind != GBDE_SAVE_PER_TRAJ)
    return fail(GBDE_ERR_INVALID, "unknown save_kind %d", prob->save_kind);
  if (prob->n_save < 0) return fail(GBDE_ERR_INVALID, "n_save must be >= 0");
  if (N > 0 && (!prob->p || !prob->u0 || !prob->t0 || !prob->tf))
    return fail(GBDE_ERR_INVALID, "p, u0, t0 and tf must be non-NULL");
  if (prob->n_save > 0 && !prob->saveat)
    return fail(GBDE_ERR_INVALID, "saveat must be non-NULL when n_save > 0");
  if (out->reduce)
    return fail(GBDE_ERR_UNSUPPORTED, "gbde_ensemble_solve_noalloc has no in-kernel reduction");
  if (N > 0 && (!out->retcode || (prob->n_save > 0 && !out->u)))
    return fail(GBDE_ERR_INVALID, "out->u and out->retcode must be non-NULL");
  if (out->u_dtype != GBDE_F64 && out->u_dtype != GBDE_F32)
    return fail(GBDE_ERR_INVALID, "u_dtype must be GBDE_F64 or GBDE_F32");
  const int alg = opts->alg;
  if (alg == GBDE_ALG_AUTO)
    return fail(GBDE_ERR_UNSUPPORTED,
                "GBDE_ALG_AUTO needs per-trajectory lists (device scratch that grows with "
                "n_traj): use gbde_ensemble_solve");
  if (!is_ode(alg) && !is_sde(alg)) return fail(GBDE_ERR_INVALID, "unknown algorithm id %d", alg);
  if (is_sde(alg) && prob->model != GBDE_MODEL_LOTKA_VOLTERRA)
    return fail(GBDE_ERR_UNSUPPORTED, "SDE algorithms need a model with a noise term");
  if (opts->precision != GBDE_PREC_FP64 && opts->precision != GBDE_PREC_MIXED &&
      opts->precision != GBDE_PREC_F32X2)
    return fail(GBDE_ERR_INVALID, "unknown precision %d", opts->precision);
  if (opts->precision == GBDE_PREC_F32X2 &&
      (is_sde(alg) || prob->model == GBDE_MODEL_VDP_RING8))
    return fail(GBDE_ERR_UNSUPPORTED,
                "GBDE_PREC_F32X2 is built for the one-thread-per-trajectory ODE kernels");
  if (opts->batching != GBDE_BATCH_PLAIN && opts->batching != GBDE_BATCH_PERSISTENT)
    return fail(GBDE_ERR_INVALID, "unknown batching %d", opts->batching);
  if (opts->adaptive && !(opts->reltol > 0.0 && opts->abstol > 0.0))
    return fail(GBDE_ERR_INVALID, "adaptive stepping needs reltol > 0 and abstol > 0");
  if (!opts->adaptive && !(opts->dt > 0.0))
    return fail(GBDE_ERR_INVALID, "fixed-step solving needs dt > 0");
  if (opts->maxiters <= 0) return fail(GBDE_ERR_INVALID, "maxiters must be > 0");
  if (opts->adaptive && !(opts->qmin > 0.0 && opts->qmax >= 1.0 && opts->gamma > 0.0))
    return fail(GBDE_ERR_INVALID, "controller needs qmin > 0, qmax >= 1, gamma > 0");
  if (opts->callback != 0)
    return fail(GBDE_ERR_UNSUPPORTED, "gbde_ensemble_solve_noalloc runs no callbacks");
  if (opts->learned)
    return fail(GBDE_ERR_STATE, "gbde_ensemble_solve_noalloc has no learned predictor (learned != 0)");
  if (alg == GBDE_ALG_ROSENBROCK23 && prob->model == GBDE_MODEL_VDP_RING8)
    return fail(GBDE_ERR_UNSUPPORTED,
                "Rosenbrock23 is built for n_state <= 3 (use Rodas5 / Rodas5P for the ring)");
  if (is_switch(alg) &&
      (opts->precision == GBDE_PREC_F32X2 || prob->model == GBDE_MODEL_VDP_RING8))
    return fail(GBDE_ERR_UNSUPPORTED,
                "the AutoTsit5 composites run one-thread models in FP64 or GBDE_PREC_MIXED");
  if (opts->threads_per_traj != 0 && opts->threads_per_traj != 1 && opts->threads_per_traj != 16)
    return fail(GBDE_ERR_INVALID, "threads_per_traj must be 0, 1 or 16");
  if (opts->threads_per_traj == 16 && prob->model != GBDE_MODEL_VDP_RING8)
    return fail(GBDE_ERR_UNSUPPORTED, "16-lane teams are built for the 16-state ring");
  if (opts->threads_per_traj == 1 && prob->model == GBDE_MODEL_VDP_RING8 &&
      alg != GBDE_ALG_TSIT5 && alg != GBDE_ALG_VERN7)
    return fail(GBDE_ERR_UNSUPPORTED,
                "Rosenbrock methods on the 16-state ring run as 16-lane teams only");
  if (opts->chunk < 0) return fail(GBDE_ERR_INVALID, "chunk must be >= 0");
  const int block = opts->block_size > 0 ? opts->block_size : 128;
  if (block > 128 || (block & 31))
    return fail(GBDE_ERR_INVALID, "block_size must be a multiple of 32 and <= 128");
  // Scratch this solve needs against what the static array holds.
  if (kWordsUsed > kScratchWords)
    return fail(GBDE_ERR_INVALID, "solve needs %d bytes of scratch; the static array holds %d",
                kWordsUsed * 8, GBDE_NOALLOC_SCRATCH_BYTES);

  int device = 0;
  NOALLOC_CUDA(cudaGetDevice(&device));
  if (device < 0 || device >= kMaxDevices)
    return fail(GBDE_ERR_INVALID, "device %d beyond the %d devices this entry point serves", device,
                kMaxDevices);
  DeviceSetup dev;
  const int rc = device_setup(device, &dev);
  if (rc != GBDE_OK) return rc;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long* queue = dev.scratch;
  int32_t* flag_dev = reinterpret_cast<int32_t*>(dev.scratch + 1);
  // The array keeps the previous call's contents: clear the counter and the
  // status word before this launch, in stream order.
  NOALLOC_CUDA(cudaMemsetAsync(dev.scratch, 0, kWordsUsed * sizeof(unsigned long long), s));

  KArgs a;
  std::memset(&a, 0, sizeof(a));
  a.N = N;
  a.n_save = prob->n_save;
  a.save_kind = prob->save_kind;
  a.p = prob->p;
  a.u0 = prob->u0;
  a.t0 = prob->t0;
  a.tf = prob->tf;
  a.saveat = prob->saveat;
  a.u_out = out->u;
  a.out_f32 = out->u_dtype == GBDE_F32;
  a.retcode = out->retcode;
  a.naccept = out->naccept;
  a.nreject = out->nreject;
  a.nf = out->nf;
  a.t_end = out->t_end;
  a.method_out = out->method;
  a.dt_first = out->dt_first;
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
  if (is_switch(alg)) {  // the stiff method steps with its own exponents (its defaults)
    gbde_opts r;
    gbde_opts_default(alg == GBDE_ALG_AUTOTSIT5_RODAS5 ? GBDE_ALG_RODAS5 : GBDE_ALG_ROSENBROCK23,
                      &r);
    a.ctl_stiff = ctl_consts(r.beta1, r.beta2, opts->gamma, opts->qmin, opts->qmax,
                             opts->qsteady_min, opts->qsteady_max, opts->qoldinit);
  }
  a.chunk = opts->chunk > 0 ? opts->chunk : 1;
  a.queue = opts->batching == GBDE_BATCH_PERSISTENT ? queue : nullptr;
  a.flag = flag_dev;

  LaunchCfg cfg;
  cfg.alg = alg;
  cfg.model = prob->model;
  cfg.precision = opts->precision;
  cfg.persistent = opts->batching == GBDE_BATCH_PERSISTENT;
  cfg.block = block;
  cfg.grid = 0;
  cfg.ctas_per_sm = opts->ctas_per_sm;
  cfg.num_sms = dev.num_sms;
  cfg.tpt = opts->threads_per_traj;

  if (N > 0) {
    const cudaError_t e = launch_alg(alg, cfg, a, s);
    if (e == cudaErrorNotSupported)
      return fail(GBDE_ERR_UNSUPPORTED, "algorithm %d is not built for model %d", alg, prob->model);
    if (e != cudaSuccess) return fail(GBDE_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  }
  int32_t flag = 0;
  NOALLOC_CUDA(cudaMemcpyAsync(&flag, flag_dev, sizeof(flag), cudaMemcpyDeviceToHost, s));
  NOALLOC_CUDA(cudaStreamSynchronize(s));
  out->device_ms = 0.0f;  // not measured: timing events are not created here
  out->total_ms = (float)std::chrono::duration<double, std::milli>(
                      std::chrono::steady_clock::now() - wall0).count();
  if (flag & 1)
    return fail(GBDE_ERR_TIMEOUT, "device deadline of %.3f s reached; unfinished trajectories "
                "carry GBDE_RET_TIMEOUT", opts->timeout_s);
  return GBDE_OK;
}
