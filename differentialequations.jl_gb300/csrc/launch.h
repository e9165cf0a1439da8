// launch.h -- internal interface between the C ABI layer and the kernel
// translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "solver.cuh"

namespace gbde {

struct LaunchCfg {
  int alg, model, precision;
  bool persistent;
  int block;          // threads per CTA
  int grid;           // CTAs (persistent) -- 0 = derive from N
  int ctas_per_sm;    // persistent: resident CTAs per SM (0 = occupancy max)
  int num_sms;
  int tpt = 0;        // threads per trajectory (0 = model default, 1, 16)
  double* dt_init = nullptr;  // scratch [N]: run the initial-dt pre-pass into it
  int callback = 0;   // gbde_callback_register id (runtime-compiled kernels)
};

// Returns cudaSuccess, or cudaErrorNotSupported for an unknown combination.
cudaError_t launch_explicit(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);
cudaError_t launch_rosenbrock(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);
cudaError_t launch_sde(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);
cudaError_t launch_autoswitch(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);

// Order of the persistent queue (order.cu): longest span first, or, with a
// learned cost per trajectory (log2 of its predicted attempted steps), most
// expensive first.
size_t span_order_scratch_bytes(int64_t n);
cudaError_t build_span_order(const double* t0, const double* tf, int64_t n, void* scratch,
                             int num_sms, cudaStream_t s, const int32_t** order_out);
cudaError_t build_cost_order(const float* log2_cost, int64_t n, void* scratch, int num_sms,
                             cudaStream_t s, const int32_t** order_out);

// Launch geometry helper shared by the translation units.
template <class K>
cudaError_t launch_kernel(K kern, const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  int block = cfg.block > 0 ? cfg.block : 128;
  int grid;
  if (cfg.persistent) {
    int per_sm = cfg.ctas_per_sm;
    if (per_sm <= 0) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) per_sm = 1;
    }
    grid = per_sm * cfg.num_sms;
    const long long need = (a.N + block - 1) / block;
    if (grid > need) grid = (int)(need > 0 ? need : 1);
  } else {
    const long long g = (a.N + block - 1) / block;
    grid = (int)(g > 0 ? g : 1);
  }
  kern<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

// Any ODE/SDE algorithm id except GBDE_ALG_AUTO (capi.cu).
cudaError_t launch_alg(int alg, LaunchCfg cfg, const KArgs& a, cudaStream_t s);

// Stiff / non-stiff lists for GBDE_ALG_AUTO (auto.cu).
size_t partition_scratch_bytes(int64_t n);
cudaError_t build_partition(const double* p, int np, double thr, const int8_t* pred, int64_t n,
                            void* scratch, unsigned* counters, int num_sms, cudaStream_t s,
                            int32_t** nonstiff, int32_t** stiff);

// Learned predictions for a solve (mlp.cu): pred_dt[N], pred_stiff[N] and
// pred_cost[N] (log2 of the attempted steps).
cudaError_t mlp_predict(int model, const float* net, const KArgs& a, float* pred_dt,
                        int8_t* pred_stiff, float* pred_cost, int num_sms, cudaStream_t s);

// One-thread-per-trajectory step kernel, preceded by the initial-dt pre-pass
// (k_init_dt) when cfg.dt_init is set.
template <class Alg, class M, class T, class K>
cudaError_t launch_step_kernel(K kern, const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.dt_init == nullptr) return launch_kernel(kern, cfg, a, s);
  const long long want = (a.N + 127) / 128, cap = 8LL * cfg.num_sms;
  const int grid = (int)(want < cap ? (want > 0 ? want : 1) : cap);
  k_init_dt<Alg, M, T><<<grid, 128, 0, s>>>(a, cfg.dt_init);
  KArgs b = a;
  b.dt_init = cfg.dt_init;
  return launch_kernel(kern, cfg, b, s);
}

// User models compiled at run time (rtc.cu): ids >= GBDE_MODEL_USER_BASE.
bool rtc_model_info(int id, int32_t* n_state, int32_t* n_param);
bool rtc_model_has_noise(int id);
int rtc_prepare(int id, int alg, int precision, int callback, std::string* err);
cudaError_t launch_rtc(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);

// Ensemble statistics over u[N][C] in device memory (summary.cu).
int summary_sum_blocks(int C, int num_sms);
size_t summary_scratch_bytes(int64_t N, int C, int u_f32, int nq, int sum_blocks);
cudaError_t enqueue_summary(const void* u, int u_f32, int64_t N, int C, int nq,
                            const double* q_host, double* mean, double* var, double* qv,
                            void* scratch, int num_sms, cudaStream_t s);

// Team kernels (team.cuh): 16 threads per trajectory.
cudaError_t launch_team(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s);

template <class K>
cudaError_t launch_team_kernel(K kern, const LaunchCfg& cfg, const KArgs& a, cudaStream_t s,
                               int lanes = 16) {
  const int block = cfg.block > 0 ? cfg.block : 128;
  const long long need = (a.N * lanes + block - 1) / block;
  int grid;
  if (cfg.persistent) {
    int per_sm = cfg.ctas_per_sm;
    if (per_sm <= 0) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) per_sm = 1;
    }
    grid = per_sm * cfg.num_sms;
    if (grid > need) grid = (int)(need > 0 ? need : 1);
  } else {
    grid = (int)(need > 0 ? need : 1);
  }
  kern<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gbde
