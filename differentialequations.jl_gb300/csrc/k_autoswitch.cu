// k_autoswitch.cu -- AutoTsit5(Rosenbrock23()) / AutoTsit5(Rodas5()) ensemble
// kernels (one trajectory per thread; built-in models with n <= 3), FP64 or
// FP32 state (autoswitch.cuh).
#include "autoswitch.cuh"
#include "launch.h"

namespace gbde {

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128) k_switch(const KArgs a) {
  integrate_all<Alg, M, T, MIXED>(a);
}

template <class M, class T, bool MIXED, class S>
static cudaError_t launch_one(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  using A = AutoSwitchAlg<M, T, S>;
  return launch_step_kernel<A, M, T>(k_switch<A, M, T, MIXED>, cfg, a, s);
}

template <class M, class T, bool MIXED>
static cudaError_t dispatch_stiff(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.alg == GBDE_ALG_AUTOTSIT5_ROSENBROCK23)
    return launch_one<M, T, MIXED, Ros23Alg<M, T>>(cfg, a, s);
  if (cfg.alg == GBDE_ALG_AUTOTSIT5_RODAS5)
    return launch_one<M, T, MIXED, RodasAlg<M, T, Rodas5Tag>>(cfg, a, s);
  return cudaErrorNotSupported;
}

template <class M>
static cudaError_t dispatch_prec(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_FP64) return dispatch_stiff<M, double, false>(cfg, a, s);
  if (cfg.precision == GBDE_PREC_MIXED) return dispatch_stiff<M, float, true>(cfg, a, s);
  return cudaErrorNotSupported;  // no FP32-pair composite
}

cudaError_t launch_autoswitch(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  switch (cfg.model) {
    case GBDE_MODEL_LINEAR: return dispatch_prec<Linear>(cfg, a, s);
    case GBDE_MODEL_LORENZ: return dispatch_prec<Lorenz>(cfg, a, s);
    case GBDE_MODEL_ROBERTSON: return dispatch_prec<Robertson>(cfg, a, s);
    case GBDE_MODEL_LOTKA_VOLTERRA: return dispatch_prec<LotkaVolterra>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

}  // namespace gbde
