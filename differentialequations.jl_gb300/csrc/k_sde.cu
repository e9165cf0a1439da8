// k_sde.cu -- Euler-Maruyama and SRI (SOSRI, SRIW1) ensemble kernels.
#include "sde.cuh"
#include "launch.h"

namespace gbde {

template <class M, class T>
__global__ void __launch_bounds__(128) k_em(const KArgs a) {
  em_all<M, T>(a);
}

template <class M, class T, bool MIXED, class Tab, int ALG>
__global__ void __launch_bounds__(128) k_sri(const KArgs a) {
  sri_all<M, T, MIXED, Tab, ALG>(a);
}

cudaError_t launch_sde(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.model != GBDE_MODEL_LOTKA_VOLTERRA) return cudaErrorNotSupported;
  using M = LotkaVolterra;
  const bool mixed = cfg.precision == GBDE_PREC_MIXED;
  if (cfg.alg == GBDE_ALG_EM)
    return mixed ? launch_kernel(k_em<M, float>, cfg, a, s) : launch_kernel(k_em<M, double>, cfg, a, s);
  if (cfg.alg == GBDE_ALG_SOSRI)
    return mixed ? launch_kernel(k_sri<M, float, true, tab::SosriTab, GBDE_ALG_SOSRI>, cfg, a, s)
                 : launch_kernel(k_sri<M, double, false, tab::SosriTab, GBDE_ALG_SOSRI>, cfg, a, s);
  if (cfg.alg == GBDE_ALG_SRIW1)
    return mixed ? launch_kernel(k_sri<M, float, true, tab::Sriw1Tab, GBDE_ALG_SRIW1>, cfg, a, s)
                 : launch_kernel(k_sri<M, double, false, tab::Sriw1Tab, GBDE_ALG_SRIW1>, cfg, a, s);
  return cudaErrorNotSupported;
}

}  // namespace gbde
