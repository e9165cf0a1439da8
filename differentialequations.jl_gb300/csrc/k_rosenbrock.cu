// k_rosenbrock.cu -- Rosenbrock23 / Rodas5 / Rodas5P ensemble kernels
// (one trajectory per thread, W-matrix LU in registers; models with n <= 3).
// In the F32X2 precision Rodas5 / Rodas5P run the compact pair stepper of
// rodas_ff.cuh and Rosenbrock23 the one of ros23_ff.cuh.
#include "rosenbrock.cuh"
#include "rodas_ff.cuh"
#include "ros23_ff.cuh"
#include "ff.cuh"
#include "launch.h"

namespace gbde {

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128) k_ros(const KArgs a) {
  integrate_all<Alg, M, T, MIXED>(a);
}

template <class M, class T, class Tag> struct RodasSel { using type = RodasAlg<M, T, Tag>; };
template <class M, class Tag> struct RodasSel<M, ff, Tag> { using type = RodasFF<M, Tag>; };
template <class M, class T> using Rodas5A = typename RodasSel<M, T, Rodas5Tag>::type;
template <class M, class T> using Rodas5PA = typename RodasSel<M, T, Rodas5PTag>::type;

template <template <class, class> class AlgT, class M>
static cudaError_t dispatch_prec(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_MIXED)
    return launch_step_kernel<AlgT<M, float>, M, float>(k_ros<AlgT<M, float>, M, float, true>,
                                                         cfg, a, s);
  if (cfg.precision == GBDE_PREC_F32X2) {
    return launch_step_kernel<AlgT<M, ff>, M, ff>(k_ros<AlgT<M, ff>, M, ff, true>, cfg, a, s);
  }
  return launch_step_kernel<AlgT<M, double>, M, double>(k_ros<AlgT<M, double>, M, double, false>,
                                                         cfg, a, s);
}

template <template <class, class> class AlgT>
static cudaError_t dispatch_model(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  switch (cfg.model) {
    case GBDE_MODEL_LINEAR: return dispatch_prec<AlgT, Linear>(cfg, a, s);
    case GBDE_MODEL_LORENZ: return dispatch_prec<AlgT, Lorenz>(cfg, a, s);
    case GBDE_MODEL_ROBERTSON: return dispatch_prec<AlgT, Robertson>(cfg, a, s);
    case GBDE_MODEL_LOTKA_VOLTERRA: return dispatch_prec<AlgT, LotkaVolterra>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_rosenbrock(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.alg == GBDE_ALG_ROSENBROCK23) return dispatch_model<Ros23A>(cfg, a, s);
  if (cfg.alg == GBDE_ALG_RODAS5) return dispatch_model<Rodas5A>(cfg, a, s);
  if (cfg.alg == GBDE_ALG_RODAS5P) return dispatch_model<Rodas5PA>(cfg, a, s);
  return cudaErrorNotSupported;
}

}  // namespace gbde
