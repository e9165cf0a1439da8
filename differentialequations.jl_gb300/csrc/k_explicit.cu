// k_explicit.cu -- Tsit5 / Vern7 ensemble kernels (one trajectory per thread).
#include "explicit_rk.cuh"
#include "ff.cuh"
#include "tsit5_ff.cuh"
#include "vern7_ff.cuh"
#include "launch.h"

namespace gbde {

// Resident CTAs of 128 threads per SM the kernel is compiled for.  Vern7's
// 7th-order dense output (seven lazy stages on saving steps) needs more
// registers than its steps: capping the kernel at the steps' need moves the
// excess to local memory on the saving path instead of costing occupancy on
// every step -- 128 registers (4 CTAs) for FP64 / FP32 state, 168 (3 CTAs)
// for FP32 pairs on up to three states.
template <class Alg> struct ErkMinBlocks { static constexpr int v = 1; };
template <class M, class T> struct ErkMinBlocks<Vern7Alg<M, T>> {
  static constexpr int v = M::N <= 3 ? 4 : 1;
};
template <class M> struct ErkMinBlocks<Vern7FF<M>> { static constexpr int v = 3; };

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128, ErkMinBlocks<Alg>::v) k_erk(const KArgs a) {
  integrate_all<Alg, M, T, MIXED>(a);
}

template <template <class, class> class AlgT, class M>
static cudaError_t dispatch_prec(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_MIXED)
    return launch_step_kernel<AlgT<M, float>, M, float>(k_erk<AlgT<M, float>, M, float, true>,
                                                         cfg, a, s);
  if (cfg.precision == GBDE_PREC_F32X2) {
    if constexpr (M::N <= 8)  // pairs double the register state; the 16-state ring has team kernels
      return launch_step_kernel<AlgT<M, ff>, M, ff>(k_erk<AlgT<M, ff>, M, ff, true>, cfg, a, s);
    else
      return cudaErrorNotSupported;
  }
  return launch_step_kernel<AlgT<M, double>, M, double>(k_erk<AlgT<M, double>, M, double, false>,
                                                         cfg, a, s);
}

template <template <class, class> class AlgT>
static cudaError_t dispatch_model(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  switch (cfg.model) {
    case GBDE_MODEL_LINEAR: return dispatch_prec<AlgT, Linear>(cfg, a, s);
    case GBDE_MODEL_LORENZ: return dispatch_prec<AlgT, Lorenz>(cfg, a, s);
    case GBDE_MODEL_ROBERTSON: return dispatch_prec<AlgT, Robertson>(cfg, a, s);
    case GBDE_MODEL_VDP_RING8: return dispatch_prec<AlgT, VdpRing8>(cfg, a, s);
    case GBDE_MODEL_LOTKA_VOLTERRA: return dispatch_prec<AlgT, LotkaVolterra>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_explicit(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.alg == GBDE_ALG_TSIT5) return dispatch_model<Tsit5A>(cfg, a, s);
  if (cfg.alg == GBDE_ALG_VERN7) return dispatch_model<Vern7A>(cfg, a, s);
  return cudaErrorNotSupported;
}

}  // namespace gbde
