// k_team.cu -- team kernels for 16-state models (ring of 8 Van der Pol
// oscillators): Rodas5 / Rodas5P with a row-distributed FP64 LU and Tsit5,
// 16 lanes per trajectory (team.cuh).
#include "team.cuh"
#include "launch.h"

namespace gbde {

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128) k_team(const KArgs a) {
  integrate_team<Alg, M, T, MIXED>(a);
}

template <class M, class T> using TeamRodas5 = TeamRodas<M, T, Rodas5Tag>;
template <class M, class T> using TeamRodas5P = TeamRodas<M, T, Rodas5PTag>;

template <template <class, class> class AlgT, class M>
static cudaError_t dispatch_prec(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_MIXED)
    return launch_team_kernel(k_team<AlgT<M, float>, M, float, true>, cfg, a, s);
  return launch_team_kernel(k_team<AlgT<M, double>, M, double, false>, cfg, a, s);
}

cudaError_t launch_team(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.model != GBDE_MODEL_VDP_RING8) return cudaErrorNotSupported;
  if (cfg.block & 31) return cudaErrorInvalidValue;  // teams must not straddle warps
  using M = VdpRing8;
  switch (cfg.alg) {
    case GBDE_ALG_TSIT5: return dispatch_prec<TeamTsit5, M>(cfg, a, s);
    case GBDE_ALG_RODAS5: return dispatch_prec<TeamRodas5, M>(cfg, a, s);
    case GBDE_ALG_RODAS5P: return dispatch_prec<TeamRodas5P, M>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

}  // namespace gbde
