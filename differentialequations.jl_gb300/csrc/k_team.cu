// k_team.cu -- team kernels for 16-state models (ring of 8 Van der Pol
// oscillators): Rodas5 / Rodas5P with a row-distributed FP64 LU, 16 lanes per
// trajectory, and Tsit5, 8 lanes per trajectory (team.cuh).
#include "team.cuh"
#include "launch.h"

namespace gbde {

// Resident CTAs of 128 threads per SM each team stepper is compiled for: the
// Rodas steppers are latency-bound on their broadcast chains (LU, triangular
// solves), so more resident warps beat more registers.  With W's rows in
// shared memory (team.cuh, 17 KB per CTA, 24 KB with the pair stages) both fit
// 6 CTAs (<= 80 registers, no spills in the Rodas5 steppers): 914 -> 625 ms on
// the 250k stiff trajectories of the 1M ring workload.  The 8-lane Tsit5 team
// (two components per lane) measured 368 / 338 / 290 / 280 ms at 1 / 4 / 5 / 6
// CTAs per SM on the 750k non-stiff trajectories (16-lane teams: 370 ms).
template <class Alg> struct TeamMinBlocks { static constexpr int v = 1; };
template <class M, class T, class Tag> struct TeamMinBlocks<TeamRodas<M, T, Tag>> {
  static constexpr int v = 6;
};
template <class M, class Tag> struct TeamMinBlocks<TeamRodasFF<M, Tag>> {
  static constexpr int v = 6;
};
template <class M, class T> struct TeamMinBlocks<TeamTsit5P<M, T>> {
  static constexpr int v = 6;
};
template <class M> struct TeamMinBlocks<TeamTsit5FF<M>> {
  static constexpr int v = 6;
};

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128, TeamMinBlocks<Alg>::v) k_team(const KArgs a) {
  integrate_team<Alg, M, T, MIXED>(a);
}

// Tsit5 on the ring: 8-lane teams, one oscillator per lane (team.cuh)
template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128, TeamMinBlocks<Alg>::v) k_team8(const KArgs a) {
  integrate_team8<Alg, M, T, MIXED>(a);
}

// Rodas in FP32 pairs is its own stepper (TeamRodasFF); Tsit5 takes the
// pair type directly.
template <class M, class T, class Tag> struct TeamRodasSel { using type = TeamRodas<M, T, Tag>; };
template <class M, class Tag> struct TeamRodasSel<M, ff, Tag> { using type = TeamRodasFF<M, Tag>; };
template <class M, class T> using TeamRodas5 = typename TeamRodasSel<M, T, Rodas5Tag>::type;
template <class M, class T> using TeamRodas5P = typename TeamRodasSel<M, T, Rodas5PTag>::type;

template <template <class, class> class AlgT, class M>
static cudaError_t dispatch_prec(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_MIXED)
    return launch_team_kernel(k_team<AlgT<M, float>, M, float, true>, cfg, a, s);
  if (cfg.precision == GBDE_PREC_F32X2)
    return launch_team_kernel(k_team<AlgT<M, ff>, M, ff, true>, cfg, a, s);
  return launch_team_kernel(k_team<AlgT<M, double>, M, double, false>, cfg, a, s);
}

cudaError_t launch_team(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.model != GBDE_MODEL_VDP_RING8) return cudaErrorNotSupported;
  if (cfg.block & 31) return cudaErrorInvalidValue;  // teams must not straddle warps
  using M = VdpRing8;
  switch (cfg.alg) {
    case GBDE_ALG_TSIT5:
      if (cfg.precision == GBDE_PREC_MIXED)
        return launch_team_kernel(k_team8<TeamTsit5P<M, float>, M, float, true>, cfg, a, s, 8);
      if (cfg.precision == GBDE_PREC_F32X2)
        return launch_team_kernel(k_team8<TeamTsit5FF<M>, M, ff, true>, cfg, a, s, 8);
      return launch_team_kernel(k_team8<TeamTsit5P<M, double>, M, double, false>, cfg, a, s, 8);
    case GBDE_ALG_RODAS5: return dispatch_prec<TeamRodas5, M>(cfg, a, s);
    case GBDE_ALG_RODAS5P: return dispatch_prec<TeamRodas5P, M>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

}  // namespace gbde
