// k_team.cu -- team kernels for 16-state models (ring of 8 Van der Pol
// oscillators, team.cuh): Rodas5 / Rodas5P with a row-distributed FP64 LU on
// 16 lanes per trajectory (FP64 and FP32 state), or on 8 lanes per trajectory
// in FP32 pairs with an FP32 LU, W^-1 and refined solves; Tsit5 on 8 lanes per
// trajectory.
#include "team.cuh"
#include "launch.h"

namespace gbde {

// Resident CTAs of 128 threads per SM each team stepper is compiled for: the
// Rodas steppers are latency-bound on their broadcast chains (LU, triangular
// solves), so more resident warps beat more registers.  With W's rows in
// shared memory (team.cuh, 17 KB per CTA) the 16-lane Rodas steppers fit 6
// CTAs (<= 80 registers, no spills).  The 8-lane pair Rodas holds 3 KB of
// shared memory per trajectory (FP32 W rows, W^-1 rows, stages): CTAs of 96
// threads (12 teams, 36.1 KB), 6 per SM, 96 registers.  7 per SM caps the
// registers at 80 and spills in the stage loop (457 against 261 ms on the
// 250k stiff trajectories, with the refined FP32 substitutions).
// The 8-lane Tsit5 teams measured 368 / 338 / 290 / 280 ms at 1 / 4 / 5 / 6
// CTAs per SM on the 750k non-stiff trajectories of the 1M ring workload.
template <class Alg> struct TeamMinBlocks { static constexpr int v = 1; };
template <class M, class T, class Tag> struct TeamMinBlocks<TeamRodas<M, T, Tag>> {
  static constexpr int v = 6;
};
template <class M, class T> struct TeamMinBlocks<TeamTsit5P<M, T>> {
  static constexpr int v = 6;
};
template <class M> struct TeamMinBlocks<TeamTsit5FF<M>> {
  static constexpr int v = 6;
};
template <class M, class Tag> struct TeamMinBlocks<TeamRodasFF8<M, Tag>> {
  static constexpr int v = 6;
};
// Threads per CTA a team kernel is compiled for (its launch's block size
// at most): 128, but the pair Rodas's kTeam8Threads (team.cuh)
template <class Alg> struct TeamThreads { static constexpr int v = 128; };
template <class M, class Tag> struct TeamThreads<TeamRodasFF8<M, Tag>> {
  static constexpr int v = kTeam8Threads;
};

template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(128, TeamMinBlocks<Alg>::v) k_team(const KArgs a) {
  integrate_team<Alg, M, T, MIXED>(a);
}

// 8-lane teams, one oscillator per lane (team.cuh)
template <class Alg, class M, class T, bool MIXED>
__global__ void __launch_bounds__(TeamThreads<Alg>::v, TeamMinBlocks<Alg>::v) k_team8(const KArgs a) {
  integrate_team8<Alg, M, T, MIXED>(a);
}

// Rodas: FP32 pairs on 8-lane teams (TeamRodasFF8); FP32 or FP64 state on
// 16-lane teams (TeamRodas).
template <class Tag, class M>
static cudaError_t launch_team_rodas(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  if (cfg.precision == GBDE_PREC_F32X2) {
    LaunchCfg c = cfg;  // its shared arrays hold kTeam8Threads threads' teams
    if (c.block <= 0 || c.block > kTeam8Threads) c.block = kTeam8Threads;
    return launch_team_kernel(k_team8<TeamRodasFF8<M, Tag>, M, ff, true>, c, a, s, 8);
  }
  if (cfg.precision == GBDE_PREC_MIXED)
    return launch_team_kernel(k_team<TeamRodas<M, float, Tag>, M, float, true>, cfg, a, s);
  return launch_team_kernel(k_team<TeamRodas<M, double, Tag>, M, double, false>, cfg, a, s);
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
    case GBDE_ALG_RODAS5: return launch_team_rodas<Rodas5Tag, M>(cfg, a, s);
    case GBDE_ALG_RODAS5P: return launch_team_rodas<Rodas5PTag, M>(cfg, a, s);
  }
  return cudaErrorNotSupported;
}

}  // namespace gbde
