"""GB300-native ensemble ODE/SDE solver: a drop-in `ensemblealg` for the
data-parallel hot path of DifferentialEquations.jl,

    solve(EnsembleProblem(prob; prob_func), alg, EnsembleGB300();
          trajectories, saveat, reltol, abstol)

The compute path is libgbde.so (hand-written sm_103a kernels behind a C ABI,
include/gbde.h); this package is the host-side mirror of the reference's
SciMLBase interface over that ABI.
"""
from . import _capi, learned, tuning
from .api import (EM, SOSRI, SRIW1, AutoTsit5, CallbackSet, ContinuousCallback, DiscreteCallback,
                  VectorContinuousCallback, EnsembleGB300, EnsembleProblem, EnsembleSerial,
                  EnsembleSolution, EnsembleThreads, ODEFunction, ODEProblem, ODESolution,
                  SDEFunction,
                  ReturnCode, EnsembleSummary, compile_model, ensemble_summary,
                  Rodas5, Rodas5P, Rosenbrock23, SDEProblem, Tsit5, Vern7, models, remake,
                  save_grid, solve, solve_arrays)

__all__ = [
    "EM", "SOSRI", "SRIW1", "AutoTsit5", "CallbackSet", "ContinuousCallback", "DiscreteCallback",
    "VectorContinuousCallback", "EnsembleGB300", "EnsembleProblem", "EnsembleSerial", "EnsembleSolution",
    "EnsembleThreads", "ODEFunction", "SDEFunction", "ODEProblem", "ODESolution", "compile_model", "EnsembleSummary", "ensemble_summary",
    "ReturnCode", "Rodas5", "Rodas5P",
    "Rosenbrock23", "SDEProblem", "Tsit5", "Vern7", "models", "remake", "save_grid", "solve",
    "solve_arrays",
]
