"""Host-side logic and the C ABI surface (no GPU compute)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "gbde.h")).read()
    return sorted(set(re.findall(r"GBDE_API\s+(?:const\s+)?\w+\*?\s+\*?(gbde_\w+)\(", src)))


def test_library_exports_every_header_symbol(capi):
    names = header_functions()
    assert "gbde_ensemble_solve" in names and len(names) >= 11
    L = C.CDLL(capi.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
    # the ctypes table covers the header exactly
    assert sorted(capi.SIGNATURES) == names


def test_header_struct_layout_matches_ctypes(capi):
    """Field order and count of the ctypes mirrors == gbde.h."""
    src = open(os.path.join(ROOT, "include", "gbde.h")).read()
    for cname, py in (("gbde_problem", capi.Problem), ("gbde_opts", capi.Opts),
                      ("gbde_outputs", capi.Outputs)):
        body = dict((n, b) for b, n in re.findall(r"typedef struct \{([^{}]*)\}\s*(\w+);", src))[cname]
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        fields = re.findall(r"(\w+)\s*(?:,|;)", body)
        assert fields == [f[0] for f in py._fields_], cname


def test_oracle_restates_the_abi(capi, oracle):
    """The oracle carries its own copy of gbde.h's structs, constants and
    option defaults (so that it never loads the product library); they must
    equal the product's, field for field."""
    for py, orc in ((capi.Problem, oracle.Problem), (capi.Opts, oracle.Opts),
                    (capi.Outputs, oracle.Outputs)):
        assert [f[0] for f in py._fields_] == [f[0] for f in orc._fields_]
        assert C.sizeof(py) == C.sizeof(orc)
        for (n, _), (n2, _) in zip(py._fields_, orc._fields_):
            assert getattr(py, n).offset == getattr(orc, n2).offset, n
    for name in ("MODEL_LINEAR", "MODEL_LORENZ", "MODEL_ROBERTSON", "MODEL_VDP_RING8",
                 "MODEL_LOTKA_VOLTERRA", "ALG_TSIT5", "ALG_VERN7", "ALG_ROSENBROCK23",
                 "ALG_RODAS5", "ALG_RODAS5P", "ALG_EM", "ALG_SOSRI", "ALG_AUTO", "ALG_SRIW1",
                 "ALG_AUTOTSIT5_ROSENBROCK23", "ALG_AUTOTSIT5_RODAS5", "SAVE_GRID",
                 "SAVE_PER_TRAJ", "MEM_HOST", "F64", "F32", "RET_SUCCESS"):
        assert getattr(capi, name) == getattr(oracle, name), name
    for mid, size in oracle.MODEL_SIZES.items():
        assert capi.model_info(mid) == size
    algs = [capi.ALG_TSIT5, capi.ALG_VERN7, capi.ALG_ROSENBROCK23, capi.ALG_RODAS5,
            capi.ALG_RODAS5P, capi.ALG_EM, capi.ALG_SOSRI, capi.ALG_AUTO, capi.ALG_SRIW1,
            capi.ALG_AUTOTSIT5_ROSENBROCK23, capi.ALG_AUTOTSIT5_RODAS5]
    for alg in algs:
        a, b = capi.opts_default(alg), oracle.opts_default(alg)
        for n, _ in capi.Opts._fields_:
            assert getattr(a, n) == getattr(b, n), (alg, n)


def test_version_and_model_info(capi):
    assert capi.lib().gbde_version() == 4
    assert capi.model_info(capi.MODEL_LORENZ) == (3, 3)
    assert capi.model_info(capi.MODEL_VDP_RING8) == (16, 2)
    with pytest.raises(capi.GBDEError):
        capi.model_info(99)


def test_opts_defaults(capi):
    o = capi.opts_default(capi.ALG_TSIT5)
    assert o.adaptive == 1 and abs(o.beta1 - 0.17) < 1e-15 and abs(o.beta2 - 0.04) < 1e-15
    assert o.qmin == 0.2 and o.qmax == 10.0 and o.gamma == 0.9
    o = capi.opts_default(capi.ALG_EM)
    assert o.adaptive == 0
    with pytest.raises(capi.GBDEError):
        capi.opts_default(42)


def test_ctx_create_without_gpu_fails_cleanly(capi):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(capi.GBDEError) as e:
        capi.Context(0)
    assert e.value.code == capi.GBDE_ERR_CUDA


def test_save_grid_semantics(de):
    g = de.save_grid(0.0, 1.0, 0.1)  # core.jl:90-96
    assert len(g) == 11 and g[0] == 0.0 and g[-1] == 1.0
    assert g[3] == 0.3  # decimal step, not 3 * 0.1
    g = de.save_grid(0.0, 1.0, 0.1, save_start=False)
    assert len(g) == 10 and g[0] == 0.1
    g = de.save_grid(0.0, 1.0, [0.5, 0.25])
    assert list(g) == [0.25, 0.5]  # vector saveat: t0/tf only when listed
    g = de.save_grid(0.0, 1.0, [0.0, 0.5, 1.0])
    assert list(g) == [0.0, 0.5, 1.0]
    g = de.save_grid(0.0, 20.0, 1.0)
    assert len(g) == 21


def test_problem_and_remake(de):
    prob = de.ODEProblem(de.models.linear, 0.5, (0.0, 1.0), [1.01])
    q = de.remake(prob, u0=1.0)  # core.jl:81-88
    assert q.u0[0] == 1.0 and prob.u0[0] == 0.5
    with pytest.raises(ValueError):
        de.ODEProblem(de.models.lorenz, [1.0, 0.0], (0.0, 1.0), [10, 28, 8 / 3])
    with pytest.raises(TypeError):
        de.ODEProblem(lambda u, p, t: u, [1.0], (0.0, 1.0))
    with pytest.raises(TypeError):
        de.SDEProblem(de.models.lorenz, None, [1.0, 0, 0], (0.0, 1.0), [1, 1, 1])


def test_solve_rejects_unsupported(de):
    prob = de.ODEProblem(de.models.linear, 0.5, (0.0, 1.0), [1.01])
    ens = de.EnsembleProblem(prob)
    for key in ("save_everystep", "tstops", "save_idxs"):
        with pytest.raises(NotImplementedError):
            de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=2, saveat=0.1,
                     **{key: True})
    with pytest.raises(TypeError):  # callbacks are the callback classes and sets of them
        de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=2, saveat=0.1,
                 callback=object())
    with pytest.raises(NotImplementedError):
        de.solve(ens, de.Tsit5(), de.EnsembleThreads(), trajectories=2, saveat=0.1)
    with pytest.raises(NotImplementedError):
        de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=2)  # no saveat
    with pytest.raises(TypeError):
        de.solve(ens, de.EM(), de.EnsembleGB300(), trajectories=2, saveat=0.1)
    with pytest.raises(TypeError):
        de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=2, saveat=0.1, bogus=1)


def test_gather_inputs_prob_func(de):
    from differentialequations_gb300 import api
    prob = de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8 / 3])
    ens = de.EnsembleProblem(prob, prob_func=lambda pr, i, rep: de.remake(pr, p=pr.p * (1 + i)))
    u0, p, tspan, saves, probs = api._gather_inputs(ens, 3)
    assert np.allclose(p[2], [30.0, 84.0, 8.0])
    assert np.allclose(u0, [[1, 0, 0]] * 3) and saves is None and len(probs) == 3
    ens = de.EnsembleProblem(prob, batch=lambda pr, n: {"tspan": np.c_[np.zeros(n), np.arange(1, n + 1)]})
    u0, p, tspan, saves, _ = api._gather_inputs(ens, 4)
    assert np.allclose(tspan[:, 1], [1, 2, 3, 4])


def test_shard_ranges_partition(de):
    from differentialequations_gb300 import distributed
    for N in (0, 1, 7, 100, 1001):
        for W in (1, 2, 3, 8):
            parts = [distributed.shard_range(N, r, W) for r in range(W)]
            covered = []
            for a, b in parts:
                covered += list(range(a, b))
            assert covered == list(range(N))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
