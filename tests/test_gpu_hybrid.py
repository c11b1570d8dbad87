"""HybridPSO local stage on the GPU vs the oracle (bit-identical per-particle
results) and the reference's L-BFGS known answers through solve()."""
import numpy as np
import pytest

from test_hybrid_oracle import CASES, hybrid_oracle

pytestmark = pytest.mark.gpu


def _problem(pps, orc, obj, name, D, lo, hi, prm):
    lb = np.full(D, lo, np.float32)
    ub = np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None, lb=lb, ub=ub)
    return prob, orc.OracleProblem(obj, D, lb, ub, params=prm)


@pytest.mark.parametrize("kind", ["lbfgs", "bfgs"])
@pytest.mark.parametrize("obj,name,D,prm", [(1, "rosenbrock", 10, [1.0, 100.0]), (3, "ackley", 10, [20.0, 0.2, 1.0]),
                                            (2, "rastrigin", 5, [10.0]), (0, "sphere", 3, []),
                                            (1, "rosenbrock", 40, [1.0, 100.0])])
def test_local_stage_matches_oracle(pps, orc, kind, obj, name, D, prm):
    if kind == "bfgs" and D > 16:
        pytest.skip("Broyden stage supports dim <= 16")
    from parallelparticleswarms import _lib

    prob, oprob = _problem(pps, orc, obj, name, D, -5.0, 5.0, prm)
    n = 3000
    with pps.Swarm(prob, n, seed=3) as sw:
        sw.init()
        sw.sync_run(20)
        st = sw.state()
        u, f, idx, ms = sw.local_stage(kind, history=10, maxiters=100, gtol=1e-5)
        xo = sw.get(_lib.FIELD_LOCAL_X)
        fo = sw.get(_lib.FIELD_LOCAL_F)
        its = sw.get(_lib.FIELD_LOCAL_ITERS)
    x0 = st["pbest"] if kind == "lbfgs" else st["x"]
    rx, rf, rit = orc.lbfgs(oprob, x0, history=10, maxiters=100, gtol=1e-5, broyden=(kind == "bfgs"))
    assert np.array_equal(fo, rf), f"max |df| {np.max(np.abs(fo - rf))}"
    assert np.array_equal(xo, rx)
    assert np.array_equal(its.astype(np.int32), rit)
    k = int(np.argmin(rf))
    assert idx == k and f == rf[k] and np.array_equal(u, rx[:, k])
    assert ms > 0


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_lbfgs_known_answers_through_solve(pps, orc, case):
    name, obj, u0, p, lb, ub, ans, pso_iters, local_iters = case
    D = len(u0)
    prob = pps.OptimizationProblem(pps.REGISTRY[{"rosen2": "rosenbrock", "rosen2_start": "rosenbrock",
                                                 "rosen2_box": "rosenbrock"}.get(name, name)],
                                   np.array(u0, np.float32), p or None,
                                   lb=None if lb is None else np.array(lb, np.float32),
                                   ub=None if ub is None else np.array(ub, np.float32))
    alg = pps.HybridPSO(pso=pps.ParallelSyncPSOKernel(64, gbest_from_position=True), local_opt=pps.SimpleLBFGS())
    sol = pps.solve(prob, alg, maxiters=pso_iters, local_maxiters=local_iters, abstol=1e-10, seed=0)
    ru, rf = hybrid_oracle(orc, obj, u0, p, lb, ub, pso_iters, local_iters)
    assert np.array_equal(sol.u, ru) and np.float32(sol.objective) == np.float32(rf)
    if name == "boundary_quadratic":
        assert sol.u[0] == pytest.approx(0.0, abs=1e-6) and sol.objective == pytest.approx(1.0, abs=1e-6)
    else:
        assert sol.objective < 1e-8
        if ans is not None:
            assert np.allclose(sol.u, ans, atol=1e-4)


def test_hybrid_config_small(pps):
    """The HybridPSO workload shape (10-D Rosenbrock / Ackley, bounds [-5, 5],
    PSO then L-BFGS m=10, Armijo 1e-4, <=100 iterations, gtol 1e-5) at 8192
    particles: the local stage reaches the global minimum."""
    for name, prm in (("rosenbrock", [1.0, 100.0]), ("ackley", [20.0, 0.2, 1.0])):
        D = 10
        prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm,
                                       lb=np.full(D, -5.0, np.float32), ub=np.full(D, 5.0, np.float32))
        alg = pps.HybridPSO(pso=pps.ParallelSyncPSOKernel(8192), local_opt=pps.SimpleLBFGS(history=10))
        sol = pps.solve(prob, alg, maxiters=200, local_maxiters=100, seed=1)
        assert np.isfinite(sol.objective) and np.all(np.isfinite(sol.u))
        assert np.all(sol.u >= -5) and np.all(sol.u <= 5)
        assert sol.objective < 1e-3, (name, sol.objective)


@pytest.mark.parametrize("obj,name,u0,prm", [
    (1, "rosenbrock", [-1.2, 1.0], [1.0, 100.0]),
    (0, "sphere", [0.5, -2.0, 3.0], []),
    (3, "ackley", [0.3, -0.2, 0.1, 0.05], [20.0, 0.2, 1.0]),
])
def test_standalone_bfgs_matches_oracle(pps, orc, obj, name, u0, prm):
    """solve(prob, BFGS()) (src/bfgs.jl:2-36): Broyden's method from u0 without
    bounds, 1000 iterations by default, bit-identical to the oracle's Broyden
    from the same point; objective = f(u, p)."""
    D = len(u0)
    u0 = np.asarray(u0, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], u0, prm or None)
    sol = pps.solve(prob, pps.BFGS())
    oprob = orc.OracleProblem(obj, D, None, None, params=prm)
    rx, rf, rit = orc.lbfgs(oprob, u0.reshape(D, 1), maxiters=1000, gtol=1e-5, broyden=True)
    assert np.array_equal(sol.u, rx[:, 0], equal_nan=True)
    want = np.float32(oprob.objective(rx[:, 0]))
    assert np.float32(sol.objective) == want or (np.isnan(sol.objective) and np.isnan(want))
    assert sol.stats.iterations == 1000
