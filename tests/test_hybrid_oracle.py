"""Pins of the oracle's HybridPSO local stage: the known answers of the
reference's L-BFGS tests (test/lbfgs.jl:38-72), re-run in Float32 on the CPU
restatement with the test's settings (ParallelSyncPSOKernel(64) on the CPU
backend, maxiters 50 / 20, local_maxiters 200 / 50, abstol 1e-10)."""
import numpy as np
import pytest

# name, objective id, u0, p, lb, ub, answer, pso iters, local iters (test/lbfgs.jl line)
CASES = [
    ("rosen2", 1, [0.0, 0.0], [1.0, 100.0], None, None, [1.0, 1.0], 50, 200),            # :40-42
    ("rosen2_start", 1, [-1.2, 1.0], [1.0, 100.0], None, None, [1.0, 1.0], 50, 200),     # :44-46
    ("rosen2_box", 1, [0.0, 0.0], [1.0, 100.0], [-2.0, -2.0], [2.0, 2.0], [1.0, 1.0], 50, 200),  # :48-51
    ("beale", 16, [1.0, 1.0], [], None, None, [3.0, 0.5], 50, 200),                      # :53-55
    ("booth", 17, [1.0, 1.0], [], None, None, [1.0, 3.0], 50, 200),                      # :57-59
    ("himmelblau", 18, [1.0, 1.0], [], None, None, None, 50, 200),                       # :61-62
    ("quadratic", 19, [4.0, 4.0], [1000.0], [-5.0, -5.0], [5.0, 5.0], [1.0, -2.0], 50, 200),  # :64-67
    ("boundary_quadratic", 20, [1.5], [], [0.0], [2.0], [0.0], 20, 50),                 # :69-75
]


def hybrid_oracle(orc, obj, u0, p, lb, ub, pso_iters, local_iters, seed=0, gtol=1e-10):
    D = len(u0)
    prob = orc.OracleProblem(obj, D, lb, ub, u0=u0, params=p)
    sw = orc.OracleSwarm(prob, 64, seed)
    sw.init(orc.SAMPLER_UNBOUNDED if lb is None else orc.SAMPLER_UNIFORM)
    sw.sync_run(pso_iters, gbest_source=orc.GBEST_FROM_POSITION)
    best_u, best_f = sw.g.copy(), prob.objective(sw.g)
    xo, fo, it = orc.lbfgs(prob, sw.pbest, history=10, maxiters=local_iters, gtol=gtol)
    k = int(np.argmin(fo))
    if fo[k] < best_f:
        best_u, best_f = xo[:, k], float(fo[k])
    return best_u, best_f


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_lbfgs_known_answers_on_oracle(orc, case):
    name, obj, u0, p, lb, ub, ans, pso_iters, local_iters = case
    u, f = hybrid_oracle(orc, obj, u0, p, lb, ub, pso_iters, local_iters)
    if name == "boundary_quadratic":
        assert u[0] == pytest.approx(0.0, abs=1e-6) and f == pytest.approx(1.0, abs=1e-6)
        return
    assert f < 1e-8
    if ans is not None:
        assert np.allclose(u, ans, atol=1e-4)
    if lb is not None:
        assert np.all(u >= np.array(lb)) and np.all(u <= np.array(ub))


def test_broyden_converges_on_quadratics(orc):
    """Broyden on grad f = 0 (src/hybrid.jl:33-45) finds stationary points."""
    prob = orc.OracleProblem(17, 2, [-10, -10], [10, 10], params=[])
    x0 = np.array([[0.0, 5.0, -3.0], [0.0, -2.0, 8.0]], np.float32)
    xo, fo, it = orc.lbfgs(prob, x0, maxiters=100, gtol=1e-5, broyden=True)
    assert np.allclose(xo, [[1.0] * 3, [3.0] * 3], atol=1e-3)
    assert np.all(fo < 1e-6)


def test_lbfgs_reduces_every_particle(orc):
    rng = np.random.default_rng(0)
    for obj, prm in ((1, [1.0, 100.0]), (3, [20.0, 0.2, 1.0])):
        D, n = 10, 64
        prob = orc.OracleProblem(obj, D, np.full(D, -5.0), np.full(D, 5.0), params=prm)
        x0 = rng.uniform(-5, 5, (D, n)).astype(np.float32)
        f0 = np.array([prob.objective(x0[:, i]) for i in range(n)])
        xo, fo, it = orc.lbfgs(prob, x0, maxiters=100, gtol=1e-5)
        assert np.all(fo <= f0)
        assert np.all(xo >= -5.0) and np.all(xo <= 5.0)
