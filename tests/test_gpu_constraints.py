"""The constrained path on the GPU: init and the sync / queue-lock steps add
the reference's penalty (src/kernels.jl:28-36, src/utils.jl:320-372) to the
cost, bit-exact against the oracle every iteration; the reference's own
constraint test passes through solve()."""
import numpy as np
import pytest

from test_constraints_oracle import CONS
from test_gpu_sync_parity import assert_state_equal

pytestmark = pytest.mark.gpu


def _random_problem(pps, orc, D, ncons, seed):
    rng = np.random.default_rng(seed)
    cons = np.stack([pps.quadratic_constraint(D, c=rng.normal(), a=rng.normal(size=D), b=rng.uniform(0, 0.5, D))
                     for _ in range(ncons)])
    lb = np.full(D, -3.0, np.float32)
    ub = np.full(D, 3.0, np.float32)
    prm = list(rng.uniform(-1, 1, min(D, 8)).astype(np.float32))
    prob = pps.OptimizationProblem(pps.shifted_sphere, np.zeros(D, np.float32), prm, lb=lb, ub=ub, cons=cons)
    oprob = orc.OracleProblem(7, D, lb, ub, params=prm, cons=cons)
    return prob, oprob


@pytest.mark.parametrize("D,ncons,n,iters", [(2, 3, 1000, 30), (7, 4, 777, 20), (12, 1, 300, 25)])
def test_constrained_sync_matches_oracle_every_iteration(pps, orc, D, ncons, n, iters):
    if D == 2:
        lb, ub = np.zeros(2, np.float32), np.full(2, 2, np.float32)
        prob = pps.OptimizationProblem(pps.shifted_sphere, np.zeros(2, np.float32), [2.0, 1.0], lb=lb, ub=ub, cons=CONS)
        oprob = orc.OracleProblem(7, 2, lb, ub, params=[2.0, 1.0], cons=CONS)
    else:
        prob, oprob = _random_problem(pps, orc, D, ncons, seed=D)
    with pps.Swarm(prob, n, seed=5) as sw:
        ref = orc.OracleSwarm(oprob, n, 5)
        sw.init()
        ref.init(orc.SAMPLER_UNIFORM)
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        # the queue-lock entry point is the same synchronous iteration
        sw.queue_run(3)
        ref.sync_run(3)
        assert_state_equal(sw, ref, "queue_run")
        # a 40-iteration run replays a captured graph
        sw.sync_run(40)
        ref.sync_run(40)
        assert_state_equal(sw, ref, "graph")


def test_reference_constraint_test(pps):
    """test/constraints.jl:25-33 through solve(): ParallelSyncPSOKernel and
    ParallelPSOKernel (queue-lock), 1000 particles, 500 iterations."""
    prob = pps.OptimizationProblem(pps.shifted_sphere, np.ones(2, np.float32), [2.0, 1.0],
                                   lb=np.zeros(2, np.float32), ub=np.full(2, 2, np.float32), cons=CONS)
    for alg in (pps.ParallelSyncPSOKernel(1000), pps.ParallelPSOKernel(1000)):
        sol = pps.solve(prob, alg, maxiters=500, seed=1234)
        assert abs(1 - 2 * sol.u[1] + sol.u[0]) < 1e-1
        # sol.objective is prob.f(u, p), without the penalty (src/solve.jl:56)
        assert sol.objective == pytest.approx((sol.u[0] - 2) ** 2 + (sol.u[1] - 1) ** 2, rel=1e-5)


def test_constrained_async_and_batch_are_refused(pps):
    prob = pps.OptimizationProblem(pps.shifted_sphere, np.ones(2, np.float32), [2.0, 1.0],
                                   lb=np.zeros(2, np.float32), ub=np.full(2, 2, np.float32), cons=CONS)
    with pps.Swarm(prob, 64, seed=1) as sw:
        sw.init()
        with pytest.raises(pps.PPSError):
            sw.async_run(3)
    with pps.Batch() as b:
        with pytest.raises(pps.PPSError):
            b.add(prob, 64, maxiters=5, seed=1)


def test_constrained_request_served_alone(pps):
    prob = pps.OptimizationProblem(pps.shifted_sphere, np.ones(2, np.float32), [2.0, 1.0],
                                   lb=np.zeros(2, np.float32), ub=np.full(2, 2, np.float32), cons=CONS)
    with pps.Server(memory_budget=64 << 20, max_launches=2) as srv:
        u, c, i, _ = srv.wait(srv.submit(prob, 200, maxiters=30, seed=9))
    with pps.Swarm(prob, 200, seed=9) as sw:
        sw.init()
        sw.sync_run(30)
        au, ac, ai = sw.gbest()
    assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)
