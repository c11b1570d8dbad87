"""Async PSO (ParallelPSOKernel(global_update=false)) on the GPU vs the oracle.

The oracle sums the objective with the same lane slices as the kernel
(orc_async_lanes), so the final state is bit-identical."""
import numpy as np
import pytest

from test_gpu_sync_parity import assert_state_equal

pytestmark = pytest.mark.gpu

# (objective id, name, dim, n, lo, hi, params, iters)
CASES = [
    (1, "rosenbrock", 3, 1000, -1.0, 10.0, [1.0, 100.0], 100),
    (2, "rastrigin", 10, 513, -5.12, 5.12, [10.0], 80),
    (2, "rastrigin", 17, 300, -5.12, 5.12, [10.0], 60),    # 2 lanes
    (1, "rosenbrock", 33, 257, -5.0, 5.0, [1.0, 100.0], 60),  # 4 lanes, coupled dims across lanes
    (2, "rastrigin", 100, 1000, -5.12, 5.12, [10.0], 40),  # 8 lanes of 14 dims
    (1, "rosenbrock", 100, 999, -5.12, 5.12, [1.0, 100.0], 40),
    (3, "ackley", 64, 200, -5.0, 5.0, [20.0, 0.2, 1.0], 40),
    (0, "sphere", 1, 1, -1.0, 1.0, [], 20),
    (17, "booth", 2, 64, -10.0, 10.0, [], 50),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[1]}-D{c[2]}-n{c[3]}")
def test_async_matches_oracle(pps, orc, case):
    obj, name, D, n, lo, hi, prm, iters = case
    lb = np.full(D, lo, np.float32)
    ub = np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None, lb=lb, ub=ub)
    oprob = orc.OracleProblem(obj, D, lb, ub, params=prm)
    with pps.Swarm(prob, n, seed=21) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, n, 21).init()
        lanes, slice_ = orc.async_lanes(D)
        info = sw.info()
        assert (info.async_lanes, info.async_slice) == (lanes, slice_)
        sw.async_run(iters, w=0.7298, wdamp=0.995)
        ref.async_run(iters, w=0.7298, wdamp=0.995, lanes=lanes)
        assert_state_equal(sw, ref, f"async {iters}")
        # a second run starts from the published global best and continues the stream
        sw.async_run(iters // 2)
        ref.async_run(iters // 2, lanes=lanes)
        assert_state_equal(sw, ref, "async second run")


def test_async_then_sync_continue(pps, orc):
    D, n = 12, 800
    lb = np.full(D, -5.12, np.float32)
    ub = np.full(D, 5.12, np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), lb=lb, ub=ub)
    oprob = orc.OracleProblem(2, D, lb, ub, params=[10.0])
    with pps.Swarm(prob, n, seed=4) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, n, 4).init()
        sw.async_run(30)
        ref.async_run(30)
        sw.sync_run(30)
        ref.sync_run(30)
        assert_state_equal(sw, ref, "async 30 + sync 30")
