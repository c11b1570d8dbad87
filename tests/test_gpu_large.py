"""Large swarms, where the oracle would take too long: size-independent
properties of the synchronous step (determinism, the global best is the
lowest-index argmin of the personal bests, bounds, monotone personal bests)
at 12.6 M particles with a ragged count, and the largest batched swarm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_large_ragged_swarm_properties(pps):
    n, D = 3 * (1 << 22) + 17, 3
    lb = np.full(D, -2.0, np.float32)
    ub = np.full(D, 2.0, np.float32)
    prob = pps.OptimizationProblem(pps.rosenbrock, np.zeros(D, np.float32), [1.0, 100.0], lb=lb, ub=ub)
    runs = []
    for _ in range(2):
        with pps.Swarm(prob, n, seed=77) as sw:
            sw.init()
            pc0 = sw.get(3)
            sw.sync_run(4)
            st = sw.state()
            g, gc, gi = sw.gbest()
            runs.append((st, g, gc, gi, pc0))
    (st, g, gc, gi, pc0), (st2, g2, gc2, gi2, _) = runs
    # deterministic: the same seed gives the same bits whatever the block schedule
    for k in ("x", "v", "pbest", "pcost", "cost"):
        assert np.array_equal(st[k], st2[k], equal_nan=True), k
    assert gi == gi2 and gc == gc2 and np.array_equal(g, g2)
    # the global best is the lowest-index argmin of the personal bests
    assert gi == int(np.argmin(st["pcost"])) and gc == st["pcost"].min()
    assert np.array_equal(g, st["pbest"][:, gi])
    # positions stay in the box; personal bests never worsen and bound the costs
    assert np.all(st["x"] >= lb[:, None]) and np.all(st["x"] <= ub[:, None])
    assert np.all(st["pcost"] <= pc0) and np.all(st["pcost"] <= st["cost"])


def test_largest_batched_swarm(pps):
    """65,536 particles (the batch limit) in a 1024-dim swarm beside a small one."""
    big = pps.OptimizationProblem(pps.sphere, np.zeros(1024, np.float32), lb=np.full(1024, -1, np.float32),
                                  ub=np.full(1024, 1, np.float32))
    small = pps.OptimizationProblem(pps.rastrigin, np.zeros(3, np.float32), [10.0],
                                    lb=np.full(3, -5.12, np.float32), ub=np.full(3, 5.12, np.float32))
    with pps.Batch() as b:
        b.add(big, 65536, maxiters=3, seed=1)
        b.add(small, 100, maxiters=50, seed=2)
        b.run()
        ub_, uc, ui = b.result(0)
        vs, vc, vi = b.result(1)
    for prob, n, it, seed, res in ((big, 65536, 3, 1, (ub_, uc, ui)), (small, 100, 50, 2, (vs, vc, vi))):
        with pps.Swarm(prob, n, seed=seed) as sw:
            sw.init()
            sw.sync_run(it)
            u, c, i = sw.gbest()
        assert i == res[2] and np.float32(c) == np.float32(res[1]) and np.array_equal(u, res[0])
