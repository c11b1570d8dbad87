"""Synchronous PSO step on the GPU vs the oracle, iteration by iteration.

Contract: with the same Philox stream the CUDA kernels and the CPU
restatement perform the same binary32 operations, so positions, velocities,
personal bests, costs, the global-best index and vector agree bit for bit
(stronger than the 1e-5 relative the workload asks for; the relative error is
reported when they do not)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_INF = np.float32(np.inf)


def _max_rel(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    fin = np.isfinite(a) & np.isfinite(b)
    return float(np.max(np.abs(a - b)[fin] / np.maximum(np.abs(b)[fin], 1e-30))) if fin.any() else 0.0


def assert_state_equal(sw, ref, where):
    st = sw.state()
    for k in ("x", "v", "pbest", "pcost", "cost"):
        got, want = st[k], getattr(ref, k)
        assert np.array_equal(got, want, equal_nan=True), f"{where}: {k} differs (max rel {_max_rel(got, want):.3e})"
    u, gcost, gidx = sw.gbest()
    assert gidx == ref.gidx, f"{where}: gbest index {gidx} != {ref.gidx}"
    assert np.float32(gcost) == np.float32(ref.gcost) or (np.isnan(gcost) and np.isnan(ref.gcost))
    assert np.array_equal(u, ref.g), f"{where}: gbest vector differs"


# (objective id, name, dim, n, lb, ub, params, iters, gbest_from_position)
CASES = [
    (1, "rosenbrock", 3, 1000, -1.0, 10.0, [1.0, 100.0], 40, False),    # the CPU config, GPU semantics
    (1, "rosenbrock", 3, 1000, -1.0, 10.0, [1.0, 100.0], 40, True),     # CPU-backend gbest quirk
    (2, "rastrigin", 100, 2048, -5.12, 5.12, [10.0], 12, False),
    (1, "rosenbrock", 100, 1111, -5.12, 5.12, [1.0, 100.0], 12, False),
    (3, "ackley", 10, 4099, -5.0, 5.0, [20.0, 0.2, 1.0], 25, False),
    (0, "sphere", 7, 63, -3.0, 3.0, [], 30, False),
    (2, "rastrigin", 1, 1, -5.12, 5.12, [10.0], 10, False),              # a single particle, one dim
    (2, "rastrigin", 5, 65, -5.12, 5.12, [10.0], 10, False),             # ragged n, odd dim
    (16, "beale", 2, 300, -4.5, 4.5, [], 20, False),
    (18, "himmelblau", 2, 257, -5.0, 5.0, [], 20, False),
    (20, "boundary_quadratic", 1, 129, 0.0, 2.0, [], 20, False),
]


def _make(pps, orc, obj, name, D, n, lo, hi, prm, gpos, seed):
    lb = np.full(D, lo, np.float32)
    ub = np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None, lb=lb, ub=ub)
    oprob = orc.OracleProblem(obj, D, lb, ub, params=prm)
    sw = pps.Swarm(prob, n, seed=seed, gbest_from_position=gpos)
    ref = orc.OracleSwarm(oprob, n, seed)
    return sw, ref


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[1]}-D{c[2]}-n{c[3]}{'-pos' if c[8] else ''}")
def test_sync_matches_oracle_every_iteration(pps, orc, case):
    obj, name, D, n, lo, hi, prm, iters, gpos = case
    sw, ref = _make(pps, orc, obj, name, D, n, lo, hi, prm, gpos, seed=7)
    src = orc.GBEST_FROM_POSITION if gpos else orc.GBEST_FROM_PBEST
    with sw:
        sw.init()
        ref.init(orc.SAMPLER_UNIFORM)
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1, gbest_source=src)
            assert_state_equal(sw, ref, f"iteration {it + 1}")


@pytest.mark.parametrize("iters", [31, 32, 33, 100])
def test_sync_long_run_uses_graph_and_matches(pps, orc, iters):
    """maxiters >= 32 replays a captured CUDA graph of step launches."""
    sw, ref = _make(pps, orc, 2, "rastrigin", 20, 3000, -5.12, 5.12, [10.0], False, seed=11)
    with sw:
        sw.init()
        ref.init()
        sw.sync_run(iters, w=0.9, wdamp=0.99)
        ref.sync_run(iters, w=0.9, wdamp=0.99)
        assert_state_equal(sw, ref, f"after {iters}")
        # a second call continues the iteration counter and the random stream
        sw.sync_run(iters, w=0.9, wdamp=0.99)
        ref.sync_run(iters, w=0.9, wdamp=0.99)
        assert_state_equal(sw, ref, f"after 2x{iters}")


def test_unbounded_sampler_matches(pps, orc):
    D, n = 4, 777
    u0 = np.array([0.0, 1.5, -2.0, 0.25], np.float32)
    prob = pps.OptimizationProblem(pps.rosenbrock, u0, [1.0, 100.0])
    oprob = orc.OracleProblem(1, D, None, None, u0=u0, params=[1.0, 100.0])
    with pps.Swarm(prob, n, seed=5) as sw:
        sw.init()  # infinite bounds -> unbounded sampler (src/init.jl:102-106)
        ref = orc.OracleSwarm(oprob, n, 5).init(orc.SAMPLER_UNBOUNDED)
        assert_state_equal(sw, ref, "init")
        sw.sync_run(50)
        ref.sync_run(50)
        assert_state_equal(sw, ref, "after 50")


def test_queue_run_equals_sync_semantics(pps, orc):
    sw, ref = _make(pps, orc, 1, "rosenbrock", 4, 2000, -1.0, 10.0, [1.0, 100.0], True, seed=3)
    with sw:
        sw.init()
        ref.init()
        # queue-lock ignores the CPU-backend quirk: block bests are pbests
        sw.queue_run(64)
        ref.sync_run(64, gbest_source=orc.GBEST_FROM_PBEST)
        assert_state_equal(sw, ref, "queue 64")


def test_zero_iterations_is_a_no_op(pps, orc):
    sw, ref = _make(pps, orc, 0, "sphere", 3, 100, -1.0, 1.0, [], False, seed=1)
    with sw:
        sw.init()
        ref.init()
        sw.sync_run(0)
        assert_state_equal(sw, ref, "0 iterations")
        assert sw.info().iteration == 0


def test_state_roundtrip_set_get(pps, orc):
    sw, ref = _make(pps, orc, 2, "rastrigin", 6, 500, -5.12, 5.12, [10.0], False, seed=9)
    with sw:
        sw.init()
        ref.init()
        sw.sync_run(5)
        ref.sync_run(5)
        snap = sw.state()
        sw.sync_run(5)
        # restore the snapshot and rerun the same iterations: identical result
        from parallelparticleswarms import _lib
        for f, k in ((_lib.FIELD_POSITION, "x"), (_lib.FIELD_VELOCITY, "v"), (_lib.FIELD_PBEST, "pbest"),
                     (_lib.FIELD_PCOST, "pcost"), (_lib.FIELD_COST, "cost")):
            sw.set(f, snap[k])
            assert np.array_equal(sw.get(f), snap[k])
