"""User objectives on the GPU (NVRTC-compiled with the library's kernels):
bit-exact against the oracle's C build of the same source every iteration,
bit-identical to the registered kernels where the source spells a registered
objective, through init, the sync / queue-lock steps, the captured-graph run
loop, constraints, point evaluation, solve() and the server."""
import numpy as np
import pytest

import user_sources as us
from test_constraints_oracle import CONS
from test_gpu_sync_parity import assert_state_equal

pytestmark = pytest.mark.gpu


def _box(D, lo, hi):
    return np.full(D, lo, np.float32), np.full(D, hi, np.float32)


def _pair(pps, orc, src, D, n, lo, hi, params, seed, data=None, cons=None, gpos=False):
    lb, ub = _box(D, lo, hi)
    f = pps.cuda_objective(src)
    prob = pps.OptimizationProblem(f, np.zeros(D, np.float32), params or None, lb=lb, ub=ub, data=data, cons=cons)
    oprob = orc.OracleProblem(0, D, lb, ub, params=params, cons=cons, user=orc.UserObjective(src), user_data=data)
    return pps.Swarm(prob, n, seed=seed, gbest_from_position=gpos), orc.OracleSwarm(oprob, n, seed)


def _polyfit_data():
    t = np.linspace(-2, 2, 64, dtype=np.float32)
    y = (0.5 - 2.0 * t + 3.0 * t * t + 0.05 * np.sin(7 * t)).astype(np.float32)
    return np.concatenate([t, y])


# (name, source, dim, n, lo, hi, params, iterations, data, gbest_from_position)
CASES = [
    ("rosenbrock-C1", us.ROSENBROCK, 3, 1000, -1.0, 10.0, [1.0, 100.0], 30, None, False),
    ("rosenbrock-C1-pos", us.ROSENBROCK, 3, 1000, -1.0, 10.0, [1.0, 100.0], 20, None, True),
    ("rastrigin-D100", us.RASTRIGIN, 100, 1024, -5.12, 5.12, [10.0], 8, None, False),
    ("polyfit-data", us.POLYFIT, 3, 777, -5.0, 5.0, [], 20, "poly", False),
    ("styblinski-sqrt", us.STYBLINSKI_SQRT, 9, 513, -5.0, 5.0, [], 20, None, False),
    ("griewank-D1", us.GRIEWANK, 1, 1, -600.0, 600.0, [], 10, None, False),
    ("griewank-ragged", us.GRIEWANK, 17, 4099, -600.0, 600.0, [], 10, None, False),
    # the fold of PPS_HAS_STREAM sources in the step kernel (no read-back)
    ("rastrigin-stream-D100", us.RASTRIGIN_STREAM, 100, 1024, -5.12, 5.12, [10.0], 8, None, False),
    ("rosenbrock-stream-C1-pos", us.ROSENBROCK_STREAM, 3, 1000, -1.0, 10.0, [1.0, 100.0], 20, None, True),
    ("rosenbrock-stream-D1", us.ROSENBROCK_STREAM, 1, 65, -1.0, 10.0, [1.0, 100.0], 10, None, False),
    ("weighted-stream-ragged", us.WEIGHTED_SPHERE_STREAM, 13, 4099, -5.0, 5.0, [], 12, "weights", False),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_user_sync_matches_oracle_every_iteration(pps, orc, case):
    _, src, D, n, lo, hi, prm, iters, data, gpos = case
    data = {"poly": _polyfit_data(), "weights": np.linspace(0.5, 4.5, D, dtype=np.float32)}.get(data)
    sw, ref = _pair(pps, orc, src, D, n, lo, hi, prm, seed=7, data=data, gpos=gpos)
    gsrc = orc.GBEST_FROM_POSITION if gpos else orc.GBEST_FROM_PBEST
    with sw:
        sw.init()
        ref.init(orc.SAMPLER_UNIFORM)
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1, gbest_source=gsrc)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        sw.sync_run(40, w=0.9, wdamp=0.99)  # graph replay
        ref.sync_run(40, w=0.9, wdamp=0.99, gbest_source=gsrc)
        assert_state_equal(sw, ref, "graph")


@pytest.mark.parametrize("src,name,D,n,lo,hi,prm", [
    (us.ROSENBROCK, "rosenbrock", 100, 4096, -5.12, 5.12, [1.0, 100.0]),
    (us.RASTRIGIN, "rastrigin", 100, 8192, -5.12, 5.12, [10.0]),
    (us.SHIFTED_SPHERE, "shifted_sphere", 6, 3000, -3.0, 3.0, [0.5, -1.0, 2.0]),
    (us.ROSENBROCK_STREAM, "rosenbrock", 100, 4096, -5.12, 5.12, [1.0, 100.0]),
    (us.RASTRIGIN_STREAM, "rastrigin", 100, 8192, -5.12, 5.12, [10.0]),
])
def test_user_source_reproduces_registered_kernel(pps, src, name, D, n, lo, hi, prm):
    """The NVRTC kernel over a source that spells a registered objective gives
    the registered (float4, software-pipelined) kernel's state bit for bit."""
    lb, ub = _box(D, lo, hi)
    reg = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm, lb=lb, ub=ub)
    usr = reg.remake(f=pps.cuda_objective(src))
    with pps.Swarm(reg, n, seed=3) as a, pps.Swarm(usr, n, seed=3) as b:
        a.init()
        b.init()
        a.sync_run(70)
        b.sync_run(70)
        sa, sb = a.state(), b.state()
        for k in ("x", "v", "pbest", "pcost", "cost"):
            assert np.array_equal(sa[k], sb[k]), k
        ua, ca, ia = a.gbest()
        ub_, cb, ib = b.gbest()
        assert ia == ib and np.float32(ca) == np.float32(cb) and np.array_equal(ua, ub_)


@pytest.mark.parametrize("src", [us.SHIFTED_SPHERE, us.SHIFTED_SPHERE_STREAM], ids=["read-back", "stream"])
def test_user_constrained_matches_registered_and_oracle(pps, orc, src):
    """test/constraints.jl's problem with f as a user source: the penalty
    path of the NVRTC kernel equals the registered one and the oracle."""
    lb, ub = np.zeros(2, np.float32), np.full(2, 2, np.float32)
    reg = pps.OptimizationProblem(pps.shifted_sphere, np.zeros(2, np.float32), [2.0, 1.0], lb=lb, ub=ub, cons=CONS)
    usr = reg.remake(f=pps.cuda_objective(src))
    oprob = orc.OracleProblem(0, 2, lb, ub, params=[2.0, 1.0], cons=CONS, user=orc.UserObjective(src))
    ref = orc.OracleSwarm(oprob, 1000, 5)
    with pps.Swarm(reg, 1000, seed=5) as a, pps.Swarm(usr, 1000, seed=5) as b:
        a.init()
        b.init()
        ref.init()
        assert_state_equal(b, ref, "init")
        for it in range(10):
            b.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(b, ref, f"iteration {it + 1}")
        b.queue_run(50)
        ref.sync_run(50)
        assert_state_equal(b, ref, "queue_run 50")
        a.sync_run(60)
        sa, sb = a.state(), b.state()
        for k in ("x", "v", "pbest", "pcost", "cost"):
            assert np.array_equal(sa[k], sb[k]), k


def test_user_unbounded_sampler(pps, orc):
    D, n = 4, 500
    u0 = np.array([0.0, 1.5, -2.0, 0.25], np.float32)
    src = us.ROSENBROCK
    prob = pps.OptimizationProblem(pps.cuda_objective(src), u0, [1.0, 100.0])
    oprob = orc.OracleProblem(0, D, None, None, u0=u0, params=[1.0, 100.0], user=orc.UserObjective(src))
    with pps.Swarm(prob, n, seed=2) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, n, 2).init(orc.SAMPLER_UNBOUNDED)
        assert_state_equal(sw, ref, "init")
        sw.sync_run(35)
        ref.sync_run(35)
        assert_state_equal(sw, ref, "after 35")


@pytest.mark.parametrize("src,D,data", [(us.STYBLINSKI_SQRT, 9, None), (us.POLYFIT, 3, "poly"),
                                        (us.GRIEWANK, 40, None)])
def test_user_eval_objective(pps, orc, src, D, data):
    data = _polyfit_data() if data == "poly" else None
    f = pps.cuda_objective(src)
    prob = pps.OptimizationProblem(f, np.zeros(D, np.float32), data=data)
    user = orc.UserObjective(src)
    x = np.random.default_rng(D).uniform(-5, 5, (1000, D)).astype(np.float32)
    got = pps.evaluate(prob, x)
    want = np.array([user(p, data=data) for p in x], np.float32)
    assert np.array_equal(got, want)


def test_user_solve_and_reference_threshold(pps):
    """solve() with a user Rosenbrock meets the reference's sync threshold
    (test/regression.jl:87: N = 3, 2000 particles, < 3e-3)."""
    D = 3
    lb, ub = _box(D, -1.0, 10.0)
    prob = pps.OptimizationProblem(pps.cuda_objective(us.ROSENBROCK), np.zeros(D, np.float32), [1.0, 100.0],
                                   lb=lb, ub=ub)
    sol = pps.solve(prob, pps.ParallelSyncPSOKernel(2000), maxiters=500, seed=42)
    assert sol.objective < 3e-3
    assert sol.original.shape == (2000, D)


@pytest.mark.parametrize("src,D,n,iters", [(us.RASTRIGIN, 20, 3000, 50), (us.POLYFIT, 3, 777, 80),
                                           (us.GRIEWANK, 1, 1, 10)])
def test_user_async_matches_oracle(pps, orc, src, D, n, iters):
    """ParallelPSOKernel(global_update=false) on a user objective: the
    in-kernel iteration loop with each particle's private global best, bit
    for bit against the oracle's async run, then a sync run after it."""
    data = _polyfit_data() if src == us.POLYFIT else None
    lo, hi = (-600.0, 600.0) if src == us.GRIEWANK else (-5.12, 5.12)
    sw, ref = _pair(pps, orc, src, D, n, lo, hi, [10.0] if src == us.RASTRIGIN else [], seed=6, data=data)
    with sw:
        sw.init()
        ref.init()
        sw.async_run(iters, w=0.9, wdamp=0.995)
        ref.async_run(iters, w=0.9, wdamp=0.995)
        assert_state_equal(sw, ref, "async")
        sw.sync_run(5)
        ref.sync_run(5)
        assert_state_equal(sw, ref, "sync after async")


def test_user_refused_paths(pps):
    prob = pps.OptimizationProblem(pps.cuda_objective(us.ROSENBROCK), np.zeros(3, np.float32), [1.0, 100.0],
                                   lb=np.full(3, -1, np.float32), ub=np.full(3, 10, np.float32))
    with pps.Swarm(prob, 256, seed=1) as sw:
        sw.init()
        sw.sync_run(3)
        with pytest.raises(pps.PPSError):
            sw.local_stage("lbfgs")
    with pps.Batch() as b:
        with pytest.raises(pps.PPSError):
            b.add(prob, 64, maxiters=5, seed=1)


def test_user_request_served_alone(pps):
    f = pps.cuda_objective(us.GRIEWANK)
    prob = pps.OptimizationProblem(f, np.zeros(10, np.float32), lb=np.full(10, -600, np.float32),
                                   ub=np.full(10, 600, np.float32))
    with pps.Server(memory_budget=64 << 20, max_launches=2) as srv:
        u, c, i, _ = srv.wait(srv.submit(prob, 300, maxiters=70, seed=9))
    with pps.Swarm(prob, 300, seed=9) as sw:
        sw.init()
        sw.sync_run(70)
        au, ac, ai = sw.gbest()
    assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


@pytest.mark.parametrize("kind,D,n", [("lbfgs", 10, 4096), ("bfgs", 10, 2048), ("lbfgs", 24, 777)])
def test_user_hybrid_local_stage(pps, orc, kind, D, n):
    """HybridPSO's local stage on a user objective with a gradient
    (PPS_HAS_GRADIENT): the NVRTC-compiled L-BFGS / Broyden kernels reproduce
    the registered Rosenbrock's local optima, values and iteration counts bit
    for bit (dim 24 takes the thread-local L-BFGS history), and the oracle's."""
    from parallelparticleswarms import _lib
    lb, ub = _box(D, -5.0, 5.0)
    reg = pps.OptimizationProblem(pps.rosenbrock, np.zeros(D, np.float32), [1.0, 100.0], lb=lb, ub=ub)
    usr = reg.remake(f=pps.cuda_objective(us.ROSENBROCK_GRAD))
    with pps.Swarm(reg, n, seed=3) as a, pps.Swarm(usr, n, seed=3) as b:
        a.init()
        b.init()
        a.sync_run(40)
        b.sync_run(40)
        ra = a.local_stage(kind, maxiters=60)
        rb = b.local_stage(kind, maxiters=60)
        assert ra[2] == rb[2] and np.float32(ra[1]) == np.float32(rb[1]) and np.array_equal(ra[0], rb[0])
        for field in (_lib.FIELD_LOCAL_X, _lib.FIELD_LOCAL_F, _lib.FIELD_LOCAL_ITERS):
            assert np.array_equal(a.get(field), b.get(field), equal_nan=True), field
        start = b.get(_lib.FIELD_PBEST if kind == "lbfgs" else _lib.FIELD_POSITION)
        got_x, got_it = b.get(_lib.FIELD_LOCAL_X), b.get(_lib.FIELD_LOCAL_ITERS)
    oprob = orc.OracleProblem(0, D, lb, ub, params=[1.0, 100.0], user=orc.UserObjective(us.ROSENBROCK_GRAD))
    xo, fo, its = orc.lbfgs(oprob, start, maxiters=60, broyden=(kind == "bfgs"))
    assert np.array_equal(xo, got_x) and np.array_equal(got_it.reshape(-1).astype(np.int32), its)

