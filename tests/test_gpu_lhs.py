"""The Latin-hypercube init on the GPU: positions, costs and the initial
global best bit-identical to the oracle for registered objectives, ODE fits
and user objectives (then the sync run continues identically), the strata
property at 2^20 particles, and the reference's LHS regression cases through
solve()."""
import numpy as np
import pytest

import user_sources as us
from test_gpu_sync_parity import assert_state_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("obj,name,D,n,lo,hi,prm", [
    (1, "rosenbrock", 3, 1000, -1.0, 10.0, [1.0, 100.0]),
    (2, "rastrigin", 100, 4099, -5.12, 5.12, [10.0]),
    (3, "ackley", 10, 1, -5.0, 5.0, [20.0, 0.2, 1.0]),
    (0, "sphere", 7, 65, -3.0, 3.0, []),
])
def test_lhs_init_and_run_match_oracle(pps, orc, obj, name, D, n, lo, hi, prm):
    lb, ub = np.full(D, lo, np.float32), np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None, lb=lb, ub=ub)
    oprob = orc.OracleProblem(obj, D, lb, ub, params=prm)
    with pps.Swarm(prob, n, seed=11) as sw:
        sw.init(pps._lib.SAMPLER_LHS)
        ref = orc.OracleSwarm(oprob, n, 11).init(orc.SAMPLER_LHS)
        assert_state_equal(sw, ref, "lhs init")
        sw.sync_run(40)
        ref.sync_run(40)
        assert_state_equal(sw, ref, "after 40")


def test_lhs_user_objective_and_ode_fit(pps, orc):
    D, n = 4, 777
    lb, ub = np.full(D, -2.0, np.float32), np.full(D, 2.0, np.float32)
    prob = pps.OptimizationProblem(pps.cuda_objective(us.STYBLINSKI_SQRT), np.zeros(D, np.float32), lb=lb, ub=ub)
    oprob = orc.OracleProblem(0, D, lb, ub, user=orc.UserObjective(us.STYBLINSKI_SQRT))
    with pps.Swarm(prob, n, seed=4) as sw:
        sw.init(pps._lib.SAMPLER_LHS)
        ref = orc.OracleSwarm(oprob, n, 4).init(orc.SAMPLER_LHS)
        assert_state_equal(sw, ref, "user lhs init")
    fit, _ = pps.ode.synthetic_fit("lv", 1)
    with pps.Swarm(fit, 300, seed=2) as a, pps.Swarm(fit, 300, seed=2) as b:
        a.init(pps._lib.SAMPLER_LHS)
        b.init(pps._lib.SAMPLER_UNIFORM)
        xa = a.state()["x"]
        assert not np.array_equal(xa, b.state()["x"])
        lo, hi = fit.lb.astype(np.float64), fit.ub.astype(np.float64)
        for d in range(xa.shape[0]):
            strata = np.floor((xa[d] - lo[d]) / (hi[d] - lo[d]) * 300).astype(np.int64)
            assert len(np.unique(np.clip(strata, 0, 299))) >= 297  # one per stratum up to edge rounding


def test_lhs_large_swarm_matches_oracle(pps, orc):
    D, n = 4, 1 << 20
    lb, ub = np.full(D, -5.0, np.float32), np.full(D, 5.0, np.float32)
    prob = pps.OptimizationProblem(pps.sphere, np.zeros(D, np.float32), lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=6) as sw:
        sw.init(pps._lib.SAMPLER_LHS)
        x = sw.state()["x"]
    ref = orc.OracleSwarm(orc.OracleProblem(0, D, lb, ub), n, 6).init(orc.SAMPLER_LHS)
    assert np.array_equal(x, ref.state()["x"])


@pytest.mark.parametrize("N", [2, 3])
def test_reference_lhs_regression(pps, N):
    """test/regression.jl:53-58,71-76 through solve(): LatinHypercubeSample
    init, ParallelPSOKernel and ParallelSyncPSOKernel, 2000 particles, 500
    iterations, retcode Default; the sync threshold of the file (3e-3) holds."""
    prob = pps.OptimizationProblem(pps.rosenbrock, np.zeros(N, np.float32), [1.0, 100.0],
                                   lb=np.full(N, -1, np.float32), ub=np.full(N, 10, np.float32))
    for alg in (pps.ParallelPSOKernel(2000), pps.ParallelSyncPSOKernel(2000)):
        sol = pps.solve_(pps.init(prob, alg, sampler=pps.LatinHypercubeSample(), seed=123), maxiters=500)
        assert sol.retcode == "Default"
        assert sol.objective < 3e-3


def test_lhs_needs_finite_bounds(pps):
    prob = pps.OptimizationProblem(pps.sphere, np.zeros(2, np.float32), lb=np.array([-1, -np.inf], np.float32),
                                   ub=np.array([1, 1], np.float32))
    with pps.Swarm(prob, 16, seed=1) as sw:
        with pytest.raises(pps.ArgumentError):
            sw.init(pps._lib.SAMPLER_LHS)
