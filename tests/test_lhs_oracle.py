"""The Latin-hypercube sampler (init(...; sampler = LatinHypercubeSample()),
src/init.jl:15-34) on the oracle: every dim deals each of the n strata to
exactly one particle, positions fall inside their stratum, dims and seeds
give different permutations, and the reference's LHS regression cases
(test/regression.jl:53-58,71-76) meet their thresholds."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 1000, 4097, 65536])
def test_strata_are_a_permutation(orc, n):
    for d in (0, 1, 7):
        s = np.array([orc.lhs_stratum(i, n, d, 42) for i in range(n)])
        assert np.array_equal(np.sort(s), np.arange(n)), (n, d)


def test_permutations_differ_by_dim_and_seed(orc):
    n = 4096
    a = np.array([orc.lhs_stratum(i, n, 0, 1) for i in range(n)])
    b = np.array([orc.lhs_stratum(i, n, 1, 1) for i in range(n)])
    c = np.array([orc.lhs_stratum(i, n, 0, 2) for i in range(n)])
    assert (a != b).mean() > 0.99 and (a != c).mean() > 0.99
    assert (a != np.arange(n)).mean() > 0.99
    # no long runs of consecutive strata: the permutation mixes
    assert np.abs(np.diff(a)).mean() > n / 8


def test_positions_fill_every_stratum(orc):
    D, n = 5, 3000
    lb = np.array([-1.0, 0.0, -5.0, 2.0, -0.5], np.float32)
    ub = np.array([1.0, 10.0, 5.0, 3.0, 0.5], np.float32)
    prob = orc.OracleProblem(0, D, lb, ub)
    sw = orc.OracleSwarm(prob, n, 9).init(orc.SAMPLER_LHS)
    x = sw.state()["x"]
    for d in range(D):
        strata = np.array([orc.lhs_stratum(i, n, d, 9) for i in range(n)])
        t = (x[d].astype(np.float64) - lb[d]) / (ub[d] - lb[d]) * n
        # each position lies in its stratum (up to one float rounding at the edges)
        assert np.all(t >= strata - 1e-3) and np.all(t <= strata + 1 + 1e-3)
        assert np.all((x[d] >= lb[d]) & (x[d] <= ub[d]))


@pytest.mark.parametrize("N", [2, 3])
def test_reference_lhs_regression(orc, N):
    """test/regression.jl:53-58,71-76: init with LatinHypercubeSample, then
    500 iterations, N-D Rosenbrock p = [1, 100] on [-1, 10], 2000 particles:
    the run converges (the reference checks retcode; the sync bound of the
    same file, 3e-3, holds)."""
    prob = orc.OracleProblem(1, N, np.full(N, -1, np.float32), np.full(N, 10, np.float32), params=[1.0, 100.0])
    sw = orc.OracleSwarm(prob, 2000, 3).init(orc.SAMPLER_LHS)
    sw.sync_run(500)
    assert sw.gcost < 3e-3
