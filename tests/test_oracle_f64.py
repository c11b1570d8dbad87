"""The C oracle against an independent float64 restatement (oracle/pso_f64.py).

Every GPU parity test compares against the C oracle, so a misreading of the
reference shared by the oracle and the kernels would pass everywhere.  The
float64 restatement is written apart from the oracle (numpy, vectorised over
particles, textbook arithmetic: pso_cpu_ref.jl:57-72 and src/kernels.jl:1-26,
the synchronous global best of src/lowerlevel_solve.jl) and shares only the
random numbers, which it takes from the oracle's export.  The two differ only
by binary32 vs float64 rounding, so:

  - per iteration, before chaotic amplification sets in (first 5
    iterations): positions and velocities agree within 1e-5 relative, the
    relative error taken against max(|value|, 1) (coordinates near zero carry
    the absolute rounding of the binary32 update, ~1e-7, that a pure relative
    measure would blow up), and the global-best index is the same;
  - final global-best objectives over 32 seeds agree within 1e-4 relative
    (|a - b| <= 1e-4 |b| + 1e-6: the absolute 1e-6 covers minima at zero,
    where the binary32 cost of a converged swarm is 0 or ~1e-12 and float64's
    ~1e-17)."""
import numpy as np
import pytest

import pps_oracle as orc
import pso_f64 as f64

# (name, oracle id, dim, n, lo, hi, params, global-best rule)
C1 = ("rosenbrock", 1, 3, 1000, -1.0, 10.0, [1.0, 100.0], f64.GBEST_FROM_POSITION)   # the CPU config
C2 = ("rastrigin", 2, 100, 2048, -5.12, 5.12, [10.0], f64.GBEST_FROM_PBEST)          # the large config's shape
ACKLEY = ("ackley", 3, 10, 4096, -5.0, 5.0, [20.0, 0.2, 1.0], f64.GBEST_FROM_PBEST)


def _pair(case, seed, n=None):
    name, oid, D, n0, lo, hi, prm, _ = case
    n = n or n0
    lb, ub = np.full(D, lo, np.float32), np.full(D, hi, np.float32)
    ref = orc.OracleSwarm(orc.OracleProblem(oid, D, lb, ub, params=prm), n, seed).init()
    s = f64.F64Swarm(name, D, n, lb, ub, prm, seed).init()
    return ref, s


def _rel_unit(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def test_draws_are_the_oracles():
    """The exported draws are the ones the oracle's init consumed."""
    _, _, D, n, lo, hi, prm, _ = C2
    ref, _ = _pair(C2, 3, n=256)
    u = f64.init_draws(3, 256, D)
    x = (u * np.float32(hi - lo)) + np.float32(lo)
    assert np.array_equal(x.astype(np.float32), ref.x)


@pytest.mark.parametrize("case", [C1, C2, ACKLEY], ids=["C1-rosenbrock3", "rastrigin100", "ackley10"])
def test_per_iteration_within_1e5(case):
    src = case[7]
    ref, s = _pair(case, 0)
    assert ref.gidx == s.gidx
    assert _rel_unit(ref.x, s.x) <= 1e-6
    for it in range(5):
        ref.sync_run(1, gbest_source=src)
        s.sync_run(1, gbest_source=src)
        ex, ev = _rel_unit(ref.x, s.x), _rel_unit(ref.v, s.v)
        assert ex <= 1e-5 and ev <= 1e-5, f"iteration {it + 1}: x {ex:.2e} v {ev:.2e}"
        assert ref.gidx == s.gidx, f"iteration {it + 1}: global best {ref.gidx} vs {s.gidx}"
        assert abs(ref.gcost - s.gcost) <= 1e-5 * max(abs(s.gcost), 1.0)


@pytest.mark.parametrize("case,iters", [(C1, 500), (C2, 30)], ids=["C1-500it", "rastrigin100-30it"])
def test_final_objectives_over_32_seeds(case, iters):
    src = case[7]
    n = 1000 if case is C1 else 512
    worst = 0.0
    for seed in range(32):
        ref, s = _pair(case, seed, n=n)
        ref.sync_run(iters, gbest_source=src)
        s.sync_run(iters, gbest_source=src)
        a, b = float(ref.gcost), float(s.gcost)
        assert abs(a - b) <= 1e-4 * abs(b) + 1e-6, f"seed {seed}: {a} vs {b}"
        worst = max(worst, abs(a - b) / max(abs(b), 1e-30))
    print(f"worst relative difference of the final objective: {worst:.2e}")
