"""The constrained path (calc_penalty, src/utils.jl:320-372) on the CPU:
known penalty values, theta_default's steps at the binary32 neighbours of its
Float64 thresholds, the reference's constraint test on the oracle, and the C
ABI's checks of constrained problems (no GPU needed)."""
import ctypes

import numpy as np
import pytest

# test/constraints.jl:7-27: f = (x1 - 2)^2 + (x2 - 1)^2 on [0, 2]^2 with
#   -x1 + 2 x2 - 1 <= 0,  x1 - 2 x2 + 1 <= 0,  x1^2 / 4 + x2^2 - 1 <= 0
CONS = np.array([[-1, -1, 2, 0, 0], [1, 1, -2, 0, 0], [-1, 0, 0, 0.25, 1]], np.float32)


def _problem(orc):
    return orc.OracleProblem(7, 2, [0, 0], [2, 2], params=[2.0, 1.0], cons=CONS)


def test_penalty_known_values(orc):
    op = _problem(orc)
    # at (1, 1): q = (0, 0, 0.25): (10 + 10 + 100) + 100 * 0.25
    assert op.penalty([1, 1], 1.0) == 145.0
    # h = sqrt: the same point weighted by sqrt(4)
    assert op.penalty([1, 1], 4.0) == 290.0
    # no constraint violated by much: q = (0, 0.1, 0) at x = (0.3, 0.7)
    x = np.array([0.3, 0.7], np.float32)
    g = [np.float32(-1) + (np.float32(-1) * x[0] + np.float32(2) * x[1]),
         np.float32(1) + (x[0] + np.float32(-2) * x[1])]
    assert op.objective(x) == pytest.approx((0.3 - 2) ** 2 + (0.7 - 1) ** 2, rel=1e-6)
    assert np.isfinite(op.penalty(x, 3.0)) and g[0] > 0


@pytest.mark.parametrize("q,theta", [(0.0, 10.0), (np.nextafter(np.float32(0.001), np.float32(0)), 10.0),
                                     (np.float32(0.001), 20.0), (np.nextafter(np.float32(0.1), np.float32(0)), 20.0),
                                     (np.float32(0.1), 100.0), (np.float32(1.0), 100.0),
                                     (np.nextafter(np.float32(1.0), np.float32(2)), 300.0)])
def test_theta_steps_at_the_float64_thresholds(orc, q, theta):
    """theta_default compares a Float32 with the Float64 literals 0.001 and 0.1
    (src/utils.jl:320-330): 0.001f and 0.1f lie above them."""
    q = np.float32(q)
    op = orc.OracleProblem(0, 1, [-1], [1], cons=[[q, 0.0, 0.0]])
    pw = q if q < 1 else np.float32(q * q)
    assert op.penalty([0.0], 1.0) == np.float32(theta + np.float32(theta * pw))


def test_reference_constraint_test_on_the_oracle(orc):
    """test/constraints.jl:25-29: 1000 particles, 500 iterations,
    |1 - 2 u2 + u1| < 0.1."""
    sw = orc.OracleSwarm(_problem(orc), 1000, 1234).init()
    sw.sync_run(500)
    assert abs(1 - 2 * sw.g[1] + sw.g[0]) < 1e-1


def test_c_abi_checks_constrained_problems(pps):
    from parallelparticleswarms import _lib

    lib = _lib.load()
    x = np.zeros(2, np.float32)
    f = np.zeros(1, np.float32)
    base = pps.OptimizationProblem(pps.shifted_sphere, np.zeros(2, np.float32), [2.0, 1.0],
                                   lb=np.zeros(2, np.float32), ub=np.full(2, 2, np.float32), cons=CONS)
    pr = base.to_c()
    pr.ncons = 5
    assert lib.pps_eval_objective(ctypes.byref(pr), 1, _lib.fptr(x), _lib.fptr(f)) == _lib.EINVAL
    pr = base.to_c()
    pr.cons = ctypes.cast(None, _lib.c_float_p)
    assert lib.pps_eval_objective(ctypes.byref(pr), 1, _lib.fptr(x), _lib.fptr(f)) == _lib.EINVAL
    bad = base.remake(cons=np.where(CONS == 2, np.inf, CONS).astype(np.float32))
    pr = bad.to_c()
    assert lib.pps_eval_objective(ctypes.byref(pr), 1, _lib.fptr(x), _lib.fptr(f)) == _lib.EINVAL
    lv, _ = pps.ode.synthetic_fit("lv", 1)
    lvc = lv.remake(cons=np.zeros((1, 9), np.float32))
    pr = lvc.to_c()
    assert lib.pps_eval_objective(ctypes.byref(pr), 1, _lib.fptr(np.zeros(4, np.float32)),
                                  _lib.fptr(f)) == _lib.ENOTSUP
    with pytest.raises(pps.ArgumentError):
        base.remake(cons=np.zeros(4, np.float32))
