"""The CUDA path against the committed golden vectors directly
(tests/golden/oracle_vectors.json): the swarm cases of
tests/golden/make_oracle_vectors.py run through the C ABI must give the same
state digests, global-best costs and indices bit for bit, without the oracle
being run."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
try:
    from make_oracle_vectors import CONS, bits, digest  # noqa: E402
finally:
    sys.path.pop(0)

WANT = json.loads((GOLDEN / "oracle_vectors.json").read_text())


def _box(D, lo, hi):
    return np.full(D, lo, np.float32), np.full(D, hi, np.float32)


def _cases(pps):
    L = pps._lib
    lb3, ub3 = _box(3, -1.0, 10.0)
    rosen3 = pps.OptimizationProblem(pps.rosenbrock, np.zeros(3, np.float32), [1.0, 100.0], lb=lb3, ub=ub3)
    lb, ub = _box(100, -5.12, 5.12)
    rast100 = pps.OptimizationProblem(pps.rastrigin, np.zeros(100, np.float32), [10.0], lb=lb, ub=ub)
    lb, ub = _box(20, -5.12, 5.12)
    rast20 = pps.OptimizationProblem(pps.rastrigin, np.zeros(20, np.float32), [10.0], lb=lb, ub=ub)
    lb, ub = _box(10, -32.0, 32.0)
    ack10 = pps.OptimizationProblem(pps.ackley, np.zeros(10, np.float32), [20.0, 0.2, 1.0], lb=lb, ub=ub)
    cons = pps.OptimizationProblem(pps.shifted_sphere, np.zeros(2, np.float32), [2.0, 1.0],
                                   lb=np.zeros(2, np.float32), ub=np.full(2, 2, np.float32), cons=CONS)
    lb, ub = _box(5, -5.12, 5.12)
    rast5 = pps.OptimizationProblem(pps.rastrigin, np.zeros(5, np.float32), [10.0], lb=lb, ub=ub)
    u0 = np.array([0.0, 1.5, -2.0, 0.25], np.float32)
    rosen4 = pps.OptimizationProblem(pps.rosenbrock, u0, [1.0, 100.0])
    # name: (problem, particles, seed, iterations, sampler, mode, gbest from position)
    return {
        "sync_rosenbrock_3d": (rosen3, 1000, 0, 20, L.SAMPLER_UNIFORM, "sync", False),
        "sync_rosenbrock_3d_gbest_from_position": (rosen3, 1000, 0, 20, L.SAMPLER_UNIFORM, "sync", True),
        "sync_rastrigin_100d": (rast100, 256, 7, 20, L.SAMPLER_UNIFORM, "sync", False),
        "async_rastrigin_20d": (rast20, 300, 3, 30, L.SAMPLER_UNIFORM, "async", False),
        "sync_ackley_10d": (ack10, 500, 5, 15, L.SAMPLER_UNIFORM, "sync", False),
        "sync_constrained_shifted_sphere": (cons, 1000, 5, 10, L.SAMPLER_UNIFORM, "sync", False),
        "init_lhs_rastrigin_5d": (rast5, 100, 9, 0, L.SAMPLER_LHS, "sync", False),
        "init_unbounded_rosenbrock_4d": (rosen4, 500, 4, 0, L.SAMPLER_UNBOUNDED, "sync", False),
    }


def test_cuda_path_reproduces_golden_vectors(pps):
    for name, (prob, n, seed, iters, sampler, mode, gpos) in _cases(pps).items():
        with pps.Swarm(prob, n, seed=seed, gbest_from_position=gpos) as sw:
            sw.init(sampler)
            if iters:
                run = sw.sync_run if mode == "sync" else sw.async_run
                run(iters, w=0.9, wdamp=0.99)
            st = sw.state()
            _, gcost, gidx = sw.gbest()
        got = {"state": digest(st["x"], st["v"], st["pbest"], st["pcost"], st["cost"]), "gcost": bits(gcost),
               "gidx": gidx}
        assert got == WANT[name], name
