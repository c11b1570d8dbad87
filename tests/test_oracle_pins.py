"""Pins of the CPU restatement (the oracle) before anything is compared to it.

The reference holds no bitwise golden vectors for this path.  What it does
hold is re-run here against the oracle, case by case with the same problem,
particle count, iteration count and threshold:
  - statistical thresholds under fixed seeds (test/regression.jl, test/gpu.jl);
  - the exact loss reduction of ode_pso (test/regression.jl:345-389);
  - the L-BFGS known answers (test/lbfgs.jl:38-72), tested in test_hybrid_oracle.py.
The random stream itself is pinned by the published Philox4x32-10 known-answer
vectors, structurally against numpy's Philox4x64-10 (same round function,
different word size) and, on the GPU, against cuRAND's Philox4_32_10
(tests/test_gpu_philox.py).  The math functions are pinned
against float64 numpy within stated ulp bounds.
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_philox_round_structure_matches_numpy(orc):
    # numpy.random.Philox is Philox4x64-10; its first block is produced from
    # counter 1 (numpy increments before generating).
    for key in ([0x123456789ABCDEF0, 0x0FEDCBA987654321], [0, 0], [2**64 - 1, 12345]):
        bg = np.random.Philox(key=np.array(key, dtype=np.uint64), counter=np.zeros(4, dtype=np.uint64))
        raw = [int(bg.random_raw()) for _ in range(8)]
        assert orc.philox4x64_10([1, 0, 0, 0], key) == raw[:4]
        assert orc.philox4x64_10([2, 0, 0, 0], key) == raw[4:]


def test_philox4x32_known_answers(orc):
    # the published known-answer vectors of Philox4x32-10 (Salmon, Moraes, Dror
    # and Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11; the
    # Random123 distribution's kat_vectors): counter, key -> output
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert orc.philox4x32_10(ctr, key) == want


def test_philox4x32_counter_sensitivity(orc):
    base = orc.philox4x32_10([0, 0, 0, 0], [0, 0])
    assert len(set(base)) == 4
    seen = {tuple(base)}
    for ctr in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]):
        out = tuple(orc.philox4x32_10(ctr, [0, 0]))
        assert out not in seen
        seen.add(out)


def test_philox_uniformity(orc):
    L = orc.load()
    vals = []
    for i in range(4096):
        o = orc.philox4x32_10([i, 7, 3, orc.TAG_STEP], [42, 0])
        vals += [L.orc_u01(v) for v in o]
    vals = np.array(vals)
    assert vals.min() >= 0.0 and vals.max() < 1.0
    assert abs(vals.mean() - 0.5) < 0.01
    hist, _ = np.histogram(vals, bins=16, range=(0, 1))
    chi2 = (((hist - len(vals) / 16) ** 2) / (len(vals) / 16)).sum()
    assert chi2 < 40.0  # 15 dof, p ~ 5e-4


def _ulp(ref):
    return np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)


def test_cos_polynomial_is_the_fit():
    """The compiled polynomial of cos(2 pi x) is the minimax fit of
    cospi_coefficients.py rounded to binary32, with relative error < 0.1 ulp."""
    import cospi_coefficients as cc

    fitted = [float(np.float32(v)) for v in cc.fit()]
    assert fitted == [float.fromhex(h) for h in cc.COMPILED]
    assert cc.max_rel_error([float.fromhex(h) for h in cc.COMPILED]) < 0.1 * 2.0 ** -24


def test_cos_sin_exp_accuracy(orc):
    L = orc.load()
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-6, 6, 20000), rng.uniform(-1e4, 1e4, 2000),
                         np.linspace(-1, 1, 4001)]).astype(np.float32)
    c = np.array([L.orc_cos2pi(float(x)) for x in xs])
    s = np.array([L.orc_sin2pi(float(x)) for x in xs])
    x64 = xs.astype(np.float64)
    rc, rs = np.cos(2 * np.pi * x64), np.sin(2 * np.pi * x64)
    assert np.max(np.abs(c - rc)) < 1.2e-7 and np.max(np.abs(s - rs)) < 1.2e-7
    m = np.abs(rc) > 1e-3
    assert np.max(np.abs(c - rc)[m] / _ulp(rc[m])) <= 2.0
    # the exact zeros of cos(2 pi x) at odd multiples of 1/4, signs of +-1 at the integers
    q = np.array([L.orc_cos2pi(float(v)) for v in (0.25, 0.75, -1.25, 2.0, -3.0, 0.5, 1e7, 3e6 + 0.5)])
    assert np.array_equal(q[:3], [0.0, 0.0, 0.0]) and np.array_equal(q[3:], [1.0, 1.0, -1.0, 1.0, -1.0])
    ex = np.concatenate([rng.uniform(-87, 88.7, 20000), np.linspace(-5, 5, 2001)]).astype(np.float32)
    e = np.array([L.orc_exp(float(x)) for x in ex])
    re = np.exp(ex.astype(np.float64))
    assert np.max(np.abs(e - re) / _ulp(re)) <= 1.0
    assert L.orc_exp(100.0) == np.inf and L.orc_exp(-100.0) == 0.0
    assert np.isnan(L.orc_cos2pi(float("inf")))


def test_objectives_match_definitions(orc):
    rng = np.random.default_rng(1)
    for D in (1, 2, 3, 10, 100):
        x = rng.uniform(-5, 5, D).astype(np.float32)
        x64 = x.astype(np.float64)
        # Rosenbrock (test/regression.jl:12-18)
        p = orc.OracleProblem(1, D, params=[1.0, 100.0])
        ref = sum(100 * (x64[i + 1] - x64[i] ** 2) ** 2 + (1 - x64[i]) ** 2 for i in range(D - 1))
        assert p.objective(x) == pytest.approx(ref, rel=1e-5, abs=1e-6)
        # Rastrigin 10D + sum(x^2 - 10 cos 2 pi x)
        p = orc.OracleProblem(2, D, params=[10.0])
        ref = 10 * D + np.sum(x64 ** 2 - 10 * np.cos(2 * np.pi * x64))
        assert p.objective(x) == pytest.approx(ref, rel=1e-5, abs=1e-4)
        # Ackley a=20, b=0.2, c=2 pi
        p = orc.OracleProblem(3, D, params=[20.0, 0.2, 1.0])
        ref = -20 * np.exp(-0.2 * np.sqrt(np.mean(x64 ** 2))) - np.exp(np.mean(np.cos(2 * np.pi * x64))) + 20 + np.e
        assert p.objective(x) == pytest.approx(ref, rel=1e-5, abs=1e-5)
        # lane-sliced summation differs from the sequential one by rounding only
        for lanes in (2, 4, 8):
            p = orc.OracleProblem(2, D, params=[10.0])
            assert p.objective(x, lanes) == pytest.approx(p.objective(x, 1), rel=1e-5, abs=1e-4)


def test_gradients_match_finite_differences(orc):
    rng = np.random.default_rng(2)
    cases = [(1, 10, [1.0, 100.0]), (2, 10, [10.0]), (3, 10, [20.0, 0.2, 1.0]), (0, 5, []),
             (16, 2, []), (17, 2, []), (18, 2, []), (19, 2, [1000.0]), (20, 1, [])]
    for obj, D, prm in cases:
        p = orc.OracleProblem(obj, D, params=prm)
        x = rng.uniform(-2, 2, D).astype(np.float32)
        f, g = p.objective_grad(x)
        h = 1e-3
        for d in range(D):
            xp, xm = x.astype(np.float64), x.astype(np.float64)
            xp = xp.copy(); xm = xm.copy()
            xp[d] += h; xm[d] -= h
            fd = (p.objective(xp.astype(np.float32)) - p.objective(xm.astype(np.float32))) / (2 * h)
            assert g[d] == pytest.approx(fd, rel=2e-2, abs=2e-2 * max(1.0, abs(f)) ** 0.5), (obj, d)


def _rosen_swarm(orc, D, n, lb, ub, seed, sampler):
    prob = orc.OracleProblem(1, D, lb, ub, params=[1.0, 100.0])
    return orc.OracleSwarm(prob, n, seed).init(sampler)


def _reference_threshold_cases():
    return json.loads((GOLDEN / "reference_thresholds.json").read_text())["cases"]


@pytest.mark.parametrize("case", _reference_threshold_cases(), ids=lambda c: c["id"])
def test_reference_threshold(orc, case):
    """The reference's own statistical tests, re-run on the oracle."""
    D, n, iters = case["dim"], case["particles"], case["maxiters"]
    lb = None if case["lb"] is None else np.full(D, float(case["lb"]), np.float32)
    ub = None if case["ub"] is None else np.full(D, float(case["ub"]), np.float32)
    unbounded = lb is None or not np.isfinite(lb).all()
    sampler = orc.SAMPLER_UNBOUNDED if unbounded else orc.SAMPLER_UNIFORM
    sw = _rosen_swarm(orc, D, n, lb, ub, case["seed"], sampler)
    f_u0 = sw.prob.objective(np.zeros(D, np.float32))
    if case["algorithm"] == "async":
        sw.async_run(iters)
    else:
        src = orc.GBEST_FROM_POSITION if case.get("cpu_backend") else orc.GBEST_FROM_PBEST
        sw.sync_run(iters, gbest_source=src)
    obj = sw.prob.objective(sw.g)
    assert obj < f_u0
    if case["threshold"] is not None:
        assert obj < case["threshold"], (case["id"], obj)


def test_reduce_losses_exact(orc):
    """test/regression.jl:345-357 and :378-389: data [1,2] at m=5 save points,
    n=7 particles of zeros -> every loss is exactly 5*(1+4) = 25."""
    m, n = 5, 7
    data = np.tile(np.array([1.0, 2.0], np.float32), (m, 1))
    us = np.zeros((n, m, 2), np.float32)
    losses = orc.reduce_losses(data, us)
    expected = ((data[None] - us) ** 2).sum(axis=2).sum(axis=1)
    assert np.array_equal(losses, expected.astype(np.float32))
    assert np.all(losses == 25.0)
