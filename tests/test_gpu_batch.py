"""Batched swarms: every swarm's result equals its solve alone (bitwise), for
every block shape, and matches the oracle."""
import numpy as np
import pytest

from test_ode_oracle import oracle_ode_problem

pytestmark = pytest.mark.gpu


def _mixed(pps):
    rng = np.random.default_rng(42)
    cases = []
    specs = [("sphere", 3, 1, 5), ("rosenbrock", 3, 1000, 60), ("rastrigin", 17, 257, 40), ("ackley", 64, 100, 30),
             ("rastrigin", 100, 1500, 10), ("rosenbrock", 2, 37, 0), ("ackley", 5, 1, 25), ("sphere", 1, 64, 3),
             ("rosenbrock", 33, 513, 20), ("rastrigin", 2, 5000, 15),
             ("rastrigin", 8, 40000, 6)]  # split over a cluster of 16 CTAs
    for k, (name, D, n, iters) in enumerate(specs):
        prm = pps.REGISTRY[name].default_params
        lo = -5.12 if name == "rastrigin" else -5.0
        prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), list(prm) or None,
                                       lb=np.full(D, lo, np.float32), ub=np.full(D, -lo, np.float32))
        cases.append((prob, n, iters, 100 + k, float(rng.uniform(0.6, 0.9)), float(rng.choice([1.0, 0.99]))))
    for k, model in enumerate(("lv", "fhn", "lv", "lv")):
        prob, _ = pps.ode.synthetic_fit(model, 50 + k)
        cases.append((prob, (64, 33, 256, 4096)[k], (8, 4, 6, 3)[k], 200 + k, 0.7298, 1.0))
    return cases


def _alone(pps, prob, n, iters, seed, w, wdamp):
    with pps.Swarm(prob, n, seed=seed) as sw:
        sw.init()
        sw.sync_run(iters, w=w, wdamp=wdamp)
        return sw.gbest(), sw.state()


@pytest.mark.parametrize("shape", [(0, 0), (128, 1), (256, 2), (512, 1)])
def test_batch_equals_alone(pps, shape):
    cases = _mixed(pps)
    with pps.Batch() as b:
        slots = [b.add(p, n, maxiters=it, seed=s, w=w, wdamp=wd) for (p, n, it, s, w, wd) in cases]
        if shape != (0, 0):
            b.set_shape(*shape)
        ms = b.run()
        assert ms > 0
        info = b.info()
        assert info["swarms"] == len(cases) and info["threads"] in (128, 256, 512)
        for slot, (p, n, it, s, w, wd) in zip(slots, cases):
            (u, c, i), st = _alone(pps, p, n, it, s, w, wd)
            bu, bc, bi = b.result(slot)
            assert bi == i and np.float32(bc) == np.float32(c), (slot, p.f.name, bc, c)
            assert np.array_equal(bu, u), slot
            bst = b.state(slot)
            for k in ("x", "v", "pbest", "pcost", "cost"):
                assert np.array_equal(bst[k], st[k], equal_nan=True), (slot, k)


def test_batch_matches_oracle(pps, orc):
    cases = _mixed(pps)
    with pps.Batch() as b:
        slots = [b.add(p, n, maxiters=it, seed=s, w=w, wdamp=wd) for (p, n, it, s, w, wd) in cases]
        b.run()
        for slot, (p, n, it, s, w, wd) in zip(slots, cases):
            if p.f.id in (4, 5):
                op = oracle_ode_problem(orc, p)
            else:
                op = orc.OracleProblem(p.f.id, p.dim, p.lb, p.ub, params=p.p)
            ref = orc.OracleSwarm(op, n, s).init()
            ref.sync_run(it, w=w, wdamp=wd)
            u, c, i = b.result(slot)
            assert i == ref.gidx and np.array_equal(u, ref.g), slot


def test_same_alone_and_in_a_mix(pps):
    cases = _mixed(pps)
    target = cases[2]
    with pps.Batch() as solo:
        solo.add(target[0], target[1], maxiters=target[2], seed=target[3], w=target[4], wdamp=target[5])
        solo.run()
        r_solo = solo.result(0)
    with pps.Batch() as mix:
        for c in cases[:2]:
            mix.add(c[0], c[1], maxiters=c[2], seed=c[3], w=c[4], wdamp=c[5])
        slot = mix.add(target[0], target[1], maxiters=target[2], seed=target[3], w=target[4], wdamp=target[5])
        for c in cases[3:]:
            mix.add(c[0], c[1], maxiters=c[2], seed=c[3], w=c[4], wdamp=c[5])
        mix.run()
        r_mix = mix.result(slot)
    assert np.array_equal(r_solo[0], r_mix[0]) and r_solo[1] == r_mix[1] and r_solo[2] == r_mix[2]


def test_batch_argument_errors(pps):
    prob = pps.OptimizationProblem(pps.beale, np.zeros(2, np.float32))
    with pps.Batch() as b:
        with pytest.raises(pps.PPSError):
            b.add(prob, 10)
        with pytest.raises(pps.PPSError):
            b.run()  # empty
        p2 = pps.OptimizationProblem(pps.sphere, np.zeros(3, np.float32), lb=np.full(3, -1.0, np.float32),
                                     ub=np.full(3, 1.0, np.float32))
        with pytest.raises(pps.ArgumentError):
            b.add(p2, 0)
        with pytest.raises(pps.ArgumentError):
            b.set_shape(100, 1)
