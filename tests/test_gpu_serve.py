"""The request server: continuous batching keeps every result equal to the
problem's solve alone; admission respects the memory budget."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(pps, prob, n, iters, seed):
    with pps.Swarm(prob, n, seed=seed) as sw:
        sw.init()
        sw.sync_run(iters)
        return sw.gbest()


NO_MLP = ("rosenbrock", "rastrigin", "ackley", "lv")


def _stream(pps, count, seed=0, small=True, objectives=None):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        prob, n, iters, s = (pps.serve.mixed_request(rng) if objectives is None
                             else pps.serve.mixed_request(rng, objectives))
        if small:  # keep the test short: scale the draws down
            n = max(16, n // 64)
            iters = max(5, iters // 40)
        out.append((prob, n, iters, s))
    return out


def test_each_result_same_alone_and_in_the_mix(pps):
    reqs = _stream(pps, 40)
    with pps.Server(memory_budget=1 << 30, max_launches=4, max_pack=16, tick_us=100.0) as srv:
        tickets = []
        for k, (prob, n, iters, s) in enumerate(reqs):
            tickets.append(srv.submit(prob, n, maxiters=iters, seed=s))
            if k % 7 == 3:
                time.sleep(0.002)  # arrivals while earlier launches run
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["launches"] >= 2
    for (prob, n, iters, s), (u, c, i, lat) in zip(reqs, results):
        au, ac, ai = _alone(pps, prob, n, iters, s)
        assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)
        assert lat > 0


def test_memory_bound_admission_queues_then_completes(pps):
    """A budget that fits about two requests at a time: the rest wait in the
    queue and are admitted as memory frees up."""
    reqs = _stream(pps, 12, seed=3, objectives=NO_MLP)
    budget = 600 << 10  # the largest scaled request needs about 200 KiB
    with pps.Server(memory_budget=budget, max_launches=8, max_pack=64, tick_us=0.0) as srv:
        tickets = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
        out = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == 12
    assert st["arena_peak_bytes"] <= budget
    assert st["launches"] >= 3  # the budget forced several admissions
    assert all(np.isfinite(c) for (_, c, _, _) in out)


def test_mlp_fits_served_beside_batched_requests(pps):
    """MLP fits run as swarms of their own on launch slots, concurrently with
    batched launches; each result equals the fit solved alone."""
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(12):
        kind = ("mlp",) if k % 3 == 0 else NO_MLP
        prob, n, iters, s = pps.serve.mixed_request(rng, kind)
        reqs.append((prob, max(16, n // 16), max(5, iters // 50), s))
    assert sum(p.f.name == "mlp_regression" for p, _, _, _ in reqs) == 4
    with pps.Server(memory_budget=1 << 30, max_launches=4, max_pack=16, tick_us=50.0) as srv:
        tickets = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
        results = [srv.wait(t) for t in tickets]
    for (prob, n, iters, s), (u, c, i, lat) in zip(reqs, results):
        au, ac, ai = _alone(pps, prob, n, iters, s)
        assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


def test_large_requests_run_as_swarms_of_their_own(pps):
    """Requests at or above single_min_n particles take the multi-block step
    kernels of a plain solve on a launch slot, the others the batched kernel;
    both kinds of result equal the problem solved alone."""
    reqs = _stream(pps, 16, seed=9, objectives=NO_MLP)
    assert any(n >= 128 for _, n, _, _ in reqs) and any(n < 128 for _, n, _, _ in reqs)
    with pps.Server(memory_budget=1 << 30, max_launches=6, max_pack=16, tick_us=50.0, single_min_n=128) as srv:
        tickets = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
        results = [srv.wait(t) for t in tickets]
    for (prob, n, iters, s), (u, c, i, lat) in zip(reqs, results):
        au, ac, ai = _alone(pps, prob, n, iters, s)
        assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


def test_ode_fits_routed_by_their_own_threshold(pps):
    """ode_single_min_n routes ODE fits apart from the other requests: with
    single_min_n = -1 every separable request is batched whatever its size,
    while ODE fits of at least 64 particles run as swarms of their own (their
    RK4 step packed two particles per thread, as for every swarm the server
    runs) and smaller ones are batched; every result equals its solve alone."""
    reqs = _stream(pps, 20, seed=13, objectives=NO_MLP)
    for k in range(4):
        prob, _ = pps.ode.synthetic_fit("lv" if k % 2 == 0 else "fhn", 70 + k)
        reqs.append((prob, (40, 64, 200, 129)[k], (3, 4, 2, 3)[k], 300 + k))
    with pps.Server(memory_budget=1 << 30, max_launches=6, max_pack=8, tick_us=50.0, single_min_n=-1,
                    ode_single_min_n=64) as srv:
        tickets = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
        results = [srv.wait(t) for t in tickets]
    for (prob, n, iters, s), (u, c, i, lat) in zip(reqs, results):
        au, ac, ai = _alone(pps, prob, n, iters, s)
        assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


def test_poll_and_errors(pps):
    reqs = _stream(pps, 1, seed=5, objectives=NO_MLP)
    prob, n, iters, s = reqs[0]
    with pps.Server(memory_budget=16 << 20) as srv:
        t = srv.submit(prob, n, maxiters=iters, seed=s)
        res = None
        for _ in range(20000):
            res = srv.poll(t)
            if res is not None:
                break
            time.sleep(0.0005)
        assert res is not None
        with pytest.raises(pps.PPSError):
            srv.poll(t)  # released
        huge = pps.OptimizationProblem(pps.sphere, np.zeros(64, np.float32), lb=np.full(64, -1, np.float32),
                                       ub=np.full(64, 1, np.float32))
        with pytest.raises(pps.PPSError, match="more than the serving arena"):
            srv.submit(huge, 60000)  # 46 MB of state, more than the 16 MiB arena
        with pytest.raises(pps.ArgumentError):
            srv.submit(prob, 0)
