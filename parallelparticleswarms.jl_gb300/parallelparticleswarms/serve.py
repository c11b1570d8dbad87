"""Serving: problems submitted as they arrive, solved with continuous batching
(pps_serve_* in include/pps.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .problem import OptimizationProblem
from .swarm import C1_DEFAULT, C2_DEFAULT, W_DEFAULT, WDAMP_DEFAULT


class Server:
    """Owns a pps_server: a device arena of ``memory_budget`` bytes and a worker
    thread that packs admitted problems into batched launches."""

    def __init__(self, memory_budget: int = 8 << 30, max_launches: int = 8, max_pack: int = 512, threads: int = 256,
                 ppt: int = 1, tick_us: float = 200.0, single_min_n: int = 0, ode_single_min_n: int = 0):
        """``single_min_n``: requests with at least this many particles run as
        a swarm of their own with the multi-block step kernels (0: the
        library's default, 2048; negative: only MLP fits, which always do).
        ``ode_single_min_n``: the same threshold for ODE fits (0: follow
        ``single_min_n``; negative: ODE fits of any size are batched)."""
        self._lib = _lib.load()
        cfg = _lib.ServeConfig(int(memory_budget), int(max_launches), int(max_pack), int(threads), int(ppt),
                               float(tick_us), int(single_min_n), int(ode_single_min_n))
        self._h = ctypes.c_void_p()
        _lib.check(self._lib.pps_serve_start(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._dims: dict[int, int] = {}

    def submit(self, prob: OptimizationProblem, n: int, *, maxiters: int = 100, seed: int = 0, w: float = W_DEFAULT,
               wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT, c2: float = C2_DEFAULT) -> int:
        t = ctypes.c_uint64()
        pr = prob.to_c()
        _lib.check(self._lib.pps_serve_submit(self._h, ctypes.byref(pr), int(n), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                              int(maxiters), float(w), float(wdamp), float(c1), float(c2),
                                              ctypes.byref(t)))
        self._dims[t.value] = prob.dim
        return int(t.value)

    def _out(self, ticket):
        # an unknown ticket still reaches the library, which reports it
        u = np.empty(max(1, self._dims.get(ticket, 1024)), np.float32)
        return u, ctypes.c_float(), ctypes.c_int64(), ctypes.c_double()

    def poll(self, ticket: int):
        """(u, cost, idx, latency_ms) when done, else None."""
        u, c, i, lat = self._out(ticket)
        rc = self._lib.pps_serve_poll(self._h, ticket, _lib.fptr(u), ctypes.byref(c), ctypes.byref(i), ctypes.byref(lat))
        if rc == _lib.EBUSY:
            return None
        _lib.check(rc)
        u = u[: self._dims.pop(ticket)]
        return u, float(c.value), int(i.value), float(lat.value)

    def wait(self, ticket: int, timeout: float = 600.0):
        u, c, i, lat = self._out(ticket)
        _lib.check(self._lib.pps_serve_wait(self._h, ticket, _lib.fptr(u), ctypes.byref(c), ctypes.byref(i),
                                            ctypes.byref(lat), float(timeout)))
        u = u[: self._dims.pop(ticket)]
        return u, float(c.value), int(i.value), float(lat.value)

    def stats(self) -> dict:
        st = _lib.ServeStats()
        _lib.check(self._lib.pps_serve_stats_get(self._h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in _lib.ServeStats._fields_}

    def stop(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pps_serve_stop(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def mixed_request(rng: np.random.Generator, objectives=("rosenbrock", "rastrigin", "ackley", "lv", "mlp")):
    """One request of the served mixed stream: objective uniform over
    ``objectives``, dim ~ U{2..64} (an ODE or MLP fit has its own parameter
    count), particles ~ U{256..16384}, maxiters ~ U{100..2000}.  Returns
    (problem, n, maxiters, seed)."""
    from . import mlp, ode
    from .problem import REGISTRY

    kind = objectives[int(rng.integers(len(objectives)))]
    n = int(rng.integers(256, 16385))
    iters = int(rng.integers(100, 2001))
    seed = int(rng.integers(0, 2**63))
    if kind == "lv":
        prob, _ = ode.synthetic_fit("lv", int(rng.integers(0, 2**31)))
        return prob, n, iters, seed
    if kind == "mlp":
        data, _ = mlp.teacher_task(1024, seed=int(rng.integers(0, 2**31)))
        return mlp.mlp_problem(data), n, iters, seed
    D = int(rng.integers(2, 65))
    obj = REGISTRY[kind]
    lo = {"rosenbrock": -5.0, "rastrigin": -5.12, "ackley": -5.0}[kind]
    prob = OptimizationProblem(obj, np.zeros(D, np.float32), list(obj.default_params),
                               lb=np.full(D, lo, np.float32), ub=np.full(D, -lo, np.float32))
    return prob, n, iters, seed
