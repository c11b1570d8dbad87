"""An independent float64 restatement of the synchronous PSO, in numpy.

TEST INFRASTRUCTURE ONLY (imported by tests/): a second restatement of the
reference's particle update, written apart from the C oracle, that pins the
C oracle's binary32 arithmetic against the textbook algorithm computed in
float64.  It shares only the random numbers: the uniform draws come from the
oracle's export (orc_init_draws / orc_step_draws), so the two runs see the
same r1, r2 and initial positions and differ only in the arithmetic.

Restated (file:line of the reference):
  - the update, pso_cpu_ref.jl:57-66 and src/kernels.jl:1-26:
      v = w v + c1 r1 (pbest - x) + c2 r2 (g - x);  x = min(max(x + v, lb), ub)
    (velocity not clamped), cost = f(x), personal best on strict <
    (pso_cpu_ref.jl:70-72, src/kernels.jl:21-24);
  - the synchronous global best: after every particle has moved, the argmin
    of the personal-best costs, lowest index first (src/kernels.jl:156-171,
    src/lowerlevel_solve.jl:23-33), its vector the winner's personal best,
    or with the CPU backend's rule its current position
    (src/lowerlevel_solve.jl:59-60);
  - init, src/utils.jl:57-84 and src/init.jl:38-54: x = u (ub - lb) + lb,
    v = 0, personal best = x, global best = argmin;
  - w damped by wdamp after each iteration (pso_cpu_ref.jl:78).
pso_cpu_ref.jl itself updates the global best inside the particle loop
(:74-77), a threaded race in its PSO and particle order in serial_PSO; the
synchronous kernels, which the oracle and the CUDA path follow, update it
once per iteration, so that is what is restated here.

Objectives in float64: Rosenbrock (test/regression.jl:12-18 with p), Rastrigin
and Ackley (the workload's formulas, numpy's cos / exp), sphere.
"""
from __future__ import annotations

import ctypes

import numpy as np

import pps_oracle as orc

GBEST_FROM_PBEST, GBEST_FROM_POSITION = 0, 1


def _draw_fns():
    L = orc.load()
    fp = ctypes.POINTER(ctypes.c_float)
    L.orc_init_draws.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, fp]
    L.orc_step_draws.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint32,
                                 fp, fp]
    return L


def init_draws(seed: int, n: int, dim: int) -> np.ndarray:
    u = np.empty((dim, n), np.float32)
    _draw_fns().orc_init_draws(seed, 0, n, dim, orc.fp(u))
    return u


def step_draws(seed: int, n: int, dim: int, t: int):
    r1 = np.empty((dim, n), np.float32)
    r2 = np.empty((dim, n), np.float32)
    _draw_fns().orc_step_draws(seed, 0, n, dim, t, orc.fp(r1), orc.fp(r2))
    return r1, r2


def objective(name: str, x: np.ndarray, p) -> np.ndarray:
    """f at the columns of x (dim, n), float64."""
    x = np.asarray(x, np.float64)
    if name == "sphere":
        return np.sum(x * x, axis=0)
    if name == "rosenbrock":
        p1, p2 = float(p[0]), float(p[1])
        return np.sum(p2 * (x[1:] - x[:-1] ** 2) ** 2 + (p1 - x[:-1]) ** 2, axis=0)
    if name == "rastrigin":
        A = float(p[0])
        return A * x.shape[0] + np.sum(x * x - A * np.cos(2.0 * np.pi * x), axis=0)
    if name == "ackley":
        a, b, k = float(p[0]), float(p[1]), float(p[2])
        D = x.shape[0]
        return (-a * np.exp(-b * np.sqrt(np.sum(x * x, axis=0) / D))
                - np.exp(np.sum(np.cos(2.0 * np.pi * k * x), axis=0) / D) + a + np.e)
    raise ValueError(name)


class F64Swarm:
    """(dim, n) float64 state stepped synchronously."""

    def __init__(self, name: str, dim: int, n: int, lb, ub, params, seed: int):
        self.name, self.dim, self.n, self.seed = name, int(dim), int(n), int(seed)
        self.lb = np.asarray(lb, np.float64).reshape(-1, 1)
        self.ub = np.asarray(ub, np.float64).reshape(-1, 1)
        self.p = list(params)
        self.t = 0

    def init(self) -> "F64Swarm":
        u = init_draws(self.seed, self.n, self.dim).astype(np.float64)
        self.x = u * (self.ub - self.lb) + self.lb
        self.v = np.zeros_like(self.x)
        self.pbest = self.x.copy()
        self.cost = objective(self.name, self.x, self.p)
        self.pcost = self.cost.copy()
        self._select(GBEST_FROM_PBEST)
        self.t = 0
        return self

    def _select(self, source: int) -> None:
        self.gidx = int(np.argmin(self.pcost))  # the first index of the minimum
        self.gcost = float(self.pcost[self.gidx])
        self.g = (self.x if source == GBEST_FROM_POSITION else self.pbest)[:, self.gidx].copy()

    def sync_run(self, iters: int, w=0.7298, wdamp=1.0, c1=1.4962, c2=1.4962, gbest_source=GBEST_FROM_PBEST):
        for _ in range(int(iters)):
            r1, r2 = step_draws(self.seed, self.n, self.dim, self.t)
            r1, r2 = r1.astype(np.float64), r2.astype(np.float64)
            g = self.g.reshape(-1, 1)
            self.v = w * self.v + c1 * r1 * (self.pbest - self.x) + c2 * r2 * (g - self.x)
            self.x = np.minimum(np.maximum(self.x + self.v, self.lb), self.ub)
            self.cost = objective(self.name, self.x, self.p)
            better = self.cost < self.pcost
            self.pcost = np.where(better, self.cost, self.pcost)
            self.pbest = np.where(better, self.x, self.pbest)
            self._select(gbest_source)
            w = w * wdamp
            self.t += 1
        return w
