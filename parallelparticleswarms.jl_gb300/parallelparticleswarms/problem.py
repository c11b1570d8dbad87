"""OptimizationProblem and the registry of device objectives.

The reference builds ``OptimizationProblem(f, u0, p; lb, ub)`` (SciMLBase) with
an arbitrary Julia function ``f(x, p)`` that its kernels compile in
(src/kernels.jl:33).  Through a C ABI the objective is chosen from the
engine's registry; the objects below name the registry entries and carry
their default parameters.  They are markers, not Python callables: objective
values are always computed on the GPU (``evaluate`` below).  Any other
objective is given as CUDA C source (``cuda_objective``), which the library
compiles at run time into its own kernels.

A plain Python callable ``f(x, p)`` is accepted only for algorithms that bring
their own loop through the ``PSOAlgorithm`` / ``pso_solve`` interface
(src/algorithms.jl:1-28, src/solve.jl:69-87); every device path (the swarm
kernels, batches, the server, ``evaluate``) refuses it with ``ArgumentError``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _lib


@dataclass(frozen=True)
class Objective:
    name: str
    id: int
    default_params: tuple = ()
    max_dim: int | None = None
    source: str | None = field(default=None, repr=False, compare=False)

    def __repr__(self) -> str:
        return f"<objective {self.name}>"


sphere = Objective("sphere", 0)
rosenbrock = Objective("rosenbrock", 1, (1.0, 100.0))
rastrigin = Objective("rastrigin", 2, (10.0,))
ackley = Objective("ackley", 3, (20.0, 0.2, 1.0))
lotka_volterra_fit = Objective("lotka_volterra_fit", 4)
fitzhugh_nagumo_fit = Objective("fitzhugh_nagumo_fit", 5)
mlp_regression = Objective("mlp_regression", 6)
# sum (x_i - p_i)^2: the objective of the reference's constraint test (test/constraints.jl:7)
shifted_sphere = Objective("shifted_sphere", 7)
# closed-form objectives of test/lbfgs.jl:20-26
beale = Objective("beale", 16, (), 2)
booth = Objective("booth", 17, (), 2)
himmelblau = Objective("himmelblau", 18, (), 2)
quadratic = Objective("quadratic", 19, (1.0,), 2)
boundary_quadratic = Objective("boundary_quadratic", 20, (), 1)

REGISTRY = {o.name: o for o in (sphere, rosenbrock, rastrigin, ackley, lotka_volterra_fit,
                               fitzhugh_nagumo_fit, mlp_regression, shifted_sphere, beale, booth, himmelblau,
                               quadratic, boundary_quadratic)}


def cuda_objective(source: str, name: str = "user", default_params=()) -> Objective:
    """An objective given as CUDA C source, the counterpart of the arbitrary
    ``f(x, p)`` the reference compiles into its kernels (src/kernels.jl:33).

    The source defines ``PPS_DEVICE float pps_objective(pps_point x, int dim,
    const float* p, const float* data, long long ndata)``: ``x[d]`` is the
    point's coordinate d, ``p`` the problem's parameters (8 floats, zero past
    the given ones), ``data`` the problem's ``data`` on the device.  NVRTC
    compiles it (``pps_objective_register``) with the library's init, step
    and evaluation kernels; ``pps_exp``, ``pps_cos2pi`` and ``pps_sin2pi`` are
    the library's exp(x), cos(2 pi x) and sin(2 pi x).  Compile errors raise
    ArgumentError with the compiler's log.  Runs with ParallelSyncPSOKernel,
    ParallelPSOKernel (both global_update modes), ``evaluate`` and
    ``Server``; with HybridPSO when the source also defines PPS_HAS_GRADIENT
    and ``PPS_DEVICE float pps_gradient(pps_point x, int dim, const float* p,
    const float* data, long long ndata, float* g)`` (g = grad f, returns f);
    batches do not take it.  A source that defines PPS_HAS_STREAM also gives
    f as a fold over the coordinates (``pps_stream`` with
    ``pps_stream_start`` / ``pps_stream_add`` / ``pps_stream_finish``, equal
    to ``pps_objective`` bit for bit), which the synchronous step evaluates in
    registers instead of reading the new position back.
    """
    oid = ctypes.c_int32()
    _lib.check(_lib.load().pps_objective_register(source.encode(), ctypes.byref(oid)))
    return Objective(name, int(oid.value), tuple(float(v) for v in default_params), source=source)


def quadratic_constraint(dim: int, c: float = 0.0, a=None, b=None) -> np.ndarray:
    """One constraint g(x) = c + sum_i a_i x_i + b_i x_i^2 <= 0 as a row (c, a, b)
    of an OptimizationProblem's ``cons``.  This is the registered form of the
    reference's ``OptimizationFunction(f; cons)`` with ``ucons = 0``: the
    engine takes no Python or Julia callable."""
    row = np.zeros(1 + 2 * dim, np.float32)
    row[0] = c
    if a is not None:
        row[1:1 + dim] = np.asarray(a, np.float32).reshape(dim)
    if b is not None:
        row[1 + dim:] = np.asarray(b, np.float32).reshape(dim)
    return row


def _f32(a, n=None):
    if a is None:
        return None
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    if n is not None and arr.size != n:
        raise _lib.ArgumentError(_lib.EINVAL, f"expected {n} values, got {arr.size}")
    return arr


@dataclass
class OptimizationProblem:
    """``OptimizationProblem(f, u0, p; lb, ub)``.

    ``lb``/``ub`` of ``None`` mean unbounded (src/utils.jl:310-318).  ``data``
    carries an objective's observations (ODE fits) or sample set (MLP).
    ``cons`` holds up to 4 constraints g_k(x) <= 0 as rows (c_k, a_k, b_k) of
    g_k(x) = c_k + a_k . x + b_k . x^2 (see ``quadratic_constraint``); they
    enter the cost through the reference's penalty (src/utils.jl:320-372).
    """

    f: Objective | Callable
    u0: np.ndarray
    p: np.ndarray | None = None
    lb: np.ndarray | None = None
    ub: np.ndarray | None = None
    data: np.ndarray | None = None
    cons: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        if isinstance(self.f, str):
            self.f = REGISTRY[self.f]
        if not isinstance(self.f, Objective) and not callable(self.f):
            raise _lib.ArgumentError(_lib.EINVAL, "f must be a registered objective (see problem.REGISTRY), a "
                                                  "cuda_objective, or a callable f(x, p) for a pso_solve algorithm")
        self.u0 = _f32(self.u0)
        self.dim = int(self.u0.size)
        if self.p is None and self.on_device:
            self.p = np.asarray(self.f.default_params, dtype=np.float32) if self.f.default_params else None
        self.p = _f32(self.p)
        self.lb = _f32(self.lb, self.dim) if self.lb is not None else None
        self.ub = _f32(self.ub, self.dim) if self.ub is not None else None
        self.data = _f32(self.data)
        if self.cons is not None:
            c = np.ascontiguousarray(np.asarray(self.cons, dtype=np.float32))
            if c.size % (1 + 2 * self.dim):
                raise _lib.ArgumentError(_lib.EINVAL, f"cons rows have 1 + 2 dim = {1 + 2 * self.dim} values")
            self.cons = c.reshape(-1, 1 + 2 * self.dim)

    @property
    def on_device(self) -> bool:
        """True when f is one of the engine's objectives (registered or CUDA source)."""
        return isinstance(self.f, Objective)

    def require_device_objective(self) -> None:
        if not self.on_device:
            raise _lib.ArgumentError(_lib.EINVAL, "a Python callable f(x, p) cannot run on the device: use a "
                                                  "registered objective or cuda_objective(source)")

    def remake(self, **kw) -> "OptimizationProblem":
        args = dict(f=self.f, u0=self.u0, p=self.p, lb=self.lb, ub=self.ub, data=self.data, cons=self.cons)
        args.update(kw)
        return OptimizationProblem(**args)

    def to_c(self) -> _lib.Problem:
        """C struct view; the numpy buffers stay referenced by this problem."""
        self.require_device_objective()
        pr = _lib.Problem()
        pr.objective = self.f.id
        pr.dim = self.dim
        pr.lb = _lib.fptr(self.lb)
        pr.ub = _lib.fptr(self.ub)
        pr.u0 = _lib.fptr(self.u0)
        pr.params = _lib.fptr(self.p)
        pr.nparams = 0 if self.p is None else int(self.p.size)
        pr.data = _lib.fptr(self.data)
        pr.ndata = 0 if self.data is None else int(self.data.size)
        pr.ncons = 0 if self.cons is None else int(self.cons.shape[0])
        pr.cons = _lib.fptr(self.cons)
        return pr


def evaluate(prob: OptimizationProblem, x) -> np.ndarray:
    """Objective values at points ``x`` (shape (npoints, dim) or (dim,)) on the GPU."""
    prob.require_device_objective()
    x = np.asarray(x, dtype=np.float32)
    single = x.ndim == 1
    pts = x.reshape(-1, prob.dim)
    soa = np.ascontiguousarray(pts.T)
    out = np.empty(pts.shape[0], dtype=np.float32)
    pr = prob.to_c()
    _lib.check(_lib.load().pps_eval_objective(ctypes.byref(pr), pts.shape[0], _lib.fptr(soa), _lib.fptr(out)))
    return out[0] if single else out
