"""ctypes wrapper of the CPU restatement (oracle/_build/libpps_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference leg as the checker; the product package
never imports it.  See pps_oracle.h for what is restated and the reference
file:line each part follows.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# PPS_ORACLE_BUILD=fast loads the timing-only build (-O3, fused multiply-adds:
# different bits), which only the CPU baseline's fast-build figure uses
LIB_PATH = HERE / "_build" / ("libpps_oracle_fast.so" if os.environ.get("PPS_ORACLE_BUILD") == "fast"
                              else "libpps_oracle.so")

TAG_INIT = 0x494E4954
TAG_STEP = 0x50534F31
SAMPLER_UNIFORM, SAMPLER_UNBOUNDED, SAMPLER_LHS = 0, 1, 2
GBEST_FROM_PBEST, GBEST_FROM_POSITION = 0, 1
ODE_LV, ODE_FHN = 0, 1
ODE_RK4, ODE_TSIT5, ODE_TSIT5_ADAPTIVE = 0, 1, 2

_fp = ctypes.POINTER(ctypes.c_float)


class OdeFit(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("nparams", ctypes.c_int32), ("u0", ctypes.c_float * 2),
                ("dt", ctypes.c_float), ("nsteps", ctypes.c_int32), ("save_every", ctypes.c_int32),
                ("nsaves", ctypes.c_int32), ("data", _fp), ("fixed", ctypes.c_float * 4),
                ("method", ctypes.c_int32), ("save_dt", ctypes.c_float), ("rtol", ctypes.c_float),
                ("atol", ctypes.c_float)]


USER_FN = ctypes.CFUNCTYPE(ctypes.c_float, _fp, ctypes.c_int, _fp, _fp, ctypes.c_longlong)
USER_GRAD = ctypes.CFUNCTYPE(ctypes.c_float, _fp, ctypes.c_int, _fp, _fp, ctypes.c_longlong, _fp)
OBJ_USER = 256


class Problem(ctypes.Structure):
    _fields_ = [("objective", ctypes.c_int32), ("dim", ctypes.c_int32), ("lb", _fp), ("ub", _fp),
                ("u0", _fp), ("params", ctypes.c_float * 8), ("nparams", ctypes.c_int32),
                ("ode", ctypes.POINTER(OdeFit)), ("mlp_data", _fp), ("mlp_samples", ctypes.c_int32),
                ("ncons", ctypes.c_int32), ("cons", _fp),
                ("user_fn", USER_FN), ("user_data", _fp), ("user_ndata", ctypes.c_int64),
                ("user_grad", USER_GRAD)]


class SwarmC(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("dim", ctypes.c_int32), ("x", _fp), ("v", _fp), ("pbest", _fp),
                ("pcost", _fp), ("cost", _fp), ("g", _fp), ("gcost", ctypes.c_float), ("gidx", ctypes.c_int64),
                ("first", ctypes.c_int64), ("nglobal", ctypes.c_int64)]


class LbfgsOpts(ctypes.Structure):
    _fields_ = [("history", ctypes.c_int32), ("maxiters", ctypes.c_int32), ("armijo_c1", ctypes.c_float),
                ("gtol", ctypes.c_float), ("max_backtracks", ctypes.c_int32)]


_lib = None


def build() -> Path:
    """Compile the restatement with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.orc_u01.restype = ctypes.c_float
        L.orc_u01.argtypes = [ctypes.c_uint32]
        for name in ("orc_cos2pi", "orc_sin2pi", "orc_exp"):
            getattr(L, name).restype = ctypes.c_float
            getattr(L, name).argtypes = [ctypes.c_float]
        L.orc_objective.restype = ctypes.c_float
        L.orc_objective.argtypes = [ctypes.POINTER(Problem), _fp, ctypes.c_int64, ctypes.c_int32]
        L.orc_penalty.restype = ctypes.c_float
        L.orc_penalty.argtypes = [ctypes.POINTER(Problem), _fp, ctypes.c_int64, ctypes.c_float]
        L.orc_objective_grad.restype = ctypes.c_float
        L.orc_objective_grad.argtypes = [ctypes.POINTER(Problem), _fp, _fp]
        L.orc_init.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(SwarmC), ctypes.c_uint64, ctypes.c_int32]
        L.orc_select_gbest.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(SwarmC), ctypes.c_int32]
        L.orc_sync_run.restype = ctypes.c_float
        L.orc_sync_run.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(SwarmC), ctypes.c_uint64,
                                   ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_int32]
        L.orc_async_run.restype = ctypes.c_float
        L.orc_async_run.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(SwarmC), ctypes.c_uint64,
                                    ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_int32]
        L.orc_async_lanes.restype = ctypes.c_int32
        L.orc_async_lanes.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.orc_argmin_key.restype = ctypes.c_uint64
        L.orc_argmin_key.argtypes = [ctypes.c_float, ctypes.c_uint32]
        L.orc_lhs_stratum.restype = ctypes.c_uint32
        L.orc_lhs_stratum.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
        for name in ("orc_lbfgs", "orc_broyden"):
            getattr(L, name).argtypes = [ctypes.POINTER(Problem), ctypes.c_int64, _fp, ctypes.POINTER(LbfgsOpts),
                                         _fp, _fp, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]
        L.orc_ode_loss.restype = ctypes.c_float
        L.orc_ode_loss.argtypes = [ctypes.POINTER(OdeFit), _fp]
        L.orc_ode_loss_adaptive.restype = ctypes.c_float
        L.orc_ode_loss_adaptive.argtypes = [ctypes.POINTER(OdeFit), _fp, ctypes.POINTER(ctypes.c_int32)]
        L.orc_log.restype = ctypes.c_float
        L.orc_log.argtypes = [ctypes.c_float]
        L.orc_ode_solve.argtypes = [ctypes.POINTER(OdeFit), _fp, _fp]
        L.orc_reduce_losses.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _fp, _fp, _fp]
        L.orc_mlp_loss.restype = ctypes.c_double
        L.orc_mlp_loss.argtypes = [_fp, _fp, _fp, ctypes.c_int32]
        L.orc_bf16_round.restype = ctypes.c_float
        L.orc_bf16_round.argtypes = [ctypes.c_float]
        _lib = L
    return _lib


def lhs_stratum(i: int, n: int, d: int, seed: int) -> int:
    """The Latin-hypercube stratum of particle i (< n) in dim d."""
    return int(load().orc_lhs_stratum(i, n, d, seed))


def fp(a: np.ndarray):
    return a.ctypes.data_as(_fp)


def philox4x32_10(ctr, key) -> list[int]:
    L = load()
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


def philox4x64_10(ctr, key) -> list[int]:
    L = load()
    c = (ctypes.c_uint64 * 4)(*ctr)
    k = (ctypes.c_uint64 * 2)(*key)
    o = (ctypes.c_uint64 * 4)()
    L.orc_philox4x64_10(c, k, o)
    return list(o)


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class OracleProblem:
    """orc_problem over numpy buffers (objective ids are include/pps.h's)."""

    def __init__(self, objective: int, dim: int, lb=None, ub=None, u0=None, params=(), ode=None, mlp_data=None,
                 cons=None, user=None, user_data=None):
        self.dim = int(dim)
        self.lb = np.ascontiguousarray(np.full(dim, -np.inf, np.float32) if lb is None else np.asarray(lb, np.float32))
        self.ub = np.ascontiguousarray(np.full(dim, np.inf, np.float32) if ub is None else np.asarray(ub, np.float32))
        self.u0 = np.ascontiguousarray(np.zeros(dim, np.float32) if u0 is None else np.asarray(u0, np.float32))
        self.c = Problem()
        self.c.objective = int(objective)
        self.c.dim = self.dim
        self.c.lb, self.c.ub, self.c.u0 = fp(self.lb), fp(self.ub), fp(self.u0)
        params = [] if params is None else list(np.asarray(params, np.float32).reshape(-1))
        for k, v in enumerate(params):
            self.c.params[k] = float(v)
        self.c.nparams = len(params)
        self.ode = ode
        if ode is not None:
            self.c.ode = ctypes.pointer(ode.c)
        self.cons = None
        if cons is not None:  # (ncons, 1 + 2 dim): c_k, a_k, b_k of g_k(x) = c_k + a_k . x + b_k . x^2 <= 0
            self.cons = np.ascontiguousarray(np.asarray(cons, np.float32).reshape(-1, 1 + 2 * self.dim))
            self.c.ncons = self.cons.shape[0]
            self.c.cons = fp(self.cons)
        self.user = user  # UserObjective: objective is OBJ_USER, f is its C build
        self.user_data = None
        if user is not None:
            self.c.objective = OBJ_USER
            self.c.user_fn = user.fn
            if user.grad is not None:
                self.c.user_grad = user.grad
            if user_data is not None:
                self.user_data = np.ascontiguousarray(np.asarray(user_data, np.float32).reshape(-1))
                self.c.user_data = fp(self.user_data)
                self.c.user_ndata = self.user_data.size
        self.mlp_data = None
        if mlp_data is not None:  # S x 16 samples followed by S targets
            self.mlp_data = np.ascontiguousarray(np.asarray(mlp_data, np.float32).reshape(-1))
            self.c.mlp_data = fp(self.mlp_data)
            self.c.mlp_samples = self.mlp_data.size // 17

    def objective(self, x, lanes: int = 1) -> float:
        x = np.ascontiguousarray(np.asarray(x, np.float32))
        return float(load().orc_objective(ctypes.byref(self.c), fp(x), 1, lanes))

    def penalty(self, x, iter: float) -> float:
        x = np.ascontiguousarray(np.asarray(x, np.float32))
        return float(load().orc_penalty(ctypes.byref(self.c), fp(x), 1, float(iter)))

    def objective_grad(self, x):
        x = np.ascontiguousarray(np.asarray(x, np.float32))
        g = np.empty_like(x)
        f = load().orc_objective_grad(ctypes.byref(self.c), fp(x), fp(g))
        return float(f), g


class OracleOdeFit:
    def __init__(self, model: int, nparams: int, u0, dt: float, nsteps: int, save_every: int, data,
                 fixed=(0.0, 0.0, 0.0, 0.0), method: int = 0, save_dt: float = 0.0, rtol: float = 0.0,
                 atol: float = 0.0):
        self.data = np.ascontiguousarray(np.asarray(data, np.float32).reshape(-1, 2))
        self.c = OdeFit()
        self.c.model, self.c.nparams = int(model), int(nparams)
        self.c.u0[0], self.c.u0[1] = float(u0[0]), float(u0[1])
        self.c.dt, self.c.nsteps, self.c.save_every = float(dt), int(nsteps), int(save_every)
        self.c.nsaves = int(self.data.shape[0])
        self.c.data = fp(self.data)
        for k, v in enumerate(fixed):
            self.c.fixed[k] = float(v)
        self.c.method, self.c.save_dt = int(method), float(save_dt)
        self.c.rtol, self.c.atol = float(rtol), float(atol)

    def loss(self, p) -> float:
        p = np.ascontiguousarray(np.asarray(p, np.float32))
        return float(load().orc_ode_loss(ctypes.byref(self.c), fp(p)))

    def loss_adaptive(self, p):
        """(loss, steps taken) of the adaptive Tsit5 fit."""
        p = np.ascontiguousarray(np.asarray(p, np.float32))
        n = ctypes.c_int32()
        f = load().orc_ode_loss_adaptive(ctypes.byref(self.c), fp(p), ctypes.byref(n))
        return float(f), int(n.value)

    def solve(self, p) -> np.ndarray:
        p = np.ascontiguousarray(np.asarray(p, np.float32))
        out = np.empty((self.c.nsaves, 2), np.float32)
        load().orc_ode_solve(ctypes.byref(self.c), fp(p), fp(out))
        return out


class OracleSwarm:
    """SoA swarm state on the host, stepped by the restatement.  With
    ``nglobal`` > 0 it is the shard of particles first .. first + n - 1 of an
    nglobal-particle swarm: after each init / step its g, gcost, gidx hold the
    shard's own best, and :meth:`record` / :meth:`apply` are the global-best
    exchange (the whole swarm's argmin over the shards' bests,
    src/lowerlevel_solve.jl:23-33)."""

    def __init__(self, prob: OracleProblem, n: int, seed: int, first: int = 0, nglobal: int = 0):
        self.prob, self.n, self.dim, self.seed = prob, int(n), prob.dim, int(seed)
        D, n = self.dim, self.n
        self.x = np.zeros((D, n), np.float32)
        self.v = np.zeros((D, n), np.float32)
        self.pbest = np.zeros((D, n), np.float32)
        self.pcost = np.zeros(n, np.float32)
        self.cost = np.zeros(n, np.float32)
        self.g = np.zeros(D, np.float32)
        self.c = SwarmC(n, D, fp(self.x), fp(self.v), fp(self.pbest), fp(self.pcost), fp(self.cost), fp(self.g),
                        0.0, 0, int(first), int(nglobal))
        self.t = 0

    def record(self) -> np.ndarray:
        """The shard's exchange record: argmin key (uint64), cost (float32), 0,
        then the vector, padded to a multiple of 16 bytes."""
        nbytes = (16 + 4 * self.dim + 15) // 16 * 16
        rec = np.zeros(nbytes, np.uint8)
        rec[0:8] = np.frombuffer(np.uint64(argmin_key(self.c.gcost, self.gidx)).tobytes(), np.uint8)
        rec[8:12] = np.frombuffer(np.float32(self.c.gcost).tobytes(), np.uint8)
        rec[16:16 + 4 * self.dim] = np.frombuffer(self.g.tobytes(), np.uint8)
        return rec

    def apply(self, records) -> None:
        """The global best := the record with the lowest key (records: nrec x bytes
        or the flat concatenation)."""
        nbytes = (16 + 4 * self.dim + 15) // 16 * 16
        recs = np.asarray(records, np.uint8).reshape(-1, nbytes)
        keys = [int(np.frombuffer(r[0:8].tobytes(), np.uint64)[0]) for r in recs]
        w = min(range(len(keys)), key=keys.__getitem__)  # the first of equal keys (equal keys are one particle)
        self.g[:] = np.frombuffer(recs[w, 16:16 + 4 * self.dim].tobytes(), np.float32)
        self.c.gcost = float(np.frombuffer(recs[w, 8:12].tobytes(), np.float32)[0])
        self.c.gidx = keys[w] & 0xFFFFFFFF

    @property
    def gcost(self) -> float:
        return float(self.c.gcost)

    @property
    def gidx(self) -> int:
        return int(self.c.gidx)

    def init(self, sampler: int = SAMPLER_UNIFORM) -> "OracleSwarm":
        load().orc_init(ctypes.byref(self.prob.c), ctypes.byref(self.c), self.seed, sampler)
        self.t = 0
        return self

    def sync_run(self, iters, w=0.7298, wdamp=1.0, c1=1.4962, c2=1.4962, gbest_source=GBEST_FROM_PBEST,
                 nthreads=None) -> float:
        wo = load().orc_sync_run(ctypes.byref(self.prob.c), ctypes.byref(self.c), self.seed, self.t, int(iters),
                                 w, wdamp, c1, c2, gbest_source, nthreads or default_threads())
        self.t += int(iters)
        return wo

    def async_run(self, iters, w=0.7298, wdamp=1.0, c1=1.4962, c2=1.4962, lanes=None, nthreads=None) -> float:
        if lanes is None:
            lanes = async_lanes(self.dim)[0]
        wo = load().orc_async_run(ctypes.byref(self.prob.c), ctypes.byref(self.c), self.seed, self.t, int(iters),
                                  w, wdamp, c1, c2, lanes, nthreads or default_threads())
        self.t += int(iters)
        return wo

    def state(self) -> dict:
        return {"x": self.x.copy(), "v": self.v.copy(), "pbest": self.pbest.copy(), "pcost": self.pcost.copy(),
                "cost": self.cost.copy()}


def argmin_key(cost: float, idx: int) -> int:
    """(orderable cost << 32) | idx, the key every argmin minimises."""
    return int(load().orc_argmin_key(float(np.float32(cost)), int(idx) & 0xFFFFFFFF))


def async_lanes(dim: int):
    s = ctypes.c_int32()
    lanes = load().orc_async_lanes(int(dim), ctypes.byref(s))
    return int(lanes), int(s.value)


def lbfgs(prob: OracleProblem, x0, history=10, maxiters=100, armijo_c1=1e-4, gtol=1e-5, max_backtracks=30,
          nthreads=None, broyden=False):
    """Local stage from start points x0 (dim, n). Returns (x, f, iters)."""
    x0 = np.ascontiguousarray(np.asarray(x0, np.float32))
    D, n = x0.shape
    xo = np.empty_like(x0)
    fo = np.empty(n, np.float32)
    it = np.empty(n, np.int32)
    o = LbfgsOpts(history, maxiters, armijo_c1, gtol, max_backtracks)
    fn = load().orc_broyden if broyden else load().orc_lbfgs
    fn(ctypes.byref(prob.c), n, fp(x0), ctypes.byref(o), fp(xo), fp(fo), it.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
       nthreads or default_threads())
    return xo, fo, it


def reduce_losses(data, us) -> np.ndarray:
    """data (m, k), us (n, m, k) -> losses (n,)."""
    data = np.ascontiguousarray(np.asarray(data, np.float32))
    us = np.ascontiguousarray(np.asarray(us, np.float32))
    n, m, k = us.shape
    out = np.empty(n, np.float32)
    load().orc_reduce_losses(m, k, n, fp(data), fp(us), fp(out))
    return out


def mlp_loss(x, X, y) -> float:
    """MLP regression loss of particle x (577) on samples X (S, 16), y (S,)."""
    x = np.ascontiguousarray(np.asarray(x, np.float32))
    X = np.ascontiguousarray(np.asarray(X, np.float32))
    y = np.ascontiguousarray(np.asarray(y, np.float32))
    return float(load().orc_mlp_loss(fp(x), fp(X), fp(y), int(y.size)))


# the prefix that makes the source of a user objective (the CUDA C of
# pps_objective_register) a C translation unit: the same arithmetic, with the
# oracle's exp / cos 2 pi x / sin 2 pi x for the library's own functions
_USER_PREFIX = """#include <math.h>
typedef const float* pps_point;
#define PPS_DEVICE
float orc_exp(float x);
float orc_cos2pi(float x);
float orc_sin2pi(float x);
#define pps_exp orc_exp
#define pps_cos2pi orc_cos2pi
#define pps_sin2pi orc_sin2pi
#line 1 "objective"
"""


# the fold of a PPS_HAS_STREAM source driven as the step kernel drives it:
# start, add for d = 0 .. dim-1, finish
_USER_STREAM_SHIM = """
float pps_stream_eval(const float* x, int dim, const float* p, const float* data, long long ndata) {
  pps_stream s;
  pps_stream_start(&s, dim, p, data, ndata);
  for (int d = 0; d < dim; ++d) pps_stream_add(&s, d, x[d], dim, p, data, ndata);
  return pps_stream_finish(&s, dim, p, data, ndata);
}
"""


class UserObjective:
    """A user objective's source compiled as C by gcc (-ffp-contract=off) into
    oracle/_build/user_<hash>.so, linked against the oracle for pps_exp etc."""

    def __init__(self, source: str):
        import hashlib
        load()
        h = hashlib.sha256(source.encode()).hexdigest()[:16]
        so = HERE / "_build" / f"user_{h}.so"
        if not so.exists():
            c = HERE / "_build" / f"user_{h}.c"
            c.write_text(_USER_PREFIX + source + "\n" + (_USER_STREAM_SHIM if "PPS_HAS_STREAM" in source else ""))
            tmp = so.with_suffix(f".{os.getpid()}.tmp")
            subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math",
                            "-o", str(tmp), str(c), str(LIB_PATH), f"-Wl,-rpath,{LIB_PATH.parent}", "-lm"],
                           check=True, capture_output=True, text=True)
            os.replace(tmp, so)
        self.source = source
        self.lib = ctypes.CDLL(str(so))
        self.fn = USER_FN(ctypes.cast(self.lib.pps_objective, ctypes.c_void_p).value)
        g = getattr(self.lib, "pps_gradient", None) if "PPS_HAS_GRADIENT" in source else None
        self.grad = USER_GRAD(ctypes.cast(g, ctypes.c_void_p).value) if g is not None else None
        st = getattr(self.lib, "pps_stream_eval", None) if "PPS_HAS_STREAM" in source else None
        self.stream_fn = USER_FN(ctypes.cast(st, ctypes.c_void_p).value) if st is not None else None

    def __call__(self, x, params=(), data=None) -> float:
        return self._call(self.fn, x, params, data)

    def stream(self, x, params=(), data=None) -> float:
        """f(x) through the source's fold (start, add in increasing d, finish)."""
        if self.stream_fn is None:
            raise ValueError("the source does not define PPS_HAS_STREAM")
        return self._call(self.stream_fn, x, params, data)

    @staticmethod
    def _call(fn, x, params, data) -> float:
        x = np.ascontiguousarray(np.asarray(x, np.float32))
        p = np.zeros(8, np.float32)
        p[:len(params)] = params
        d = None if data is None else np.ascontiguousarray(np.asarray(data, np.float32).reshape(-1))
        return float(fn(fp(x), x.size, fp(p), fp(d) if d is not None else ctypes.cast(None, _fp),
                        0 if d is None else d.size))


def ode_fit_problem(prob) -> OracleProblem:
    """OracleProblem for an ODE-fit problem of the package (duck-typed: f.name,
    dim, p = [u0_1, u0_2, dt, nsteps, save_every, l(, method, save_dt)], data,
    lb, ub)."""
    p = np.asarray(prob.p, np.float32)
    model = ODE_LV if prob.f.name == "lotka_volterra_fit" else ODE_FHN
    method, save_dt = (int(p[6]), float(p[7])) if p.size > 7 else (0, 0.0)
    if method == ODE_TSIT5_ADAPTIVE:  # p[3], p[4] = reltol, abstol
        fit = OracleOdeFit(model, prob.dim, (p[0], p[1]), p[2], 0, 0, prob.data, fixed=(p[5], 0.0, 0.0, 0.0),
                           method=method, save_dt=save_dt, rtol=float(p[3]), atol=float(p[4]))
    else:
        fit = OracleOdeFit(model, prob.dim, (p[0], p[1]), p[2], int(p[3]), int(p[4]), prob.data,
                           fixed=(p[5], 0.0, 0.0, 0.0), method=method, save_dt=save_dt)
    return OracleProblem(4 if model == ODE_LV else 5, prob.dim, prob.lb, prob.ub, ode=fit)
