"""Thin owner of one ``pps_swarm`` handle (device-resident swarm state)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .problem import OptimizationProblem

# defaults of src/lowerlevel_solve.jl:6-7 and src/kernels.jl:130-131
W_DEFAULT = 0.7298
WDAMP_DEFAULT = 1.0
C1_DEFAULT = 1.4962
C2_DEFAULT = 1.4962


class Swarm:
    """Device swarm of ``n`` particles for ``prob`` (SoA state in HBM)."""

    def __init__(self, prob: OptimizationProblem, n: int, seed: int = 0, gbest_from_position: bool = False):
        self.prob = prob
        self.n = int(n)
        self.dim = prob.dim
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        flags = _lib.FLAG_GBEST_FROM_POSITION if gbest_from_position else 0
        pr = prob.to_c()
        _lib.check(self._lib.pps_swarm_create(ctypes.byref(pr), self.n, self.seed, flags, ctypes.byref(self._h)))
        self.last_device_ms = 0.0

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pps_swarm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- operations -------------------------------------------------------
    def init(self, sampler: int = _lib.SAMPLER_AUTO) -> "Swarm":
        _lib.check(self._lib.pps_swarm_init(self._h, int(sampler)))
        return self

    def _run(self, fn, maxiters, w, wdamp, c1, c2) -> float:
        ms = ctypes.c_float(0.0)
        _lib.check(fn(self._h, int(maxiters), float(w), float(wdamp), float(c1), float(c2), ctypes.byref(ms)))
        self.last_device_ms = float(ms.value)
        return self.last_device_ms

    def sync_run(self, maxiters, w=W_DEFAULT, wdamp=WDAMP_DEFAULT, c1=C1_DEFAULT, c2=C2_DEFAULT) -> float:
        return self._run(self._lib.pps_sync_run, maxiters, w, wdamp, c1, c2)

    def async_run(self, maxiters, w=W_DEFAULT, wdamp=WDAMP_DEFAULT, c1=C1_DEFAULT, c2=C2_DEFAULT) -> float:
        return self._run(self._lib.pps_async_run, maxiters, w, wdamp, c1, c2)

    def queue_run(self, maxiters, w=W_DEFAULT, wdamp=WDAMP_DEFAULT, c1=C1_DEFAULT, c2=C2_DEFAULT) -> float:
        return self._run(self._lib.pps_queue_run, maxiters, w, wdamp, c1, c2)

    # -- state ------------------------------------------------------------
    def gbest(self):
        u = np.empty(self.dim, dtype=np.float32)
        c = ctypes.c_float()
        i = ctypes.c_int64()
        _lib.check(self._lib.pps_get_gbest(self._h, _lib.fptr(u), ctypes.byref(c), ctypes.byref(i)))
        return u, float(c.value), int(i.value)

    def local_stage(self, kind: str, history=10, maxiters=50, armijo_c1=1e-4, gtol=1e-5, max_backtracks=30):
        """HybridPSO local stage on every particle: kind "lbfgs" (from personal
        bests) or "bfgs" (Broyden, from positions).  Returns (u, f, idx, device_ms)
        of the best local result."""
        o = _lib.LocalOpts(int(history), int(maxiters), float(armijo_c1), float(gtol), int(max_backtracks))
        u = np.empty(self.dim, dtype=np.float32)
        f = ctypes.c_float()
        i = ctypes.c_int64()
        ms = ctypes.c_float()
        fn = self._lib.pps_hybrid_lbfgs if kind == "lbfgs" else self._lib.pps_hybrid_bfgs
        _lib.check(fn(self._h, ctypes.byref(o), _lib.fptr(u), ctypes.byref(f), ctypes.byref(i), ctypes.byref(ms)))
        return u, float(f.value), int(i.value), float(ms.value)

    def get(self, field: int) -> np.ndarray:
        """(dim, n) for position / velocity / pbest / local optima, (n,) otherwise."""
        vec = field in (_lib.FIELD_POSITION, _lib.FIELD_VELOCITY, _lib.FIELD_PBEST, _lib.FIELD_LOCAL_X)
        out = np.empty((self.dim if vec else 1, self.n), dtype=np.float32)
        _lib.check(self._lib.pps_get_state(self._h, int(field), _lib.fptr(out)))
        return out if vec else out[0]

    def set(self, field: int, values) -> None:
        rows = self.dim if field in (_lib.FIELD_POSITION, _lib.FIELD_VELOCITY, _lib.FIELD_PBEST) else 1
        arr = np.ascontiguousarray(np.asarray(values, dtype=np.float32).reshape(rows, self.n))
        _lib.check(self._lib.pps_set_state(self._h, int(field), _lib.fptr(arr)))

    def positions(self) -> np.ndarray:
        """(dim, n) SoA positions."""
        return self.get(_lib.FIELD_POSITION)

    def record_dtype(self) -> np.dtype:
        """SPSOParticle{position, velocity, cost, best_position, best_cost}
        (src/ParallelParticleSwarms.jl:34-44) as a numpy record."""
        D = self.dim
        return np.dtype([("position", np.float32, (D,)), ("velocity", np.float32, (D,)), ("cost", np.float32),
                         ("best_position", np.float32, (D,)), ("best_cost", np.float32)])

    def particles(self) -> np.ndarray:
        """Every particle as the reference's record (an (n,) structured array)."""
        out = np.empty(self.n, self.record_dtype())
        _lib.check(self._lib.pps_get_particles(self._h, _lib.LAYOUT_AOS,
                                               out.ctypes.data_as(_lib.c_float_p)))
        return out

    def set_particles(self, records) -> None:
        """Replace every particle by the given records (structured array or
        (n, 3 dim + 2) floats); the global best becomes the argmin of best_cost."""
        arr = np.ascontiguousarray(records)
        if arr.dtype != self.record_dtype():
            arr = np.ascontiguousarray(np.asarray(records, np.float32).reshape(self.n, 3 * self.dim + 2))
        if arr.nbytes != self.n * (3 * self.dim + 2) * 4:
            raise _lib.ArgumentError(_lib.EINVAL, f"expected {self.n} records of {3 * self.dim + 2} floats")
        _lib.check(self._lib.pps_set_particles(self._h, _lib.LAYOUT_AOS, arr.ctypes.data_as(_lib.c_float_p)))

    def positions_on_device(self) -> "DevicePositions":
        """A device snapshot of the positions (the reference's sol.original)."""
        return DevicePositions(self, _lib.FIELD_POSITION)

    def state(self) -> dict:
        return {
            "x": self.get(_lib.FIELD_POSITION),
            "v": self.get(_lib.FIELD_VELOCITY),
            "pbest": self.get(_lib.FIELD_PBEST),
            "pcost": self.get(_lib.FIELD_PCOST),
            "cost": self.get(_lib.FIELD_COST),
        }

    def info(self) -> _lib.SwarmInfo:
        inf = _lib.SwarmInfo()
        _lib.check(self._lib.pps_swarm_info_get(self._h, ctypes.byref(inf)))
        return inf


class DevicePositions:
    """Every particle's position as an (n, dim) array that stays in device memory
    until it is read: the reference's sol.original = get_pos.(particles) is a new
    device array (src/solve.jl:51-56).  ``np.asarray`` (or ``.numpy()``) copies it
    to the host once; the swarm it came from may be re-run or closed meanwhile."""

    def __init__(self, swarm: Swarm, field: int):
        self._lib = swarm._lib
        self._h = ctypes.c_void_p()
        self.shape = (swarm.n, swarm.dim)
        self.dtype = np.dtype(np.float32)
        self._host = None
        _lib.check(self._lib.pps_field_copy_create(swarm._h, int(field), ctypes.byref(self._h)))

    def numpy(self) -> np.ndarray:
        if self._host is None:
            n, dim = self.shape
            soa = np.empty((dim, n), np.float32)
            _lib.check(self._lib.pps_field_copy_read(self._h, _lib.fptr(soa)))
            self._host = soa.T  # (n, dim) view of the SoA copy
            self.close()
        return self._host

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a if dtype is None else a.astype(dtype)

    def __len__(self) -> int:
        return self.shape[0]

    def __getitem__(self, idx):
        return self.numpy()[idx]

    @property
    def ndim(self) -> int:
        return 2

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pps_field_copy_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self) -> str:
        where = "host" if self._host is not None else "device"
        return f"<DevicePositions {self.shape[0]} x {self.shape[1]} float32 on the {where}>"
