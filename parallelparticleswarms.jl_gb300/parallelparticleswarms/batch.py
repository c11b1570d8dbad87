"""Many independent swarms in one persistent launch (pps_batch_* in include/pps.h).

Each swarm is a full synchronous solve with the same result as solving it
alone through Swarm.init() + Swarm.sync_run(maxiters)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .problem import OptimizationProblem
from .swarm import C1_DEFAULT, C2_DEFAULT, W_DEFAULT, WDAMP_DEFAULT


class Batch:
    def __init__(self):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        _lib.check(self._lib.pps_batch_create(ctypes.byref(self._h)))
        self.problems: list[OptimizationProblem] = []
        self.sizes: list[int] = []
        self.last_device_ms = 0.0

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pps_batch_destroy(self._h)
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

    def add(self, prob: OptimizationProblem, n: int, *, maxiters: int = 100, seed: int = 0, w: float = W_DEFAULT,
            wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT, c2: float = C2_DEFAULT) -> int:
        slot = ctypes.c_int32()
        pr = prob.to_c()
        _lib.check(self._lib.pps_batch_add(self._h, ctypes.byref(pr), int(n), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                           int(maxiters), float(w), float(wdamp), float(c1), float(c2),
                                           ctypes.byref(slot)))
        self.problems.append(prob)
        self.sizes.append(int(n))
        return int(slot.value)

    def set_shape(self, threads: int = 0, ppt: int = 0) -> None:
        _lib.check(self._lib.pps_batch_set_shape(self._h, int(threads), int(ppt)))

    def run(self) -> float:
        ms = ctypes.c_float()
        _lib.check(self._lib.pps_batch_run(self._h, ctypes.byref(ms)))
        self.last_device_ms = float(ms.value)
        return self.last_device_ms

    def info(self) -> dict:
        ns, th, pp, by = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
        _lib.check(self._lib.pps_batch_info(self._h, ctypes.byref(ns), ctypes.byref(th), ctypes.byref(pp),
                                            ctypes.byref(by)))
        return {"swarms": ns.value, "threads": th.value, "ppt": pp.value, "device_bytes": by.value}

    def result(self, slot: int):
        u = np.empty(self.problems[slot].dim, np.float32)
        c = ctypes.c_float()
        i = ctypes.c_int64()
        _lib.check(self._lib.pps_batch_result(self._h, int(slot), _lib.fptr(u), ctypes.byref(c), ctypes.byref(i)))
        return u, float(c.value), int(i.value)

    def state(self, slot: int) -> dict:
        D, n = self.problems[slot].dim, self.sizes[slot]
        out = {}
        for name, f, vec in (("x", _lib.FIELD_POSITION, True), ("v", _lib.FIELD_VELOCITY, True),
                             ("pbest", _lib.FIELD_PBEST, True), ("pcost", _lib.FIELD_PCOST, False),
                             ("cost", _lib.FIELD_COST, False)):
            a = np.empty((D if vec else 1, n), np.float32)
            _lib.check(self._lib.pps_batch_get_state(self._h, int(slot), f, _lib.fptr(a)))
            out[name] = a if vec else a[0]
        return out
