"""ctypes binding of libpps_cuda.so (the C ABI declared in include/pps.h).

The shared library is the only compute path: if it is missing or no CUDA
device is present, every solve raises :class:`PPSError`; nothing falls back to
the CPU.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "lib" / "libpps_cuda.so"

# pps_status
OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EBUSY, ENOTSUP, ENODEV = range(8)
STATUS_NAMES = {0: "PPS_OK", 1: "PPS_EINVAL", 2: "PPS_ENOMEM", 3: "PPS_ECUDA", 4: "PPS_ETIMEOUT",
                5: "PPS_EBUSY", 6: "PPS_ENOTSUP", 7: "PPS_ENODEV"}

# samplers, flags, fields
SAMPLER_AUTO, SAMPLER_UNIFORM, SAMPLER_UNBOUNDED, SAMPLER_LHS = 0, 1, 2, 3
FLAG_GBEST_FROM_POSITION = 1
FIELD_POSITION, FIELD_VELOCITY, FIELD_PBEST, FIELD_PCOST, FIELD_COST = range(5)
FIELD_LOCAL_X, FIELD_LOCAL_F, FIELD_LOCAL_ITERS = 5, 6, 7
LAYOUT_SOA, LAYOUT_AOS = 0, 1

c_float_p = ctypes.POINTER(ctypes.c_float)


class PPSError(RuntimeError):
    """A libpps_cuda.so call failed (status code + the library's message)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class ArgumentError(PPSError, ValueError):
    """Invalid argument (the reference raises ArgumentError / AssertionError)."""


class Problem(ctypes.Structure):
    _fields_ = [
        ("objective", ctypes.c_int32),
        ("dim", ctypes.c_int32),
        ("lb", c_float_p),
        ("ub", c_float_p),
        ("u0", c_float_p),
        ("params", c_float_p),
        ("nparams", ctypes.c_int32),
        ("data", c_float_p),
        ("ndata", ctypes.c_int64),
        ("ncons", ctypes.c_int32),
        ("cons", c_float_p),
    ]


class SwarmInfo(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("dim", ctypes.c_int32),
        ("objective", ctypes.c_int32),
        ("iteration", ctypes.c_uint32),
        ("async_lanes", ctypes.c_int32),
        ("async_slice", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("device_bytes", ctypes.c_uint64),
    ]


class LocalOpts(ctypes.Structure):
    _fields_ = [
        ("history", ctypes.c_int32),
        ("maxiters", ctypes.c_int32),
        ("armijo_c1", ctypes.c_float),
        ("gtol", ctypes.c_float),
        ("max_backtracks", ctypes.c_int32),
    ]


class ServeConfig(ctypes.Structure):
    _fields_ = [
        ("memory_budget", ctypes.c_uint64),
        ("max_launches", ctypes.c_int32),
        ("max_pack", ctypes.c_int32),
        ("threads", ctypes.c_int32),
        ("ppt", ctypes.c_int32),
        ("tick_us", ctypes.c_double),
        ("single_min_n", ctypes.c_int32),
        ("ode_single_min_n", ctypes.c_int32),
    ]


class ServeStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("launches", ctypes.c_uint64),
        ("solves_per_s", ctypes.c_double),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("mean_pack", ctypes.c_double),
        ("arena_bytes", ctypes.c_uint64),
        ("arena_peak_bytes", ctypes.c_uint64),
        ("queued", ctypes.c_int32),
        ("running", ctypes.c_int32),
    ]


class DeviceSwarm(ctypes.Structure):
    """pps_device_swarm: a swarm in device buffers owned by the caller."""

    _fields_ = [
        ("n", ctypes.c_int64),
        ("ld", ctypes.c_int64),
        ("dim", ctypes.c_int32),
        ("x", ctypes.c_void_p),
        ("v", ctypes.c_void_p),
        ("pbest", ctypes.c_void_p),
        ("pcost", ctypes.c_void_p),
        ("cost", ctypes.c_void_p),
        ("lb", ctypes.c_void_p),
        ("ub", ctypes.c_void_p),
        ("g", ctypes.c_void_p),
    ]


_P = ctypes.c_void_p
_SIGNATURES = {
    "pps_version": (ctypes.c_int32, []),
    "pps_last_error": (ctypes.c_char_p, []),
    "pps_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32)]),
    "pps_set_device": (ctypes.c_int, [ctypes.c_int32]),
    "pps_swarm_create": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.c_int64, ctypes.c_uint64,
                                        ctypes.c_uint32, ctypes.POINTER(_P)]),
    "pps_swarm_destroy": (ctypes.c_int, [_P]),
    "pps_swarm_init": (ctypes.c_int, [_P, ctypes.c_int32]),
    "pps_swarm_info_get": (ctypes.c_int, [_P, ctypes.POINTER(SwarmInfo)]),
    "pps_sync_run": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, c_float_p]),
    "pps_async_run": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, c_float_p]),
    "pps_queue_run": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, c_float_p]),
    "pps_get_gbest": (ctypes.c_int, [_P, c_float_p, c_float_p, ctypes.POINTER(ctypes.c_int64)]),
    "pps_get_state": (ctypes.c_int, [_P, ctypes.c_int32, c_float_p]),
    "pps_set_state": (ctypes.c_int, [_P, ctypes.c_int32, c_float_p]),
    "pps_get_particles": (ctypes.c_int, [_P, ctypes.c_int32, c_float_p]),
    "pps_set_particles": (ctypes.c_int, [_P, ctypes.c_int32, c_float_p]),
    "pps_field_copy_create": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(_P)]),
    "pps_field_copy_read": (ctypes.c_int, [_P, c_float_p]),
    "pps_field_copy_destroy": (ctypes.c_int, [_P]),
    "pps_eval_objective": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.c_int64, c_float_p, c_float_p]),
    "pps_batch_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "pps_batch_destroy": (ctypes.c_int, [_P]),
    "pps_batch_add": (ctypes.c_int, [_P, ctypes.POINTER(Problem), ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.POINTER(ctypes.c_int32)]),
    "pps_batch_run": (ctypes.c_int, [_P, c_float_p]),
    "pps_batch_set_shape": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "pps_batch_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_uint64)]),
    "pps_batch_result": (ctypes.c_int, [_P, ctypes.c_int32, c_float_p, c_float_p, ctypes.POINTER(ctypes.c_int64)]),
    "pps_batch_get_state": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, c_float_p]),
    "pps_serve_start": (ctypes.c_int, [ctypes.POINTER(ServeConfig), ctypes.POINTER(_P)]),
    "pps_serve_submit": (ctypes.c_int, [_P, ctypes.POINTER(Problem), ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "pps_serve_poll": (ctypes.c_int, [_P, ctypes.c_uint64, c_float_p, c_float_p, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_double)]),
    "pps_serve_wait": (ctypes.c_int, [_P, ctypes.c_uint64, c_float_p, c_float_p, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_double]),
    "pps_serve_stats_get": (ctypes.c_int, [_P, ctypes.POINTER(ServeStats)]),
    "pps_serve_stop": (ctypes.c_int, [_P]),
    "pps_hybrid_lbfgs": (ctypes.c_int, [_P, ctypes.POINTER(LocalOpts), c_float_p, c_float_p,
                                        ctypes.POINTER(ctypes.c_int64), c_float_p]),
    "pps_hybrid_bfgs": (ctypes.c_int, [_P, ctypes.POINTER(LocalOpts), c_float_p, c_float_p,
                                       ctypes.POINTER(ctypes.c_int64), c_float_p]),
    "pps_objective_register": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32)]),
    "pps_shard_create": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(_P)]),
    "pps_shard_record": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_P)]),
    "pps_shard_bind": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32]),
    "pps_shard_step": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float]),
    "pps_shard_async": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float]),
    "pps_shard_apply": (ctypes.c_int, [_P]),
    "pps_shard_finish": (ctypes.c_int, [_P]),
    "pps_sync_run_noalloc": (ctypes.c_int, [ctypes.c_int32, c_float_p, ctypes.c_int32, ctypes.POINTER(DeviceSwarm),
                                            ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float,
                                            ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32,
                                            ctypes.c_void_p, c_float_p, ctypes.POINTER(ctypes.c_int64)]),
}

_lock = threading.Lock()
_lib = None


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Load libpps_cuda.so once; raise PPSError if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise PPSError(ENODEV, f"{p} is missing: build it with parallelparticleswarms.jl_gb300/csrc/build.py "
                                   "(CUDA is required; there is no CPU fallback)")
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def declared_symbols() -> list[str]:
    return sorted(_SIGNATURES)


def check(rc: int) -> None:
    if rc != OK:
        msg = load().pps_last_error().decode(errors="replace")
        if rc == EINVAL:
            raise ArgumentError(rc, msg)
        raise PPSError(rc, msg)


def fptr(a) -> c_float_p:
    """float* of a C-contiguous float32 numpy array (or NULL for None)."""
    if a is None:
        return ctypes.cast(None, c_float_p)
    return a.ctypes.data_as(c_float_p)
