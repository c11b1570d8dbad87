"""One swarm split into particle-range shards, with one global-best exchange
per iteration.

The synchronous loop couples its particles only through the global best of
each iteration: block bests, then their minimum (src/kernels.jl:156-171,
src/lowerlevel_solve.jl:23-33).  A shard (``pps_shard_create``) holds a
contiguous range of a swarm's particles and moves them exactly as the whole
swarm does; after its init or step it leaves an exchange record (its best
particle's argmin key, cost and vector).  One iteration of a sharded swarm is

    step every shard  ->  gather every shard's record  ->  apply (lowest key wins)

and reproduces the whole swarm's iteration bit for bit.  The async run
exchanges once, after its last iteration.

Pieces:
  :func:`shard_ranges`       the contiguous particle ranges of k shards
  :class:`TorchDistExchange` the exchange between ranks: an all-gather of the
                             fixed-size records over ``torch.distributed``
                             (NCCL between GPUs), ordered on the shard's stream
  :class:`DeviceShard`       one shard on this process's GPU
  :class:`ShardedSwarm`      this rank's shard of a swarm spread over ranks
  :class:`LocalShards`       several shards of one swarm in one process (one
                             GPU): they share one record array, so no copy is
                             needed, only stream ordering
  :func:`sync_loop`          the sharded synchronous loop over any shard and
                             exchange with this interface

torch is the plumbing for the record buffers, the streams and the collective;
it is imported when a shard is made.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .problem import OptimizationProblem
from .swarm import C1_DEFAULT, C2_DEFAULT, W_DEFAULT, WDAMP_DEFAULT


def shard_ranges(n_global: int, nshards: int) -> list[tuple[int, int]]:
    """(first, count) of each of ``nshards`` contiguous ranges of ``n_global``
    particles, balanced to within one particle."""
    n, k = int(n_global), int(nshards)
    if k < 1 or n < k:
        raise _lib.ArgumentError(_lib.EINVAL, f"cannot split {n} particles into {k} non-empty shards")
    return [(r * n // k, (r + 1) * n // k - r * n // k) for r in range(k)]


def record_bytes(dim: int) -> int:
    """Bytes of one exchange record: key (8), cost (4), 4 zero bytes, dim floats, padded to 16."""
    return (16 + 4 * int(dim) + 15) // 16 * 16


class TorchDistExchange:
    """The record exchange between ranks: every rank's ``local`` record into
    ``gathered`` (rank r's at r * bytes), one all-gather on the current
    stream (NCCL) or on the host (gloo)."""

    def __init__(self, group=None):
        self.group = group

    def __call__(self, local, gathered) -> None:
        import torch.distributed as dist

        dist.all_gather_into_tensor(gathered, local, group=self.group)


def sync_loop(shard, exchange, maxiters: int, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT,
              c1: float = C1_DEFAULT, c2: float = C2_DEFAULT) -> None:
    """``maxiters`` synchronous iterations of a sharded swarm: per iteration
    the shard's step, the exchange of records, the global best applied.  The
    shard provides step / ordered / local / gathered / apply / finish."""
    for k in range(int(maxiters)):
        shard.step(k == 0, w, wdamp, c1, c2)
        with shard.ordered():
            exchange(shard.local, shard.gathered)
        shard.apply()
    shard.finish()


class DeviceShard:
    """Particles ``first .. first + count - 1`` of an ``n_global``-particle swarm
    on the current GPU.  Its record goes to ``local`` (a device tensor of
    ``record_bytes(dim)`` bytes) and its global best is applied from
    ``gathered`` (``nrecords`` records).  Passing ``local`` / ``gathered``
    binds buffers the caller owns (e.g. slots of one array shared by shards
    of one process)."""

    def __init__(self, prob: OptimizationProblem, n_global: int, first: int, count: int, seed: int = 0,
                 nrecords: int = 1, local=None, gathered=None, gbest_from_position: bool = False):
        import torch

        self.prob, self.dim = prob, prob.dim
        self.n_global, self.first, self.n = int(n_global), int(first), int(count)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        flags = _lib.FLAG_GBEST_FROM_POSITION if gbest_from_position else 0
        pr = prob.to_c()
        _lib.check(self._lib.pps_shard_create(ctypes.byref(pr), self.n_global, self.first, self.n, self.seed, flags,
                                              ctypes.byref(self._h)))
        nb, stream = ctypes.c_int64(), ctypes.c_void_p()
        _lib.check(self._lib.pps_shard_record(self._h, None, ctypes.byref(nb), ctypes.byref(stream)))
        self.record_bytes = int(nb.value)
        assert self.record_bytes == record_bytes(self.dim)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.local = local if local is not None else torch.zeros(self.record_bytes, dtype=torch.uint8, device=dev)
        self.gathered = gathered if gathered is not None else torch.zeros(int(nrecords) * self.record_bytes,
                                                                          dtype=torch.uint8, device=dev)
        nrec = self.gathered.numel() // self.record_bytes
        _lib.check(self._lib.pps_shard_bind(self._h, ctypes.c_void_p(self.local.data_ptr()),
                                            ctypes.c_void_p(self.gathered.data_ptr()), nrec))
        self.stream = torch.cuda.ExternalStream(stream.value, device=dev)
        # the buffers were filled on torch's current stream, which the shard's
        # (non-blocking) stream does not wait for: finish the fill before the
        # shard's first kernel writes its record
        torch.cuda.current_stream(dev).synchronize()

    # -- the shard protocol of sync_loop ------------------------------------
    def ordered(self):
        """Work issued inside runs on the shard's stream (after its step)."""
        import torch

        return torch.cuda.stream(self.stream)

    def init(self, sampler: int = _lib.SAMPLER_AUTO) -> "DeviceShard":
        """Sample the shard's particles; its record then holds the shard's best."""
        _lib.check(self._lib.pps_swarm_init(self._h, int(sampler)))
        return self

    def step(self, begin: bool, w: float, wdamp: float, c1: float, c2: float) -> None:
        _lib.check(self._lib.pps_shard_step(self._h, 1 if begin else 0, float(w), float(wdamp), float(c1), float(c2)))

    def async_run(self, maxiters: int, w: float, wdamp: float, c1: float, c2: float) -> None:
        _lib.check(self._lib.pps_shard_async(self._h, int(maxiters), float(w), float(wdamp), float(c1), float(c2)))

    def apply(self) -> None:
        _lib.check(self._lib.pps_shard_apply(self._h))

    def finish(self) -> None:
        _lib.check(self._lib.pps_shard_finish(self._h))

    # -- results --------------------------------------------------------------
    def gbest(self):
        u = np.empty(self.dim, dtype=np.float32)
        c, i = ctypes.c_float(), ctypes.c_int64()
        _lib.check(self._lib.pps_get_gbest(self._h, _lib.fptr(u), ctypes.byref(c), ctypes.byref(i)))
        return u, float(c.value), int(i.value)

    def get(self, field: int) -> np.ndarray:
        vec = field in (_lib.FIELD_POSITION, _lib.FIELD_VELOCITY, _lib.FIELD_PBEST)
        out = np.empty((self.dim if vec else 1, self.n), dtype=np.float32)
        _lib.check(self._lib.pps_get_state(self._h, int(field), _lib.fptr(out)))
        return out if vec else out[0]

    def state(self) -> dict:
        return {"x": self.get(_lib.FIELD_POSITION), "v": self.get(_lib.FIELD_VELOCITY),
                "pbest": self.get(_lib.FIELD_PBEST), "pcost": self.get(_lib.FIELD_PCOST),
                "cost": self.get(_lib.FIELD_COST)}

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


class ShardedSwarm:
    """This rank's shard of a swarm of ``n_global`` particles spread over
    ``world`` ranks (one GPU each), exchanging records through ``exchange``
    (default: an all-gather over the default process group)."""

    def __init__(self, prob: OptimizationProblem, n_global: int, rank: int, world: int, seed: int = 0,
                 exchange=None, gbest_from_position: bool = False):
        first, count = shard_ranges(n_global, world)[rank]
        self.rank, self.world = int(rank), int(world)
        if world == 1 and exchange is None:
            # a lone shard: its record is the whole gathered array, nothing to exchange
            self.shard = DeviceShard(prob, n_global, first, count, seed, gbest_from_position=gbest_from_position)
            self.shard.gathered = self.shard.local
            _lib.check(self.shard._lib.pps_shard_bind(self.shard._h, ctypes.c_void_p(self.shard.local.data_ptr()),
                                                      ctypes.c_void_p(self.shard.local.data_ptr()), 1))
            self.exchange = lambda local, gathered: None
        else:
            self.shard = DeviceShard(prob, n_global, first, count, seed, nrecords=world,
                                     gbest_from_position=gbest_from_position)
            self.exchange = exchange if exchange is not None else TorchDistExchange()

    def _exchange(self) -> None:
        with self.shard.ordered():
            self.exchange(self.shard.local, self.shard.gathered)
        self.shard.apply()

    def init(self, sampler: int = _lib.SAMPLER_AUTO) -> "ShardedSwarm":
        self.shard.init(sampler)
        self._exchange()
        self.shard.finish()
        return self

    def sync_run(self, maxiters: int, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT,
                 c2: float = C2_DEFAULT) -> None:
        sync_loop(self.shard, self.exchange, maxiters, w, wdamp, c1, c2)

    def async_run(self, maxiters: int, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT,
                  c2: float = C2_DEFAULT) -> None:
        self.shard.async_run(maxiters, w, wdamp, c1, c2)
        self._exchange()
        self.shard.finish()

    def gbest(self):
        return self.shard.gbest()

    def state(self) -> dict:
        return self.shard.state()

    def close(self) -> None:
        self.shard.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class LocalShards:
    """``nshards`` shards of one swarm in this process (one GPU), each on its
    own stream.  They share one record array: shard r writes slot r and every
    shard applies the whole array, so the exchange is stream ordering only
    (every apply after every step; every step after every apply of the
    previous iteration, since a step rewrites its slot)."""

    def __init__(self, prob: OptimizationProblem, n_global: int, nshards: int, seed: int = 0,
                 gbest_from_position: bool = False):
        import torch

        self.ranges = shard_ranges(n_global, nshards)
        nb = record_bytes(prob.dim)
        self.records = torch.zeros(nshards * nb, dtype=torch.uint8, device=torch.device("cuda"))
        self.shards = [DeviceShard(prob, n_global, f, c, seed, local=self.records[r * nb:(r + 1) * nb],
                                   gathered=self.records, gbest_from_position=gbest_from_position)
                       for r, (f, c) in enumerate(self.ranges)]

    def _join(self) -> None:
        """Every shard's stream waits for the work issued so far on all of them."""
        import torch

        events = []
        for sh in self.shards:
            ev = torch.cuda.Event()
            ev.record(sh.stream)
            events.append(ev)
        for sh in self.shards:
            for ev in events:
                sh.stream.wait_event(ev)

    def _apply_all(self) -> None:
        self._join()
        for sh in self.shards:
            sh.apply()
        self._join()

    def init(self, sampler: int = _lib.SAMPLER_AUTO) -> "LocalShards":
        for sh in self.shards:
            sh.init(sampler)
        self._apply_all()
        for sh in self.shards:
            sh.finish()
        return self

    def sync_run(self, maxiters: int, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT,
                 c2: float = C2_DEFAULT) -> None:
        for k in range(int(maxiters)):
            for sh in self.shards:
                sh.step(k == 0, w, wdamp, c1, c2)
            self._apply_all()
        for sh in self.shards:
            sh.finish()

    def async_run(self, maxiters: int, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT, c1: float = C1_DEFAULT,
                  c2: float = C2_DEFAULT) -> None:
        for sh in self.shards:
            sh.async_run(maxiters, w, wdamp, c1, c2)
        self._apply_all()
        for sh in self.shards:
            sh.finish()

    def gbest(self):
        return self.shards[0].gbest()

    def state(self) -> dict:
        """The whole swarm's state, shards concatenated along the particle axis."""
        parts = [sh.state() for sh in self.shards]
        return {k: np.concatenate([p[k] for p in parts], axis=-1) for k in parts[0]}

    def close(self) -> None:
        for sh in self.shards:
            sh.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
