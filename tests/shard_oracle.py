"""The oracle's restatement of one shard of a swarm, with the shard protocol
that parallelparticleswarms.shard.sync_loop drives (step / ordered / local /
gathered / apply / finish), its records in CPU tensors so that a gloo
all-gather can exchange them.  Test infrastructure: the oracle is the
checker; the loop and the exchange it runs are the package's own."""
import contextlib

import numpy as np


class OracleShard:
    def __init__(self, orc, oprob, n_global, first, count, seed, nrecords, gbest_source=0):
        import torch

        self.orc = orc
        self.ref = orc.OracleSwarm(oprob, count, seed, first=first, nglobal=n_global)
        self.nb = (16 + 4 * oprob.dim + 15) // 16 * 16
        self.local = torch.zeros(self.nb, dtype=torch.uint8)
        self.gathered = torch.zeros(int(nrecords) * self.nb, dtype=torch.uint8)
        self.src = gbest_source
        self.w = None

    def _publish(self):
        import torch

        self.local.copy_(torch.from_numpy(self.ref.record()))

    def init(self, sampler=0):
        self.ref.init(sampler)
        self._publish()
        return self

    def step(self, begin, w, wdamp, c1, c2):
        if begin:
            self.w = w
        # one synchronous iteration; the oracle returns w damped in binary32
        self.w = self.ref.sync_run(1, w=self.w, wdamp=wdamp, c1=c1, c2=c2, gbest_source=self.src)
        self._publish()

    def async_run(self, iters, w, wdamp, c1, c2):
        self.ref.async_run(iters, w=w, wdamp=wdamp, c1=c1, c2=c2)
        self._publish()

    def ordered(self):
        return contextlib.nullcontext()

    def apply(self):
        self.ref.apply(self.gathered.numpy())

    def finish(self):
        pass


def local_exchange(shards):
    """The exchange of shards in one process: every shard's record, concatenated."""
    recs = np.concatenate([s.local.numpy() for s in shards])
    for s in shards:
        s.gathered.copy_(__import__("torch").from_numpy(recs.copy()))
