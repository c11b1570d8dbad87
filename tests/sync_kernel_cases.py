"""Final states of a few synchronous runs, for comparing the two step kernels.

The library has two kernels for the synchronous step of a registered
objective without constraints: the register-prefetch one (k_sync_step, the
default) and the TMA-staged one (k_sync_step_bulk: the swarm state streamed
through shared memory by bulk copies), which PPS_SYNC_KERNEL=bulk selects for
the whole process.  Both must move every particle by the same binary32
operations.  Run as a script,
``python tests/sync_kernel_cases.py OUT.npz`` writes the final state of every
case to OUT.npz under whatever kernel the environment selects; the GPU test
runs the cases in its own process too and compares the two files' arrays."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent

# (objective, dim, particles, lo, hi, params, iterations, global best from position)
CASES = [
    ("rastrigin", 100, 5000, -5.12, 5.12, [10.0], 9, False),      # 9 full tiles of 512 and a ragged one
    ("rosenbrock", 3, 1000, -1.0, 10.0, [1.0, 100.0], 40, True),  # graph-replayed chunk, CPU-backend rule
    ("ackley", 11, 777, -5.0, 5.0, [20.0, 0.2, 1.0], 30, False),  # odd dim: the last dim of a stage alone
    ("sphere", 1, 300, -3.0, 3.0, [], 25, False),                 # one dim
    ("rastrigin", 1000, 1100, -5.12, 5.12, [10.0], 5, False),     # 12 kB of bounds beside the ring
    ("himmelblau", 2, 70000, -5.0, 5.0, [], 33, False),           # 137 tiles over the resident blocks
    ("rastrigin", 4096, 96, -5.12, 5.12, [10.0], 3, False),       # the largest dim: 48 kB of bounds
]


def case_id(c):
    return f"{c[0]}-D{c[1]}-n{c[2]}"


def run_cases(pps) -> dict:
    out = {}
    for c in CASES:
        name, D, n, lo, hi, prm, iters, gpos = c
        prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None,
                                       lb=np.full(D, lo, np.float32), ub=np.full(D, hi, np.float32))
        with pps.Swarm(prob, n, seed=23, gbest_from_position=gpos) as sw:
            sw.init()
            sw.sync_run(iters)
            st = sw.state()
            u, cost, idx = sw.gbest()
        key = case_id(c)
        for k in ("x", "v", "pbest", "pcost", "cost"):
            out[f"{key}/{k}"] = st[k]
        out[f"{key}/g"] = np.asarray(u, np.float32)
        out[f"{key}/gcost"] = np.float32(cost)
        out[f"{key}/gidx"] = np.int64(idx)
    return out


if __name__ == "__main__":
    sys.path.insert(0, str(ROOT / "parallelparticleswarms.jl_gb300"))
    import parallelparticleswarms as pps

    np.savez(sys.argv[1], **run_cases(pps))
