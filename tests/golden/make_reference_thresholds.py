"""Writes reference_thresholds.json: the statistical pins of the reference's
tests for the PSO step, transcribed from its test files (file:line in each
case).  Run from this directory: ``python make_reference_thresholds.py``.

The reference cannot run in this environment (no Julia toolchain), so these
cases are re-run against the oracle (tests/test_oracle_pins.py) and against
the CUDA path (tests/test_gpu_reference_thresholds.py).
"""
import json
from pathlib import Path

INF = "inf"
NINF = "-inf"
cases = []


def add(id_, src, alg, D, n, iters, lb, ub, thr, seed, cpu_backend=False):
    cases.append(dict(id=id_, source=src, algorithm=alg, dim=D, particles=n, maxiters=iters,
                      lb=lb, ub=ub, threshold=thr, seed=seed, cpu_backend=cpu_backend))


# test/regression.jl: N = 2, 3 Rosenbrock, 2000 particles, Random.seed!(123)
for N in (2, 3):
    add(f"reg_N{N}_queue_box", "test/regression.jl:63-69", "queue", N, 2000, 500, -1.0, 10.0, 1e-4, 123)
    add(f"reg_N{N}_sync_box", "test/regression.jl:81-87", "sync", N, 2000, 500, -1.0, 10.0, 3e-3, 123, True)
    add(f"reg_N{N}_queue_inf", "test/regression.jl:121-127", "queue", N, 2000, 500, NINF, INF, 1e-4, 123)
    add(f"reg_N{N}_sync_inf", "test/regression.jl:139-145", "sync", N, 2000, 500, NINF, INF, 2e-4, 123, True)
    add(f"reg_N{N}_queue_nothing", "test/regression.jl:176-182", "queue", N, 2000, 500, None, None, 1e-4, 123)
    add(f"reg_N{N}_sync_nothing", "test/regression.jl:192-198", "sync", N, 2000, 500, None, None, 2e-2, 123, True)
# test/regression.jl: N = 4, Random.seed!(1)
add("reg_N4_queue_box", "test/regression.jl:257-263", "queue", 4, 2000, 2000, -1.0, 10.0, 2e-2, 1)
add("reg_N4_sync_box", "test/regression.jl:275-281", "sync", 4, 2000, 2000, -1.0, 10.0, 3e-2, 1, True)
add("reg_N4_queue_nothing", "test/regression.jl:318-324", "queue", 4, 2000, 1000, None, None, 2e-3, 1)
add("reg_N4_sync_nothing", "test/regression.jl:336-342", "sync", 4, 2000, 2000, None, None, 4e-1, 1, True)
# test/gpu.jl: N = 2..4, 5000 particles, Random.seed!(1234)
for N in (2, 3, 4):
    add(f"gpu_N{N}_queue", "test/gpu.jl:31-35", "queue", N, 5000, 500, -1.0, 10.0, 2e-3, 1234)
    add(f"gpu_N{N}_async", "test/gpu.jl:39-45", "async", N, 5000, 1000, -1.0, 10.0, None, 1234)
    add(f"gpu_N{N}_sync", "test/gpu.jl:49-57", "sync", N, 5000, 500, -1.0, 10.0, 6e-4, 1234)

doc = {
    "about": ("Statistical pins of the reference's own tests for the PSO step: Rosenbrock p=[1,100], Float32, "
              "x0=0. Each case gives the reference file:line, the algorithm (sync = ParallelSyncPSOKernel, "
              "queue = ParallelPSOKernel(global_update=true), async = ParallelPSOKernel(global_update=false)), "
              "dims, particles, maxiters, bounds (null = `nothing`), the objective threshold (null: only "
              "f(u0) > objective is asserted) and the seed. The reference seeds Julia's global RNG with `seed`; "
              "here it is the Philox key. cpu_backend marks the reference's CPU-backend sync loop (next global "
              "best position taken from the winner's current position, src/lowerlevel_solve.jl:59-60)."),
    "generated_by": "tests/golden/make_reference_thresholds.py",
    "cases": cases,
}

if __name__ == "__main__":
    out = Path(__file__).resolve().parent / "reference_thresholds.json"
    out.write_text(json.dumps(doc, indent=1) + "\n")
    print(f"wrote {len(cases)} cases to {out}")
