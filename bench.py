"""Benchmark of the synchronous PSO step on its headline workload.

Workload (one "step"): a ParallelSyncPSOKernel solve of 2^20 particles x
D = 100 Rastrigin, Float32, bounds [-5.12, 5.12], positions uniform from the
seed, velocities zero, 1000 iterations.  As in the reference
(src/solve.jl:15-26) the timed region is the iteration loop; every step starts
from a fresh init (untimed).  The iteration loop streams 2.1 GB of swarm state
per iteration, far beyond the 129 MB L2, so no L2 flush is needed between
iterations.

Prints ONE JSON line (rank 0).  Extra measurements ride in the same line:
  e2e          the same metric through the public solve() API with host
               buffers: allocation, init, the loop, and the copy-back of the
               solution and of every particle's position (sol.original)
  roofline     the step kernel against the measured HBM copy bandwidth
  cpu_baseline the oracle (C restatement, all host cores) on a bounded sample
  async        ParallelPSOKernel(global_update=false) on the same workload
With --impl reference the oracle's CPU implementation is timed instead
(the Julia reference cannot run here: no Julia toolchain).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "parallelparticleswarms.jl_gb300"))

N_PARTICLES = 1 << 20
DIM = 100
ITERS = 1000
LO, HI = -5.12, 5.12
BYTES_PER_PARTICLE_ITER = 4 * (5 * DIM + 2)  # read x, v, pbest, pcost; write x, v, pcost
METRIC = "PSO particle-iters/s"
UNIT = "particle-iters/s"
WORKLOAD = "sync PSO, 2^20 particles x 100-D Rastrigin, Float32, bounds [-5.12,5.12], 1000 iterations"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        mhz, maxm, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                maxm.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": max(maxm), "reasons": sorted(reasons),
                "samples": len(mhz)}


def measured_hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per step launch from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "k_sync_step_rastrigin_2p20x100.txt"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("dram_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def make_problem(pps):
    lb = np.full(DIM, LO, np.float32)
    ub = np.full(DIM, HI, np.float32)
    return pps.OptimizationProblem(pps.rastrigin, np.zeros(DIM, np.float32), [10.0], lb=lb, ub=ub)


def cpu_oracle_rate(n: int, iters: int, threads: int, seed: int = 0):
    """Oracle sync PSO on the host: returns (particle-iters/s, seconds)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pps_oracle as orc

    lb = np.full(DIM, LO, np.float32)
    ub = np.full(DIM, HI, np.float32)
    prob = orc.OracleProblem(2, DIM, lb, ub, params=[10.0])
    sw = orc.OracleSwarm(prob, n, seed).init()
    sw.sync_run(1, nthreads=threads)  # warm the pages and threads
    t0 = time.perf_counter()
    sw.sync_run(iters, nthreads=threads)
    dt = time.perf_counter() - t0
    return n * iters / dt, dt


def run_reference(args, rank, world):
    """--impl reference: the oracle's CPU implementation on the same metric."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n_sample, it_sample = 1 << 18, 4
    sample = f"{n_sample} particles x {DIM}-D Rastrigin, {it_sample} sync iterations per step (bounded sample)"
    rates = []
    for k in range(args.warmup + args.steps):
        r, _ = cpu_oracle_rate(n_sample, it_sample, threads, seed=k)
        if k >= args.warmup:
            rates.append(r)
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * n_sample * it_sample / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "ParallelParticleSwarms.jl is Julia and no Julia toolchain exists here; the timed CPU path "
                    "is the C restatement of its sync CPU-backend loop (oracle/), threaded over particles"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pps", choices=["pps", "reference"])
    ap.add_argument("--iters", type=int, default=ITERS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-async", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU-baseline sample")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        return run_reference(args, rank, world)

    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist

    import parallelparticleswarms as pps
    from parallelparticleswarms import _lib

    _lib.check(_lib.load().pps_set_device(local))
    prob = make_problem(pps)
    iters = args.iters
    seed0 = 1000 * rank

    def barrier():
        if dist:
            dist.barrier()

    # ---- device-timed loop (inputs resident in HBM) ----------------------
    sw = pps.Swarm(prob, N_PARTICLES, seed=seed0)
    for k in range(args.warmup):
        sw.init()
        sw.sync_run(iters)
    step_ms = []
    barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            sw.init()  # fresh swarm; init is outside the timed loop as in src/solve.jl:15-26
            step_ms.append(sw.sync_run(iters))  # CUDA events on the swarm's stream
    barrier()
    total_ms = sum(step_ms)
    if dist:
        import torch

        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    _, gcost, _ = sw.gbest()
    sw.close()
    units = N_PARTICLES * iters * args.steps * world
    value = units / (total_ms / 1000.0)
    launch_ms = total_ms / (args.steps * iters)
    algo_bytes = N_PARTICLES * BYTES_PER_PARTICLE_ITER
    achieved = algo_bytes / (launch_ms / 1000.0) / 1e9
    peak, peak_src = measured_hbm_peak()
    traffic = profiled_traffic()

    # ---- async at the same size -----------------------------------------
    async_rate = None
    if rank == 0 and not args.no_async:
        sa = pps.Swarm(prob, N_PARTICLES, seed=seed0 + 1)
        sa.init()
        sa.async_run(50)
        sa.init()
        ams = sa.async_run(iters)
        async_rate = N_PARTICLES * iters / (ams / 1000.0)
        sa.close()

    # ---- end to end through solve() with host buffers --------------------
    e2e = None
    if not args.no_e2e:
        alg = pps.ParallelSyncPSOKernel(N_PARTICLES)
        pps.solve(prob, alg, maxiters=iters, seed=seed0)  # warm
        barrier()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 3))
        for k in range(e2e_steps):
            sol = pps.solve(prob, alg, maxiters=iters, seed=seed0 + k)
            _ = sol.objective
        barrier()
        e2e_s = time.perf_counter() - t0
        h2d = 4 * (3 * DIM + 1)  # lb, ub, u0, p
        d2h = 4 * DIM + 8 + 4 + 4 * N_PARTICLES * DIM  # u, gbest cost+index, objective, original positions
        e2e = {"value": N_PARTICLES * iters * e2e_steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
               "path": "parallelparticleswarms.solve -> libpps_cuda.so C ABI (pps_swarm_create/init/sync_run/"
                       "get_gbest/get_state/eval_objective)"}

    # ---- CPU baseline (oracle on the host cores) --------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n_s = 1 << 18
        rate0, _ = cpu_oracle_rate(n_s, 1, threads)  # size the sample to about --cpu-seconds
        it_s = max(1, min(200, int(args.cpu_seconds * rate0 / n_s)))
        rate, secs = cpu_oracle_rate(n_s, it_s, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n_s} particles x {DIM}-D Rastrigin, {it_s} sync iterations ({secs:.1f} s), "
                         "C restatement threaded over particles"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": N_PARTICLES, "dim": DIM, "iterations_per_step": iters,
                       "objective": "rastrigin", "algorithm": "ParallelSyncPSOKernel",
                       "l2": "inputs larger than L2: 2.1 GB of swarm state streamed per iteration",
                       "parallelism": f"{world} independent swarm(s), one per GPU" if world > 1 else "single swarm"},
            "e2e": e2e,
            "gpu_launches": args.steps * (iters + 2),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_sync_step<Rastrigin>", "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": algo_bytes,
                         "avg_launch_ms": launch_ms},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "async": None if async_rate is None else {"metric": METRIC, "value": async_rate, "unit": UNIT,
                      "workload": "ParallelPSOKernel(global_update=false), same size, one launch"},
            "final_gbest_cost": gcost,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
