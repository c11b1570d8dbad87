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
               buffers: allocation, init, the loop, the device snapshot of
               every particle's position (sol.original, which the reference
               also keeps on the device, src/solve.jl:51-56) and the copy-back
               of the solution u and f(u); reading sol.original to the host
               afterwards is timed separately (original_to_host_ms)
  roofline     the step kernel against the measured HBM copy bandwidth
  cpu_baseline the oracle (C restatement, all host cores) on a bounded sample
  async        ParallelPSOKernel(global_update=false) on the same workload
  hybrid       HybridPSO: 65,536 x 10-D Rosenbrock and Ackley, 200 sync PSO
               iterations then L-BFGS (m=10, Armijo 1e-4, <=100 iterations,
               gtol 1e-5) on every particle
  ode_batch    512 Lotka-Volterra + 512 FitzHugh-Nagumo fits (particles per fit
               from {256, 1024, 4096}, 100 iterations, RK4 dt=0.01) in one
               batched launch, against the same fits solved one at a time
  served       the mixed request stream of the served workload (Rosenbrock /
               Rastrigin / Ackley / Lotka-Volterra fit / MLP fit, dim U{2..64},
               particles U{256..16384}, maxiters U{100..2000}) through the
               continuous-batching server: a closed-loop saturation run, a
               Poisson(2000/s) open-loop run, p50/p99 time to solution, against
               one-at-a-time plain solves; served_without_mlp the same without
               MLP fits (whose tensor-core kernel fills the GPU on its own)
  mlp          the MLP fit (16,384 particles x 577 parameters, 1024 samples)
               by sync PSO: particle-iters/s and the tanh rate against the
               special-function pipe
  configs      C1 (3-D Rosenbrock, 1000 particles, 500 iterations) on the GPU
               and the oracle; C2 with Rosenbrock
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

# the server keeps up to 16 launches in flight on separate streams; give them
# separate hardware queues (must be set before the CUDA context exists)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

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


def cpu_oracle_rate_fast(n: int, iters: int, threads: int):
    """The same sample on the oracle's timing-only fast build (-O3, fused
    multiply-adds, unrolled), in a child process: (particle-iters/s, seconds)."""
    env = dict(os.environ, PPS_ORACLE_BUILD="fast")
    code = f"import bench; r, s = bench.cpu_oracle_rate({n}, {iters}, {threads}); print(r, s)"
    out = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), env=env, capture_output=True, text=True,
                         check=True, timeout=900)
    r, sec = out.stdout.split()[-2:]
    return float(r), float(sec)


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


# --------------------------------------------------------------------------
# further workloads (each returns a dict for the JSON line)
# --------------------------------------------------------------------------
def run_hybrid(pps) -> dict:
    """HybridPSO: 65,536 x 10-D Rosenbrock and Ackley, bounds [-5, 5], 200
    synchronous PSO iterations, then L-BFGS from every particle's best."""
    out = {"workload": "HybridPSO 65536 x 10-D, 200 sync PSO iterations + per-particle L-BFGS "
                       "(m=10, Armijo c1=1e-4, <=100 iterations, gtol 1e-5)"}
    n, D = 65536, 10
    for name, prm in (("rosenbrock", [1.0, 100.0]), ("ackley", [20.0, 0.2, 1.0])):
        prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm,
                                       lb=np.full(D, -5.0, np.float32), ub=np.full(D, 5.0, np.float32))
        with pps.Swarm(prob, n, seed=7) as sw:
            sw.init()
            sw.sync_run(20)  # warm
            sw.init()
            pso_ms = sw.sync_run(200)
            _, pso_cost, _ = sw.gbest()
            # the first call loads the kernel's module; the local stage leaves
            # the swarm unchanged, so the second call is the timed one
            sw.local_stage("lbfgs", history=10, maxiters=100, armijo_c1=1e-4, gtol=1e-5)
            u, f, idx, local_ms = sw.local_stage("lbfgs", history=10, maxiters=100, armijo_c1=1e-4, gtol=1e-5)
            iters = sw.get(7)
            sw.local_stage("bfgs", maxiters=100, gtol=1e-5)  # warm
            _, fb, _, bfgs_ms = sw.local_stage("bfgs", maxiters=100, gtol=1e-5)
        out[name] = {"pso_ms": pso_ms, "pso_particle_iters_per_s": n * 200 / (pso_ms / 1e3),
                     "pso_best": pso_cost, "local_ms": local_ms, "local_particles_per_s": n / (local_ms / 1e3),
                     "local_mean_iters": float(np.mean(iters)), "best": f, "solve_ms": pso_ms + local_ms,
                     "broyden_ms": bfgs_ms, "broyden_best": fb}
    return out


def _ode_fits(pps, count_each=512, seed=0):
    rng = np.random.default_rng(seed)
    fits = []
    for k in range(2 * count_each):
        prob, truth = pps.ode.synthetic_fit("lv" if k < count_each else "fhn", k)
        fits.append((prob, truth, int(rng.choice([256, 1024, 4096]))))
    return fits


def run_ode_batch(pps, count_each=512) -> dict:
    """512 LV + 512 FHN fits in one batched launch vs the same fits one at a
    time (a sample, scaled to all 1024)."""
    fits = _ode_fits(pps, count_each)
    with pps.Batch() as b:
        for k, (p, tr, n) in enumerate(fits):
            b.add(p, n, maxiters=100, seed=k)
        b.run()  # autotune + warm
        t0 = time.perf_counter()
        ms = b.run()
        wall = time.perf_counter() - t0
        res = [b.result(k) for k in range(len(fits))]
        shape = b.info()
    rel = [float(np.max(np.abs(r[0] - f[1]) / np.abs(f[1]))) for r, f in zip(res, fits)]
    # plain: the same fits solved alone, one after another (a stratified sample)
    sample = list(range(0, count_each, 32)) + list(range(count_each, 2 * count_each, 32))
    plain_ms = {}
    same = True
    for k in sample:
        p, tr, n = fits[k]
        with pps.Swarm(p, n, seed=k) as sw:
            sw.init()
            t0 = time.perf_counter()
            sw.sync_run(100)
            u, c, i = sw.gbest()
            plain_ms[k] = (time.perf_counter() - t0) * 1e3
        same &= bool(np.array_equal(u, res[k][0]) and c == res[k][1])
    lv = [plain_ms[k] for k in sample if k < 512]
    fhn = [plain_ms[k] for k in sample if k >= 512]
    plain_total_s = count_each * (np.mean(lv) + np.mean(fhn)) / 1e3
    return {"workload": f"{count_each} Lotka-Volterra + {count_each} FitzHugh-Nagumo fits, particles per fit from {{256,1024,4096}}, "
                        "100 iterations, RK4 dt=0.01, SSE",
            "batched_device_ms": ms, "batched_wall_s": wall, "batched_solves_per_s": len(fits) / wall,
            "plain_solves_per_s": len(fits) / plain_total_s, "plain_sample": len(sample),
            "speedup_vs_plain": plain_total_s / wall, "same_result_alone_and_batched": same,
            "param_rel_err_median": float(np.median(rel)), "param_rel_err_p90": float(np.percentile(rel, 90)),
            "block_shape": shape}


# the Rastrigin objective written as the CUDA C source of a user objective
USER_RASTRIGIN = """PPS_DEVICE float pps_objective(pps_point x, int dim, const float* p, const float* data,
                                long long ndata) {
  float s = 0.0f;
  for (int i = 0; i < dim; ++i) s = s + (x[i] * x[i] - p[0] * pps_cos2pi(x[i]));
  return p[0] * (float)dim + s;
}
"""

# the same with the fold the step kernel evaluates as each coordinate moves
USER_RASTRIGIN_STREAM = "#define PPS_HAS_STREAM 1\n" + USER_RASTRIGIN + """
typedef struct { float s; } pps_stream;
PPS_DEVICE void pps_stream_start(pps_stream* st, int dim, const float* p, const float* data, long long ndata) {
  st->s = 0.0f;
}
PPS_DEVICE void pps_stream_add(pps_stream* st, int d, float v, int dim, const float* p, const float* data,
                               long long ndata) {
  st->s = st->s + (v * v - p[0] * pps_cos2pi(v));
}
PPS_DEVICE float pps_stream_finish(const pps_stream* st, int dim, const float* p, const float* data,
                                   long long ndata) {
  return p[0] * (float)dim + st->s;
}
"""


def run_user(pps, n: int = N_PARTICLES, iters: int = ITERS) -> dict:
    """C2 Rastrigin (n x 100-D, bounds [-5.12, 5.12]) with f given as CUDA C
    source: the NVRTC-compiled step kernel of a user objective against the
    registered kernel, same seed, same result."""
    lb, ub = np.full(DIM, LO, np.float32), np.full(DIM, HI, np.float32)
    reg = pps.OptimizationProblem(pps.rastrigin, np.zeros(DIM, np.float32), [10.0], lb=lb, ub=ub)
    usr = reg.remake(f=pps.cuda_objective(USER_RASTRIGIN, "rastrigin_source"))
    res = {}

    def measure(key, prob):
        with pps.Swarm(prob, n, seed=2) as sw:
            sw.init()
            sw.sync_run(10)  # warm (the first use loads the compiled library)
            sw.init()
            ms = sw.sync_run(iters)
            res[key] = (ms, sw.gbest())

    def same(key):
        return bool(np.array_equal(res[key][1][0], res["registered"][1][0])
                    and res[key][1][2] == res["registered"][1][2])

    measure("registered", reg)
    measure("source", usr)
    ms = res["source"][0]
    out = {"workload": f"{n} particles x {DIM}-D Rastrigin, {iters} sync iterations, f as CUDA C source "
                       "(NVRTC, 2 particles per thread)",
           "device_ms": ms, "particle_iters_per_s": n * iters / (ms / 1e3),
           "hbm_gbs": n * BYTES_PER_PARTICLE_ITER / (ms / iters / 1e3) / 1e9,
           "registered_device_ms": res["registered"][0], "vs_registered": res["registered"][0] / ms,
           "same_result_as_registered": same("source")}
    try:  # the same source with PPS_HAS_STREAM: the step folds f in registers
        measure("stream", reg.remake(f=pps.cuda_objective(USER_RASTRIGIN_STREAM, "rastrigin_stream")))
        sms = res["stream"][0]
        out["stream"] = {"device_ms": sms, "particle_iters_per_s": n * iters / (sms / 1e3),
                         "hbm_gbs": n * BYTES_PER_PARTICLE_ITER / (sms / iters / 1e3) / 1e9,
                         "vs_registered": res["registered"][0] / sms, "same_result_as_registered": same("stream")}
    except pps.PPSError as e:
        out["stream"] = {"error": str(e)}
    return out


def run_configs(pps) -> dict:
    """The other sync configurations of the workload: C1 (3-D Rosenbrock, p =
    [1, 100], bounds [-1, 10], 1000 particles, 500 iterations: the reference's
    CPU-backend case) on the GPU and on the oracle, and C2 with Rosenbrock
    (2^20 x 100-D, bounds [-5.12, 5.12], 1000 iterations)."""
    out = {}
    c1 = pps.OptimizationProblem(pps.rosenbrock, np.zeros(3, np.float32), [1.0, 100.0],
                                 lb=np.full(3, -1.0, np.float32), ub=np.full(3, 10.0, np.float32))
    with pps.Swarm(c1, 1000, seed=0) as sw:
        sw.init()
        sw.sync_run(500)  # warm
        ms = []
        for k in range(5):
            sw.init()
            ms.append(sw.sync_run(500))
        _, cost, _ = sw.gbest()
    gpu_ms = statistics.median(ms)
    try:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pps_oracle as orc
        op = orc.OracleProblem(1, 3, np.full(3, -1.0, np.float32), np.full(3, 10.0, np.float32), params=[1.0, 100.0])
        cms = []
        for k in range(5):
            ref = orc.OracleSwarm(op, 1000, 0).init()
            t0 = time.perf_counter()
            ref.sync_run(500)
            cms.append((time.perf_counter() - t0) * 1e3)
        cpu = {"ms": statistics.median(cms), "cores": os.cpu_count(), "same_gbest_cost": bool(ref.gcost == cost)}
    except Exception as e:  # the oracle is optional on a machine without its build
        cpu = {"unavailable": str(e)}
    out["c1_rosenbrock_3d_1000x500"] = {"gpu_ms": gpu_ms, "particle_iters_per_s": 1000 * 500 / (gpu_ms / 1e3),
                                        "gbest_cost": cost, "cpu_oracle": cpu}
    c2 = pps.OptimizationProblem(pps.rosenbrock, np.zeros(DIM, np.float32), [1.0, 100.0],
                                 lb=np.full(DIM, LO, np.float32), ub=np.full(DIM, HI, np.float32))
    with pps.Swarm(c2, N_PARTICLES, seed=1) as sw:
        sw.init()
        sw.sync_run(50)  # warm
        sw.init()
        ms = sw.sync_run(ITERS)
    launch_ms = ms / ITERS
    out["c2_rosenbrock_2p20x100"] = {"device_ms": ms, "particle_iters_per_s": N_PARTICLES * ITERS / (ms / 1e3),
                                     "hbm_gbs": N_PARTICLES * BYTES_PER_PARTICLE_ITER / (launch_ms / 1e3) / 1e9}
    # one large Lotka-Volterra fit solved alone (k_sync_step_ode: update, RK4,
    # SSE, personal best and argmin fused, one launch per iteration)
    fit, _ = pps.ode.synthetic_fit("lv", 3)
    with pps.Swarm(fit, 16384, seed=3) as sw:
        sw.init()
        sw.sync_run(5)  # warm
        sw.init()
        ms = sw.sync_run(100)
    steps = 1000 * 16384 * 100  # RK4 steps
    out["ode_lv_16384x100_alone"] = {"device_ms": ms, "particle_iters_per_s": 16384 * 100 / (ms / 1e3),
                                     "rk4_steps_per_s": steps / (ms / 1e3)}
    # the reference's own ode_pso benchmarks: Tsit5 at dt = 0.1, saves every
    # 0.01 on [0, 3] from its continuous extension, 10,000 particles, 100 iterations
    for model in ("lv", "fhn"):
        prob, truth = pps.ode.reference_benchmark_fit(model)
        with pps.Swarm(prob, 10_000, seed=0) as sw:
            sw.init()
            sw.sync_run(5)  # warm
            sw.init()
            ms = sw.sync_run(100)
            u, cost, _ = sw.gbest()
        entry = {"device_ms": ms, "particle_iters_per_s": 10_000 * 100 / (ms / 1e3), "gbest_cost": cost,
                 "max_rel_err_vs_truth": float(np.max(np.abs(u - truth) / truth))}
        try:
            ref = orc.OracleSwarm(orc.ode_fit_problem(prob), 2000, 0).init()
            t0 = time.perf_counter()
            ref.sync_run(10)
            sec = time.perf_counter() - t0
            entry["cpu_oracle"] = {"particle_iters_per_s": 2000 * 10 / sec, "cores": os.cpu_count(),
                                   "sample": "2000 particles x 10 iterations"}
        except Exception as e:  # the oracle is optional on a machine without its build
            entry["cpu_oracle"] = {"unavailable": str(e)}
        out[f"ode_{model}_tsit5_reference_benchmark"] = entry
    # the same LV benchmark with adaptive steps (parameter_estim_ode!(..., Val(true)), reltol 1e-3,
    # abstol 1e-6, first step 0.1)
    prob, truth = pps.ode.reference_benchmark_fit("lv")
    aprob = pps.ode.adaptive(prob)
    with pps.Swarm(aprob, 10_000, seed=0) as sw:
        sw.init()
        sw.sync_run(5)  # warm
        sw.init()
        ms = sw.sync_run(100)
        u, cost, _ = sw.gbest()
    out["ode_lv_tsit5_adaptive_reference_benchmark"] = {
        "device_ms": ms, "particle_iters_per_s": 10_000 * 100 / (ms / 1e3), "gbest_cost": cost,
        "max_rel_err_vs_truth": float(np.max(np.abs(u - truth) / truth)), "reltol": 1e-3, "abstol": 1e-6}
    out["separable_batch_256"] = run_separable_batch(pps)
    return out


def _nvtx_range(name):
    """An NVTX range (ncu --nvtx --nvtx-include) around a region, when torch is importable."""
    import contextlib

    try:
        import torch

        @contextlib.contextmanager
        def rng():
            torch.cuda.nvtx.range_push(name)
            try:
                yield
            finally:
                torch.cuda.nvtx.range_pop()
        return rng()
    except Exception:
        return contextlib.nullcontext()


def run_separable_batch(pps, plain: bool = True) -> dict:
    """Many small separable swarms in one batched launch (the autotuner's first
    run, then the timed run inside the NVTX range "batch_timed") against the
    same swarms solved one at a time (a sample of 32)."""
    rng = np.random.default_rng(5)
    swarms = []
    for k in range(256):
        name = ("rosenbrock", "rastrigin", "ackley")[k % 3]
        D = int(rng.integers(2, 65))
        lo = -5.12 if name == "rastrigin" else -5.0
        obj = pps.REGISTRY[name]
        prob = pps.OptimizationProblem(obj, np.zeros(D, np.float32), list(obj.default_params),
                                       lb=np.full(D, lo, np.float32), ub=np.full(D, -lo, np.float32))
        swarms.append((prob, int(rng.integers(256, 2049))))
    with pps.Batch() as b:
        for k, (prob, n) in enumerate(swarms):
            b.add(prob, n, maxiters=500, seed=k)
        b.run()  # autotune + warm
        with _nvtx_range("batch_timed"):
            t0 = time.perf_counter()
            bms = b.run()
            bwall = time.perf_counter() - t0
        res = [b.result(k) for k in range(len(swarms))]
        shape = b.info()
    out = {"workload": "256 swarms (Rosenbrock / Rastrigin / Ackley, dim U{2..64}, particles U{256..2048}), "
                       "500 iterations, one launch",
           "batched_device_ms": bms, "batched_solves_per_s": len(swarms) / bwall, "block_shape": shape}
    if not plain:
        return out
    same = True
    t0 = time.perf_counter()
    sample = list(range(0, len(swarms), 8))
    for k in sample:
        prob, n = swarms[k]
        with pps.Swarm(prob, n, seed=k) as sw:
            sw.init()
            sw.sync_run(500)
            u, c, i = sw.gbest()
        same &= bool(np.array_equal(u, res[k][0]) and i == res[k][2])
    rate = len(sample) / (time.perf_counter() - t0)
    out.update({"plain_solves_per_s": rate, "speedup_vs_plain": len(swarms) / bwall / rate,
                "same_result_alone_and_batched": same})
    return out


MLP_PARTICLES = 16384
MLP_SAMPLES = 1024
SFU_PER_CLK_PER_SM = 16  # tanh.approx results per clock per SM (special-function pipe)


def run_mlp(pps, iters: int = 100, cpu_seconds: float = 3.0) -> dict:
    """Training the 16 -> 32 tanh -> 1 MLP by ParallelSyncPSOKernel: 16,384
    particles x 577 parameters, 1024 samples of a synthetic teacher, bounds
    [-1, 1].  Each iteration is the position update plus the tensor-core loss
    kernel (bf16 tcgen05 GEMM of the hidden layer, tanh, output layer, MSE)."""
    data, _ = pps.mlp.teacher_task(MLP_SAMPLES, seed=0)
    prob = pps.mlp.mlp_problem(data)
    n = MLP_PARTICLES
    with pps.Swarm(prob, n, seed=3) as sw:
        sw.init()
        sw.sync_run(10)  # warm
        sw.init()
        _, first, _ = sw.gbest()
        with ClockSampler(0) as clk:
            ms = sw.sync_run(iters)
        clocks = clk.summary()
        _, last, _ = sw.gbest()
    evals = n * iters
    sec = ms / 1e3
    gemm_flops = 2.0 * MLP_SAMPLES * 16 * 32 * evals
    tanh = MLP_SAMPLES * 32.0 * evals
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    sfu_peak = SFU_PER_CLK_PER_SM * 152 * sm_mhz * 1e6
    out = {"workload": f"MLP fit by sync PSO: {n} particles x 577 parameters (16 -> 32 tanh -> 1), "
                       f"{MLP_SAMPLES} samples of a synthetic teacher, MSE, {iters} iterations",
           "device_ms": ms, "particle_iters_per_s": evals / sec, "ms_per_iteration": ms / iters,
           "hidden_gemm_tflops": gemm_flops / sec / 1e12, "tanh_per_s": tanh / sec,
           "sfu_peak_tanh_per_s": sfu_peak, "sfu_frac": tanh / sec / sfu_peak,
           "loss_first": first, "loss_after": last, "clocks": clocks}
    # the oracle on the host cores (float64 loss), a bounded sample
    try:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pps_oracle as orc
        op = orc.OracleProblem(6, 577, prob.lb, prob.ub, mlp_data=data)
        ns = 64
        ref = orc.OracleSwarm(op, ns, 3).init()
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < cpu_seconds:
            ref.sync_run(1)
            k += 1
        cs = time.perf_counter() - t0
        out["cpu_oracle"] = {"particle_iters_per_s": ns * k / cs, "cores": os.cpu_count(),
                             "sample": f"{ns} particles x {k} iterations"}
    except Exception as e:  # the oracle is optional on a machine without its build
        out["cpu_oracle"] = {"unavailable": str(e)}
    return out


def _request_pool(pps, count, seed, with_mlp=True):
    """Mixed requests: objective uniform over Rosenbrock, Rastrigin, Ackley,
    the Lotka-Volterra fit and (with_mlp) the MLP fit; LV fits reuse a pool of
    64 synthetic datasets, MLP fits a pool of 8 teacher tasks (1024 samples)."""
    rng = np.random.default_rng(seed)
    lv_pool = [pps.ode.synthetic_fit("lv", 10_000 + k)[0] for k in range(64)]
    mlp_pool = [pps.mlp.mlp_problem(pps.mlp.teacher_task(MLP_SAMPLES, seed=20_000 + k)[0]) for k in range(8)] \
        if with_mlp else []
    kinds = 5 if with_mlp else 4
    reqs = []
    for _ in range(count):
        kind = int(rng.integers(kinds))
        n = int(rng.integers(256, 16385))
        iters = int(rng.integers(100, 2001))
        s = int(rng.integers(0, 2**62))
        if kind == 3:
            reqs.append((lv_pool[int(rng.integers(64))], n, iters, s))
            continue
        if kind == 4:
            reqs.append((mlp_pool[int(rng.integers(8))], n, iters, s))
            continue
        D = int(rng.integers(2, 65))
        name = ("rosenbrock", "rastrigin", "ackley")[kind]
        lo = -5.12 if name == "rastrigin" else -5.0
        obj = pps.REGISTRY[name]
        reqs.append((pps.OptimizationProblem(obj, np.zeros(D, np.float32), list(obj.default_params),
                                             lb=np.full(D, lo, np.float32), ub=np.full(D, -lo, np.float32)),
                     n, iters, s))
    return reqs


def run_served(pps, args, with_mlp=True) -> dict:
    """The served mixed stream through the continuous-batching server: a
    closed-loop saturation run, a Poisson(2000/s) open-loop run, p50/p99 time
    to solution, against the same requests solved one at a time (plain)."""
    cfg = dict(memory_budget=24 << 30, max_launches=32, max_pack=128, threads=256, ppt=2, tick_us=200.0,
               single_min_n=2048)
    mix = "Rosenbrock, Rastrigin, Ackley, Lotka-Volterra fit" + (", MLP fit (577 parameters, 1024 samples)"
                                                                 if with_mlp else "")
    out = {"workload": f"mixed stream: objective U{{{mix}}}, dim U{{2..64}}, particles U{{256..16384}}, "
                       "maxiters U{100..2000}", "server": dict(cfg)}
    count = args.serve_requests_mlp if with_mlp else args.serve_requests
    window = args.serve_seconds_mlp if with_mlp else args.serve_seconds
    # closed loop: all requests submitted at once, throughput at saturation
    reqs = _request_pool(pps, count, 1, with_mlp)
    with pps.Server(**cfg) as srv:
        t0 = time.perf_counter()
        ts = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
        res = [srv.wait(t) for t in ts]
        wall = time.perf_counter() - t0
        st = srv.stats()
    out["closed_loop"] = {"requests": len(reqs), "wall_s": wall, "solves_per_s": len(reqs) / wall,
                          "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "launches": st["launches"],
                          "mean_pack": st["mean_pack"], "arena_peak_bytes": st["arena_peak_bytes"]}
    # plain: the same requests one at a time through solve()
    sample = reqs[:min(len(reqs), 100)]
    t0 = time.perf_counter()
    same = True
    for k, (p, n, it, s) in enumerate(sample):
        sol = pps.solve(p, pps.ParallelSyncPSOKernel(n), maxiters=it, seed=s)
        same &= bool(np.array_equal(sol.u, res[k][0]))
    plain = len(sample) / (time.perf_counter() - t0)
    out["plain_solves_per_s"] = plain
    out["plain_sample"] = len(sample)
    out["speedup_vs_plain"] = out["closed_loop"]["solves_per_s"] / plain
    out["same_result_alone_and_served"] = same
    if not with_mlp:
        # the same requests with every separable request batched whatever its size
        # (ODE fits of 2048 particles or more still run on their own), packs of <= 32:
        # more swarms per launch, each result the same as with the default routing
        bcfg = dict(cfg, single_min_n=-1, ode_single_min_n=2048, max_pack=32)
        with pps.Server(**bcfg) as srv:
            t0 = time.perf_counter()
            ts = [srv.submit(p, n, maxiters=it, seed=s) for (p, n, it, s) in reqs]
            bres = [srv.wait(t) for t in ts]
            bwall = time.perf_counter() - t0
            bst = srv.stats()
        out["closed_loop_batched_routing"] = {
            "server": bcfg, "wall_s": bwall, "solves_per_s": len(reqs) / bwall,
            "speedup_vs_plain": len(reqs) / bwall / plain, "p50_ms": bst["p50_ms"], "p99_ms": bst["p99_ms"],
            "launches": bst["launches"], "mean_pack": bst["mean_pack"],
            "same_results_as_default_routing": all(
                np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(np.float32(a[1]), np.float32(b[1]),
                                                                               equal_nan=True) and a[2] == b[2]
                for a, b in zip(res, bres))}
    # open loop: Poisson arrivals at 2000/s over the window, then drain
    out["open_loop"] = _open_loop(pps, cfg, 2000.0, window, with_mlp, seed=2)
    out["open_loop"]["note"] = "offered load above the measured closed-loop capacity: latency includes queueing"
    if not with_mlp and args.serve_sustained_s > 0:
        # and at a load the server sustains (about 78 % of its closed-loop
        # capacity), where p50 / p99 are service times, not queueing
        out["open_loop_sustained"] = _open_loop(pps, cfg, 250.0, args.serve_sustained_s, with_mlp, seed=4)
    return out


def _open_loop(pps, cfg, rate, window, with_mlp, seed) -> dict:
    """Poisson arrivals at `rate` per second over `window` seconds, then drain."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, int(rate * window * 1.2) + 8))
    arrivals = arrivals[arrivals < window]
    pool = _request_pool(pps, len(arrivals), seed + 1, with_mlp)
    with pps.Server(**cfg) as srv:
        t0 = time.perf_counter()
        tickets = []
        for k, at in enumerate(arrivals):
            while time.perf_counter() - t0 < at:
                time.sleep(0.0001)
            p, n, it, s = pool[k]
            tickets.append(srv.submit(p, n, maxiters=it, seed=s))
        submit_s = time.perf_counter() - t0
        for t in tickets:
            srv.wait(t)
        wall = time.perf_counter() - t0
        st = srv.stats()
    return {"offered_per_s": rate, "arrival_window_s": window, "requests": len(tickets), "submit_s": submit_s,
            "drain_wall_s": wall, "solves_per_s": len(tickets) / wall, "p50_ms": st["p50_ms"],
            "p99_ms": st["p99_ms"], "max_ms": st["max_ms"], "launches": st["launches"],
            "mean_pack": st["mean_pack"], "arena_peak_bytes": st["arena_peak_bytes"]}


def run_sharded(pps, args, rank, world, local, dist) -> int:
    """--shard: the 2^20 x 100-D swarm split into `world` particle ranges, one
    per rank; every iteration is the shard's step, an all-gather of the ranks'
    records (NCCL) and the global best applied, all on the shard's stream.
    The whole job processes the same 2^20 particles per iteration at every N
    (strong scaling)."""
    import torch

    prob = make_problem(pps)
    iters = args.iters
    torch.cuda.set_device(local)
    sh = pps.ShardedSwarm(prob, N_PARTICLES, rank, world, seed=0)
    stream = sh.shard.stream
    for k in range(args.warmup):
        sh.init()
        sh.sync_run(iters)
    step_ms = []
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            sh.init()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sh.sync_run(iters)  # ends with a wait for the shard's stream
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    if dist:
        dist.barrier()
    total_ms = multi_max(sum(step_ms), dist, local)
    _, gcost, gidx = sh.gbest()
    count = sh.shard.n
    sh.close()
    value = N_PARTICLES * iters * args.steps / (total_ms / 1e3)
    launch_ms = total_ms / (args.steps * iters)
    algo_bytes = count * BYTES_PER_PARTICLE_ITER
    peak, peak_src = measured_hbm_peak()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "particles": N_PARTICLES, "dim": DIM, "iterations_per_step": iters,
                           "objective": "rastrigin", "algorithm": "ParallelSyncPSOKernel",
                           "l2": "inputs larger than L2: 2.1 GB of swarm state streamed per iteration",
                           "parallelism": f"one swarm in {world} particle-range shard(s), one per GPU, "
                                          "all-gather of the shards' best-particle records per iteration"},
                "e2e": None,
                "gpu_launches": args.steps * (2 * iters + 3),
                "roofline": {"bound": "hbm", "unit": "GB/s", "kernel": "k_sync_step<Rastrigin> on one shard",
                             "achieved_per_iteration_incl_exchange": algo_bytes / (launch_ms / 1e3) / 1e9,
                             "peak": peak, "peak_source": peak_src,
                             "frac": algo_bytes / (launch_ms / 1e3) / 1e9 / peak,
                             "algorithmic_bytes_per_launch": algo_bytes, "avg_iteration_ms": launch_ms,
                             "traffic": None},
                "cpu_baseline": None, "clocks": clk.summary(), "final_gbest_cost": gcost, "final_gbest_index": gidx}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def multi_max(value, dist, local):
    from parallelparticleswarms import multi

    return multi.max_over_ranks(value, dist, f"cuda:{local}")


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
    ap.add_argument("--no-extras", action="store_true", help="skip the hybrid, ODE-batch and served measurements")
    ap.add_argument("--mlp-iters", type=int, default=100, help="iterations of the MLP-fit measurement")
    ap.add_argument("--user-n", type=int, default=N_PARTICLES,
                    help="particles of the user-objective (CUDA C source) measurement")
    ap.add_argument("--only", choices=["sync", "async", "hybrid", "ode", "serve", "mlp", "configs", "user", "batch"],
                    default=None,
                    help="run one workload only (for profiling); prints its result")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU-baseline sample")
    ap.add_argument("--serve-requests", type=int, default=1500,
                    help="requests of the closed-loop served run without MLP fits")
    ap.add_argument("--serve-seconds", type=float, default=1.0,
                    help="arrival window of the open-loop served run without MLP fits")
    ap.add_argument("--serve-sustained-s", type=float, default=4.0,
                    help="arrival window of the open-loop served run at 250 requests/s (0: skip)")
    ap.add_argument("--serve-requests-mlp", type=int, default=400,
                    help="requests of the closed-loop served run of the full mix (MLP fits included)")
    ap.add_argument("--serve-seconds-mlp", type=float, default=0.25,
                    help="arrival window of the open-loop served run of the full mix")
    ap.add_argument("--ode-fits", type=int, default=512, help="fits of each model in the batched ODE run")
    ap.add_argument("--shard", action="store_true",
                    help="one swarm of 2^20 particles split by particle ranges over the ranks, one global-best "
                         "exchange (all-gather of 416-byte records) per iteration: strong scaling")
    args = ap.parse_args()
    from parallelparticleswarms import multi

    rank, world, local = multi.rank_env()

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
    seed0 = multi.swarm_seed(0, rank)

    if args.only in ("hybrid", "ode", "serve", "mlp", "configs", "user", "batch"):
        fn = {"hybrid": lambda: run_hybrid(pps), "ode": lambda: run_ode_batch(pps, args.ode_fits),
              "serve": lambda: {"served": run_served(pps, args, True),
                                "served_without_mlp": run_served(pps, args, False)},
              "mlp": lambda: run_mlp(pps, args.mlp_iters), "configs": lambda: run_configs(pps),
              "user": lambda: run_user(pps, args.user_n),
              "batch": lambda: run_separable_batch(pps, plain=False)}[args.only]
        if rank == 0:
            print(json.dumps({args.only: fn()}), flush=True)
        return 0
    if args.shard:
        return run_sharded(pps, args, rank, world, local, dist)
    if args.only == "async":
        sa = pps.Swarm(prob, N_PARTICLES, seed=seed0 + 1)
        sa.init()
        ams = sa.async_run(iters)
        if rank == 0:
            print(json.dumps({"async": {"ms": ams, "particle_iters_per_s": N_PARTICLES * iters / (ams / 1e3)}}))
        return 0

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
    total_ms = multi.max_over_ranks(sum(step_ms), dist, f"cuda:{local}")
    _, gcost, _ = sw.gbest()
    sw.close()
    value = multi.job_throughput(N_PARTICLES * iters * args.steps, world, total_ms)
    launch_ms = total_ms / (args.steps * iters)
    algo_bytes = N_PARTICLES * BYTES_PER_PARTICLE_ITER
    achieved = algo_bytes / (launch_ms / 1000.0) / 1e9
    peak, peak_src = measured_hbm_peak()
    traffic = profiled_traffic()

    # ---- async at the same size -----------------------------------------
    async_rate = None
    if rank == 0 and not args.no_async and args.only is None:
        sa = pps.Swarm(prob, N_PARTICLES, seed=seed0 + 1)
        sa.init()
        sa.async_run(50)
        sa.init()
        ams = sa.async_run(iters)
        async_rate = N_PARTICLES * iters / (ams / 1000.0)
        sa.close()

    # ---- end to end through solve() with host buffers --------------------
    e2e = None
    if not args.no_e2e and args.only is None:
        alg = pps.ParallelSyncPSOKernel(N_PARTICLES)
        pps.solve(prob, alg, maxiters=iters, seed=seed0)  # warm
        barrier()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 3))
        for k in range(e2e_steps):
            sol = pps.solve(prob, alg, maxiters=iters, seed=seed0 + k)
            _ = sol.objective
        barrier()
        e2e_s = multi.max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{local}")
        t1 = time.perf_counter()
        original = np.asarray(sol.original)  # every position to the host, once
        original_ms = (time.perf_counter() - t1) * 1e3
        h2d = 4 * (3 * DIM + 1) + 4 * DIM  # lb, ub, u0, p; the point u of f(u)
        d2h = 4 * DIM + 4 + 8 + 4  # u, gbest cost and index, f(u)
        e2e = {"value": N_PARTICLES * iters * e2e_steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
               "original_to_host_ms": original_ms, "original_shape": list(original.shape),
               "path": "parallelparticleswarms.solve -> libpps_cuda.so C ABI (pps_swarm_create/init/sync_run/"
                       "get_gbest/field_copy_create/eval_objective)"}

    # ---- CPU baseline (oracle on the host cores) --------------------------
    extras = {}
    if rank == 0 and not args.no_extras and args.only is None:
        def extra(fn):
            # a failed extra measurement is reported in its place; it does not cost the headline line
            try:
                return fn()
            except Exception as e:
                return {"error": f"{type(e).__name__}: {e}"[:300]}

        extras["hybrid"] = extra(lambda: run_hybrid(pps))
        extras["ode_batch"] = extra(lambda: run_ode_batch(pps, args.ode_fits))
        extras["served"] = extra(lambda: run_served(pps, args, True))
        extras["served_without_mlp"] = extra(lambda: run_served(pps, args, False))
        extras["mlp"] = extra(lambda: run_mlp(pps, args.mlp_iters))
        extras["configs"] = extra(lambda: run_configs(pps))
        extras["user_objective"] = extra(lambda: run_user(pps, args.user_n))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.only is None:
        threads = os.cpu_count() or 1
        n_s = 1 << 18
        rate0, _ = cpu_oracle_rate(n_s, 1, threads)  # size the sample to about --cpu-seconds
        it_s = max(1, min(200, int(args.cpu_seconds * rate0 / n_s)))
        rate, secs = cpu_oracle_rate(n_s, it_s, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n_s} particles x {DIM}-D Rastrigin, {it_s} sync iterations ({secs:.1f} s), "
                         "C restatement threaded over particles (-O2, no contraction: the checker's bits)"}
        try:
            frate, fsecs = cpu_oracle_rate_fast(n_s, it_s, threads)
            cpu["fast_build"] = {"value": frate, "unit": UNIT, "seconds": fsecs,
                                 "flags": "-O3 -ffp-contract=fast -funroll-loops (timing only: different bits)"}
        except Exception as e:  # the figure is informative; the baseline above stands without it
            cpu["fast_build"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}

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
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
