/*
 * pps.h -- C ABI of libpps_cuda.so, the GB300 (sm_103a) particle-swarm engine
 * that sits below ParallelParticleSwarms.jl's solve/init/solve!/reinit! API.
 *
 * Conventions
 *   - Every entry point returns a pps_status; on failure pps_last_error()
 *     returns a message for the calling thread.  No exception or longjmp
 *     crosses the ABI.
 *   - Pointers are HOST pointers unless a name says otherwise; the library
 *     owns every device allocation it makes.
 *   - Arrays of particle data are structure-of-arrays, particle fastest:
 *     element (particle i, dim d) of an n-particle array is at [d*n + i].
 *     The reference keeps an array of SPSOParticle structs
 *     (src/ParallelParticleSwarms.jl:34-40); pps_get_particles /
 *     pps_set_particles move a swarm in that record layout.
 *   - A pps_swarm handle owns one CUDA stream.  A handle is not thread-safe;
 *     distinct handles may be used from distinct threads.
 *   - All arithmetic is IEEE binary32 (the reference's Float32 problems).
 */
#ifndef PPS_H
#define PPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPS_VERSION 100 /* 0.1.0 */

#if defined(__GNUC__)
#define PPS_API __attribute__((visibility("default")))
#else
#define PPS_API
#endif

typedef enum pps_status {
  PPS_OK = 0,
  PPS_EINVAL = 1,   /* bad argument (the reference raises ArgumentError / AssertionError) */
  PPS_ENOMEM = 2,   /* device or host allocation failed */
  PPS_ECUDA = 3,    /* a CUDA call failed */
  PPS_ETIMEOUT = 4, /* a bounded device-side wait gave up */
  PPS_EBUSY = 5,    /* result not ready yet */
  PPS_ENOTSUP = 6,  /* valid request this build does not support */
  PPS_ENODEV = 7    /* no usable CUDA device */
} pps_status;

/* Objective registry.  The reference compiles an arbitrary Julia closure
 * into its kernels (src/kernels.jl:33); a C ABI cannot take a closure, so the
 * engine evaluates a registered set selected by id with a float parameter
 * vector (the reference's `p`). */
typedef enum pps_objective {
  PPS_OBJ_SPHERE = 0,     /* sum x_i^2 */
  PPS_OBJ_ROSENBROCK = 1, /* sum_{i<D} p2 (x_{i+1}-x_i^2)^2 + (p1-x_i)^2; p=(p1,p2), default (1,100) */
  PPS_OBJ_RASTRIGIN = 2,  /* A D + sum (x_i^2 - A cos 2 pi x_i); p=(A), default 10 */
  PPS_OBJ_ACKLEY = 3,     /* -a exp(-b sqrt(mean x^2)) - exp(mean cos 2 pi k x) + a + e; p=(a,b,k) default (20,0.2,1) */
  PPS_OBJ_LV_FIT = 4,     /* SSE of an RK4 Lotka-Volterra solve vs observations (data) */
  PPS_OBJ_FHN_FIT = 5,    /* SSE of an RK4 FitzHugh-Nagumo solve vs observations (data) */
  PPS_OBJ_MLP = 6,        /* MSE of a 2-layer tanh MLP on a sample set (data) */
  PPS_OBJ_SHIFTED_SPHERE = 7, /* sum (x_i - p_i)^2, p_i = 0 past nparams: the objective of the
                                 reference's constraint test (test/constraints.jl:7) */
  /* the closed-form objectives of the reference's L-BFGS tests (test/lbfgs.jl:20-26) */
  PPS_OBJ_BEALE = 16,
  PPS_OBJ_BOOTH = 17,
  PPS_OBJ_HIMMELBLAU = 18,
  PPS_OBJ_QUADRATIC = 19,         /* p1 (x1-1)^2 + (x2+2)^2 */
  PPS_OBJ_BOUNDARY_QUADRATIC = 20, /* (x1+1)^2 */
  /* ids handed out by pps_objective_register, in registration order */
  PPS_OBJ_USER_BASE = 256
} pps_objective;

/* An OptimizationProblem(f, u0, p; lb, ub) (SciMLBase) restated. */
typedef struct pps_problem {
  int32_t objective;     /* pps_objective */
  int32_t dim;           /* length(u0) */
  const float* lb;       /* dim floats; NULL means -Inf (check_init_bounds, src/utils.jl:310-318) */
  const float* ub;       /* dim floats; NULL means +Inf */
  const float* u0;       /* dim floats; NULL means zeros (used by the unbounded sampler) */
  const float* params;   /* objective parameters p */
  int32_t nparams;
  const float* data;     /* objective data (observations / samples), may be NULL */
  int64_t ndata;         /* floats in data */
  /* Constraints g_k(x) <= 0 (OptimizationFunction(f; cons) with lcons = -Inf, ucons = 0),
   * handled by the reference's penalty calc_penalty (src/utils.jl:320-372, h = sqrt,
   * theta_default, gamma_default) in init and the sync / queue-lock steps.  A C ABI takes
   * no Julia closure, so each constraint has the registered form
   *   g_k(x) = c_k + sum_i a_ki x_i + b_ki x_i^2,
   * cons = ncons rows of (c_k, a_k[dim], b_k[dim]) floats, 0 <= ncons <= 4. */
  int32_t ncons;
  const float* cons;
} pps_problem;

typedef struct pps_swarm pps_swarm;

/* samplers (src/algorithms.jl:33-37 GPUUniformSampler / GPUUnboundedSampler) */
enum {
  PPS_SAMPLER_AUTO = 0,      /* unbounded if every bound is infinite, else uniform (src/init.jl:102-106) */
  PPS_SAMPLER_UNIFORM = 1,   /* x = U (ub - lb) + lb           (src/utils.jl:57-84) */
  PPS_SAMPLER_UNBOUNDED = 2, /* x = u0 + U |u0| or U if u0 = 0 (src/utils.jl:23-55) */
  /* Latin hypercube (init(...; sampler = LatinHypercubeSample()), src/init.jl:15-34): in each dim
   * the n strata are dealt to the particles by a random permutation (a keyed Feistel bijection of
   * [0, n)), x = ((stratum + U) / n) (ub - lb) + lb; needs finite bounds */
  PPS_SAMPLER_LHS = 3
};

/* swarm flags */
enum {
  /* The CPU-backend sync loop takes the next global best's position from the
   * winner's CURRENT position, not its personal best
   * (src/lowerlevel_solve.jl:59-60).  Off: the GPU semantics
   * (src/lowerlevel_solve.jl:31). */
  PPS_FLAG_GBEST_FROM_POSITION = 1u
};

/* state fields for pps_get_state / pps_set_state */
enum {
  PPS_FIELD_POSITION = 0, /* dim*n */
  PPS_FIELD_VELOCITY = 1, /* dim*n */
  PPS_FIELD_PBEST = 2,    /* dim*n */
  PPS_FIELD_PCOST = 3,    /* n */
  PPS_FIELD_COST = 4,     /* n */
  /* results of the last HybridPSO local stage (read-only) */
  PPS_FIELD_LOCAL_X = 5,     /* dim*n: each particle's local optimum */
  PPS_FIELD_LOCAL_F = 6,     /* n: its objective, non-finite -> +Inf */
  PPS_FIELD_LOCAL_ITERS = 7  /* n: iterations used (as float) */
};

typedef struct pps_swarm_info {
  int64_t n;
  int32_t dim;
  int32_t objective;
  uint32_t iteration;   /* iterations run since the last pps_swarm_init */
  int32_t async_lanes;  /* threads per particle of pps_async_run */
  int32_t async_slice;  /* dims per lane of pps_async_run (even) */
  int32_t device;
  uint64_t seed;
  uint64_t device_bytes;
} pps_swarm_info;

/* ---- library ---- */
PPS_API int32_t pps_version(void);
PPS_API const char* pps_last_error(void);
PPS_API int pps_device_count(int32_t* count);
/* make `device` current for the calling thread (swarms are created on the
 * current device; the reference selects it through its backend object) */
PPS_API int pps_set_device(int32_t device);

/* ---- swarm lifetime: init (src/init.jl:56-115) / reinit! (src/init.jl:117-141) ---- */
/* Allocates the swarm on the current device.  n >= 1, 1 <= dim <= 4096. */
PPS_API int pps_swarm_create(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags,
                     pps_swarm** out);
PPS_API int pps_swarm_destroy(pps_swarm* s);
/* Samples positions, zero velocities, evaluates costs and selects the initial
 * global best (gpu_init_particles!, src/utils.jl:23-84; src/init.jl:38-54).
 * Resets the iteration counter. */
PPS_API int pps_swarm_init(pps_swarm* s, int32_t sampler);
PPS_API int pps_swarm_info_get(pps_swarm* s, pps_swarm_info* info);

/* ---- the PSO step ---- */
/* ParallelSyncPSOKernel: maxiters synchronous iterations, global best
 * recomputed after each (src/lowerlevel_solve.jl:1-65, src/kernels.jl:1-26,
 * 127-194).  w is damped by wdamp after each iteration.  device_ms (may be
 * NULL) receives the device time of the iteration loop. */
PPS_API int pps_sync_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                 float* device_ms);
/* ParallelPSOKernel(global_update=false): one launch runs all iterations,
 * each particle against a private global best (src/kernels.jl:196-225). */
PPS_API int pps_async_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                  float* device_ms);
/* ParallelPSOKernel(global_update=true) (src/kernels.jl:38-125,
 * src/lowerlevel_solve.jl:67-93).  The reference publishes block bests under
 * a spin lock while other blocks read the global best mid-kernel, so its
 * result depends on scheduling.  This engine publishes through a lock-free
 * 64-bit atomicMin and lets every block read the previous iteration's best:
 * the interleaving in which all reads precede all writes, i.e. the
 * synchronous iteration. */
PPS_API int pps_queue_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                  float* device_ms);

/* ---- HybridPSO local stage (src/hybrid.jl:47-158) ---- */
typedef struct pps_local_opts {
  int32_t history;        /* L-BFGS pairs m (1..16); ignored by the Broyden stage */
  int32_t maxiters;       /* local_maxiters (the reference's default is 50) */
  float armijo_c1;        /* sufficient-decrease constant of the backtracking search */
  float gtol;             /* stop when ||projected gradient|| (L-BFGS) or ||grad|| (Broyden) <= gtol */
  int32_t max_backtracks; /* halvings of the step before a search fails */
} pps_local_opts;
/* HybridPSO{SimpleLBFGS}: one projected L-BFGS per particle from its personal
 * best within [lb, ub] (lbfgs_run!, src/lbfgs.jl:9-21), then the argmin over
 * the results (src/hybrid.jl:145-146).  u (dim floats), f and idx receive the
 * best local result; every particle's result is in PPS_FIELD_LOCAL_*.
 * dim <= 64. */
PPS_API int pps_hybrid_lbfgs(pps_swarm* s, const pps_local_opts* opts, float* u, float* f, int64_t* idx,
                             float* device_ms);
/* HybridPSO{BFGS}: Broyden's method on grad f = 0 from every particle's current
 * position, gradient 1e15 outside the box grown by twice its width
 * (simplebfgs_run!, src/hybrid.jl:15-45), then the argmin.  dim <= 16. */
PPS_API int pps_hybrid_bfgs(pps_swarm* s, const pps_local_opts* opts, float* u, float* f, int64_t* idx,
                            float* device_ms);

/* ---- batches: many independent swarms in one persistent launch ---- */
/* No single reference call does this: the reference solves one problem per
 * solve() (src/solve.jl:61-67) or one ODE fit per parameter_estim_ode!
 * (src/ode_pso.jl:113-170).  Each added swarm is a full synchronous solve
 * (sampling, maxiters iterations, global best from personal bests) with the
 * same results as pps_swarm_create + pps_swarm_init + pps_sync_run on it.
 * Objectives: sphere, Rosenbrock, Rastrigin, Ackley (dim <= 1024) and the
 * ODE fits; n <= 65536 per swarm. */
typedef struct pps_batch pps_batch;
PPS_API int pps_batch_create(pps_batch** out);
PPS_API int pps_batch_destroy(pps_batch* b);
/* queue one swarm; *slot identifies it in the results */
PPS_API int pps_batch_add(pps_batch* b, const pps_problem* prob, int64_t n, uint64_t seed, int32_t maxiters,
                          float w, float wdamp, float c1, float c2, int32_t* slot);
/* solve every queued swarm in one launch (longest work first); the block
 * shape comes from the autotuner unless pps_batch_set_shape fixed it */
PPS_API int pps_batch_run(pps_batch* b, float* device_ms);
/* threads in {128, 256, 512}, ppt (particles per thread) in {1, 2};
 * (0, 0) returns to autotuning */
PPS_API int pps_batch_set_shape(pps_batch* b, int32_t threads, int32_t ppt);
PPS_API int pps_batch_info(pps_batch* b, int32_t* nswarms, int32_t* threads, int32_t* ppt,
                           uint64_t* device_bytes);
PPS_API int pps_batch_result(pps_batch* b, int32_t slot, float* u, float* cost, int64_t* idx);
PPS_API int pps_batch_get_state(pps_batch* b, int32_t slot, int32_t field, float* out);

/* ---- serving: continuous batching of arriving problems ---- */
/* No counterpart in the reference (one solve() owns the device at a time).
 * A worker thread admits submitted problems first-come first-served while
 * their swarm state fits in a device arena of memory_budget bytes, packs them
 * into batched launches (the kernel of pps_batch_run) and keeps up to
 * max_launches launches in flight on separate streams, so requests that
 * arrive while others run start on the SMs those leave free.  Each result
 * equals the problem's solve alone (same seed) bit for bit. */
typedef struct pps_serve_config {
  uint64_t memory_budget; /* HBM arena for swarm state, bytes (0: 8 GiB) */
  int32_t max_launches;   /* launches in flight (0: 8, at most 64) */
  int32_t max_pack;       /* swarms per launch (0: 512, at most 4096) */
  int32_t threads;        /* block size of the batched kernel (0: 256) */
  int32_t ppt;            /* particles per thread (0: 1) */
  double tick_us;         /* while launches are in flight, the oldest queued request
                             waits at most this long for a fuller pack */
  int32_t single_min_n;   /* requests with at least this many particles run as a swarm
                             of their own with the multi-block step kernels, like a
                             plain solve, instead of in a batched launch (0: 2048,
                             negative: only MLP fits, which always do) */
  int32_t ode_single_min_n; /* the same threshold for ODE fits (0: single_min_n; negative:
                             ODE fits of any size are batched) */
} pps_serve_config;
typedef struct pps_serve_stats {
  uint64_t submitted, completed, launches;
  double solves_per_s;    /* completed / (last completion - first submission) */
  double p50_ms, p99_ms, mean_ms, max_ms; /* time to solution: submit -> result ready */
  double mean_pack;       /* swarms per launch */
  uint64_t arena_bytes, arena_peak_bytes;
  int32_t queued, running;
} pps_serve_stats;
typedef struct pps_server pps_server;
PPS_API int pps_serve_start(const pps_serve_config* cfg, pps_server** out);
/* queue one problem (validated here; PPS_ENOMEM if it can never fit) */
PPS_API int pps_serve_submit(pps_server* s, const pps_problem* prob, int64_t n, uint64_t seed, int32_t maxiters,
                             float w, float wdamp, float c1, float c2, uint64_t* ticket);
/* PPS_OK and the result (the ticket is then released), or PPS_EBUSY */
PPS_API int pps_serve_poll(pps_server* s, uint64_t ticket, float* u, float* cost, int64_t* idx,
                           double* latency_ms);
/* block until done or timeout_s seconds pass (PPS_ETIMEOUT; a negative timeout
 * does not wait, NaN is PPS_EINVAL); a ticket whose result another call has
 * taken is PPS_EINVAL */
PPS_API int pps_serve_wait(pps_server* s, uint64_t ticket, float* u, float* cost, int64_t* idx,
                           double* latency_ms, double timeout_s);
PPS_API int pps_serve_stats_get(pps_server* s, pps_serve_stats* stats);
/* finish queued and running requests, then release everything */
PPS_API int pps_serve_stop(pps_server* s);

/* ---- results ---- */
/* global best position (dim floats), cost and particle index; any may be NULL */
PPS_API int pps_get_gbest(pps_swarm* s, float* u, float* cost, int64_t* idx);
/* copy a state field to / from host memory (SoA, particle fastest) */
PPS_API int pps_get_state(pps_swarm* s, int32_t field, float* out);
PPS_API int pps_set_state(pps_swarm* s, int32_t field, const float* in);
/* The whole swarm in the reference's particle records, SPSOParticle{position, velocity,
 * cost, best_position, best_cost} (src/ParallelParticleSwarms.jl:34-44): 3 dim + 2 floats
 * per particle.  PPS_LAYOUT_AOS: n records one after another (a Julia caller wraps the
 * buffer as Vector{SPSOParticle}); PPS_LAYOUT_SOA: the five fields one after another, each
 * particle-fastest.  Setting the particles makes the global best the argmin of best_cost,
 * as init does (src/init.jl:49-51). */
enum { PPS_LAYOUT_SOA = 0, PPS_LAYOUT_AOS = 1 };
PPS_API int pps_get_particles(pps_swarm* s, int32_t layout, float* out);
PPS_API int pps_set_particles(pps_swarm* s, int32_t layout, const float* in);
/* A device snapshot of a state field: sol.original = get_pos.(particles), which the
 * reference keeps on the device as a new array (src/solve.jl:51-56).  The swarm may be
 * re-run or destroyed while the snapshot lives; read copies it to host memory in
 * pps_get_state's layout (SoA, particle fastest). */
typedef struct pps_field_copy pps_field_copy;
PPS_API int pps_field_copy_create(pps_swarm* s, int32_t field, pps_field_copy** out);
PPS_API int pps_field_copy_read(pps_field_copy* c, float* out);
PPS_API int pps_field_copy_destroy(pps_field_copy* c);
/* evaluate the problem's objective at npoints points (SoA dim x npoints) on
 * the device; used for sol.objective = f(u, p) (src/solve.jl:54-57) */
PPS_API int pps_eval_objective(const pps_problem* prob, int64_t npoints, const float* x, float* f);

/* ---- user objectives ---- */
/* Registers an objective given as CUDA C source and returns its id (>=
 * PPS_OBJ_USER_BASE) for pps_problem.objective.  Replaces the objective
 * closure that the reference compiles into its kernels (cost =
 * prob.f(x, p), src/kernels.jl:33).  The source defines
 *
 *   PPS_DEVICE float pps_objective(pps_point x, int dim, const float* p,
 *                                  const float* data, long long ndata)
 *
 * with x[d] the point's coordinate d, p the problem's 8 parameters (zero past
 * nparams) and data / ndata the problem's data buffer on the device.  It is
 * compiled by NVRTC (loaded at run time) with --fmad=false for the current
 * device, together with the library's init, synchronous-step and evaluation
 * kernels; pps_exp, pps_cos2pi and pps_sin2pi are the library's exp(x),
 * cos(2 pi x) and sin(2 pi x).  The same source registered again returns the
 * same id.  Errors: PPS_EINVAL with the compiler log (pps_last_error) when
 * the source does not compile, PPS_ENOTSUP without NVRTC.
 * A user objective runs through pps_swarm_create / pps_swarm_init,
 * pps_sync_run, pps_queue_run, pps_async_run, pps_eval_objective and the
 * server (as a swarm of its own), constraints included (not with
 * pps_async_run).  The HybridPSO local stage (pps_hybrid_lbfgs / _bfgs) needs
 * a gradient: a source that defines PPS_HAS_GRADIENT also defines
 *   PPS_DEVICE float pps_gradient(pps_point x, int dim, const float* p,
 *                                 const float* data, long long ndata, float* g)
 * (g = grad f(x), returns f(x)); without it, and for batches and
 * pps_sync_run_noalloc, the call returns PPS_ENOTSUP.
 * A source that defines PPS_HAS_STREAM also gives f as a fold over the
 * coordinates in increasing order (a state type pps_stream and
 * pps_stream_start / pps_stream_add / pps_stream_finish, declared in
 * pps_user_prelude.cuh); the synchronous step then evaluates f in registers
 * as each coordinate moves instead of reading the new position back.  The
 * fold must equal pps_objective bit for bit.
 * The library cannot bound the running time of the user's code: a function
 * that does not return hangs the run. */
PPS_API int pps_objective_register(const char* source, int32_t* objective);

/* ---- particle-range shards of one swarm ---- */
/* The synchronous loop couples particles only through its per-iteration
 * global best: block bests, then their minimum (src/kernels.jl:156-171,
 * src/lowerlevel_solve.jl:23-33).  A shard holds particles first .. first +
 * count - 1 of an n_global-particle swarm and moves them exactly as the whole
 * swarm does (random streams, argmin keys and the penalty's particle index
 * use the global index), so the swarm splits over processes or GPUs with one
 * exchange per iteration:
 *   pps_shard_step (or pps_swarm_init)  writes the shard's exchange record:
 *        its best particle's argmin key (uint64 at byte 0: orderable cost << 32
 *        | global index), cost (float at byte 8) and vector (dim floats from
 *        byte 16), pps_shard_record's `bytes` in all;
 *   the caller gathers every shard's record into one array (an all-gather of
 *        fixed-size records, e.g. ncclAllGather, or device copies);
 *   pps_shard_apply makes the lowest key of that array the global best.
 * Objectives: the registered closed-form ones (constraints included).  A
 * shard is stepped only through the calls below: pps_sync_run, pps_async_run,
 * pps_queue_run, the local stage and pps_set_particles return PPS_ENOTSUP on
 * it.  Nothing below waits for the device except pps_shard_finish; all work of
 * a shard is ordered on its stream (pps_shard_record returns it). */
PPS_API int pps_shard_create(const pps_problem* prob, int64_t n_global, int64_t first, int64_t count,
                             uint64_t seed, uint32_t flags, pps_swarm** out);
/* the shard's own exchange record (device address), its size in bytes and the
 * shard's cudaStream_t; any may be NULL */
PPS_API int pps_shard_record(pps_swarm* s, void** record, int64_t* bytes, void** stream);
/* Exchange buffers of the caller's (device memory, 16-byte aligned): the shard
 * writes its record to `record` and pps_shard_apply reads `nrecords` records
 * from `records` (record r at r * bytes).  Until bound, both are the shard's
 * own record with nrecords = 1 (a swarm of one shard). */
PPS_API int pps_shard_bind(pps_swarm* s, void* record, const void* records, int32_t nrecords);
/* One synchronous iteration of the shard's particles (vectorized_solve! of
 * ParallelSyncPSOKernel, one trip of src/lowerlevel_solve.jl:1-36); begin != 0
 * starts a run: inertia w, damped by wdamp after each iteration. */
PPS_API int pps_shard_step(pps_swarm* s, int32_t begin, float w, float wdamp, float c1, float c2);
/* ParallelPSOKernel(global_update=false) on the shard (src/kernels.jl:196-225):
 * maxiters iterations in one launch, the record written after the last */
PPS_API int pps_shard_async(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2);
/* the global best := the bound record with the lowest key */
PPS_API int pps_shard_apply(pps_swarm* s);
/* the deferred personal-best copies (so pps_get_state reads canonical state);
 * waits for the shard's stream */
PPS_API int pps_shard_finish(pps_swarm* s);

/* ---- caller-owned device buffers, no allocation ---- */
/* A swarm whose device arrays belong to the caller.  All pointers are DEVICE
 * pointers, 16-byte aligned.  Element (particle i, dim d) is at [d*ld + i];
 * ld is a multiple of 32 with n <= ld; columns n..ld-1 are padding that the
 * kernels overwrite.  pcost and cost hold ld floats, lb, ub and g dim floats. */
typedef struct pps_device_swarm {
  int64_t n;
  int64_t ld;
  int32_t dim;
  float* x;         /* positions, in/out */
  float* v;         /* velocities, in/out */
  float* pbest;     /* personal bests, in/out */
  float* pcost;     /* personal best costs, in/out */
  float* cost;      /* current costs, out */
  const float* lb;  /* lower bounds (may hold -inf) */
  const float* ub;  /* upper bounds (may hold +inf) */
  float* g;         /* global best position, out */
} pps_device_swarm;

/* The synchronous run of pps_sync_run on buffers the caller owns, with no
 * allocation: no cudaMalloc, cudaFree, stream or event creation.  It has no
 * counterpart in the reference (whose Julia host allocates through
 * KernelAbstractions).  It is for callers that cannot let a library
 * allocate: memory held by a pooled allocator such as CUDA.jl's, where a
 * hidden cudaMalloc can fail while the pool holds the memory and
 * synchronises the device, or a host framework that hands every buffer to
 * its plugins from its own arena.
 *   objective, params, nparams  the registered objective (pps_objective)
 *   seed, iteration             Philox key and the iteration counter of the
 *                               first step (0 after an init; add maxiters per call)
 *   flags                       PPS_FLAG_GBEST_FROM_POSITION or 0
 *   stream                      cudaStream_t to launch on (NULL: the legacy default stream)
 *   gcost_out, gidx_out         host pointers, may be NULL; when given, the call
 *                               waits for the stream and returns the global best,
 *                               or PPS_ETIMEOUT if a bounded wait of the step
 *                               kernel gave up (without them that is not checked)
 * The run starts from the argmin of pcost (its pbest, or its position with
 * PPS_FLAG_GBEST_FROM_POSITION) and leaves the global best in g.
 * Scratch: the per-iteration argmin state and one byte per particle live in a
 * static device array of 1 MiB + 256 B in the library, so n and ld are limited
 * to 1,048,576 particles (larger requests fail with PPS_EINVAL before any
 * device work).  Every GPU that loads the library holds that array until the
 * process exits.  The first call on a device looks up the array's address
 * with that device current; make it before any stream capture begins.  Each
 * call clears the part it uses, but all calls share the array: calls that
 * overlap on the GPU (other streams, unordered host threads) race. */
PPS_API int pps_sync_run_noalloc(int32_t objective, const float* params, int32_t nparams,
                                 const pps_device_swarm* swarm, uint64_t seed, uint32_t iteration,
                                 int32_t maxiters, float w, float wdamp, float c1, float c2,
                                 uint32_t flags, void* stream, float* gcost_out, int64_t* gidx_out);

#ifdef __cplusplus
}
#endif
#endif /* PPS_H */
