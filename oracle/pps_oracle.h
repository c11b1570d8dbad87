/*
 * pps_oracle.h -- CPU restatement of ParallelParticleSwarms.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it may be loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline /
 * reference leg, never by the product path (libpps_cuda.so and the Python
 * package do not link, import or execute anything here).
 *
 * What it restates (file:line of the reference project):
 *   - particle update        src/kernels.jl:1-26   (update_particle_state)
 *   - sync CPU-backend loop  src/lowerlevel_solve.jl:38-65, src/kernels.jl:182-194
 *   - sync GPU loop (gbest from the winner's personal best)
 *                            src/lowerlevel_solve.jl:1-36, src/kernels.jl:127-177
 *   - async in-kernel loop   src/kernels.jl:196-225, src/lowerlevel_solve.jl:95-121
 *   - uniform / unbounded init  src/utils.jl:23-84, src/init.jl:38-54
 *   - argmin ordering        src/ParallelParticleSwarms.jl:59-71 (isless on cost)
 *   - defaults w=0.7298, wdamp=1, c1=c2=1.4962
 *                            src/lowerlevel_solve.jl:6-7, src/kernels.jl:130-131
 *   - Rosenbrock objective   test/regression.jl:12-18, test/gpu.jl:14-20
 *   - HybridPSO local stage  src/hybrid.jl:100-158, src/lbfgs.jl:9-21
 *   - ode_pso loop and SSE   src/ode_pso.jl:1-52,113-170
 *
 * Random numbers: the reference draws r1, r2 with rand() (src/kernels.jl:3,8);
 * this restatement and the CUDA kernels draw them from the same counter-based
 * Philox4x32-10 stream (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers:
 * As Easy as 1, 2, 3", SC'11), so the two can be compared iteration by
 * iteration.  Counter layout:
 *   update draws: ctr = {particle, dim/2, iteration, PPS_TAG_STEP}, key = seed
 *                 out = {r1[2j], r2[2j], r1[2j+1], r2[2j+1]}
 *   init draws:   ctr = {particle, dim/4, 0, PPS_TAG_INIT}, out[k] -> dim 4j+k
 *   u01(o) = (o >> 8) * 2^-24
 *
 * Arithmetic: every operation is a single IEEE-754 binary32 operation in the
 * reference's evaluation order; fused multiply-add appears only where written
 * as fmaf() (the CUDA kernels use __fmaf_rn at the same places), so results are
 * bit-identical to the kernels.  Build with -ffp-contract=off.
 *
 * Parity pins: the reference's own tests are thresholds under fixed seeds
 * (test/regression.jl, test/gpu.jl), an exact loss-reduction check
 * (test/regression.jl:345-389) and L-BFGS known answers (test/lbfgs.jl:3-73);
 * tests/test_oracle_pins.py re-runs each of them against this library.
 */
#ifndef PPS_ORACLE_H
#define PPS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_TAG_INIT 0x494E4954u  /* "INIT" */
#define ORC_TAG_STEP 0x50534F31u  /* "PSO1" */

enum {
  ORC_OBJ_SPHERE = 0,
  ORC_OBJ_ROSENBROCK = 1,
  ORC_OBJ_RASTRIGIN = 2,
  ORC_OBJ_ACKLEY = 3,
  ORC_OBJ_LV_FIT = 4,   /* SSE of an RK4 Lotka-Volterra solve vs data */
  ORC_OBJ_FHN_FIT = 5,  /* SSE of an RK4 FitzHugh-Nagumo solve vs data */
  ORC_OBJ_MLP = 6,      /* MLP regression loss (16 -> 32 tanh -> 1, MSE) */
  ORC_OBJ_SHIFTED_SPHERE = 7, /* sum (x_i - p_i)^2, p_i = 0 past nparams (test/constraints.jl:7) */
  /* closed-form objectives of the reference's L-BFGS tests (test/lbfgs.jl:20-26) */
  ORC_OBJ_BEALE = 16,
  ORC_OBJ_BOOTH = 17,
  ORC_OBJ_HIMMELBLAU = 18,
  ORC_OBJ_QUADRATIC = 19,          /* p1 (x1-1)^2 + (x2+2)^2 */
  ORC_OBJ_BOUNDARY_QUADRATIC = 20, /* (x1+1)^2 */
  /* a user objective (include/pps.h pps_objective_register): user_fn, the
   * same source compiled as C (pps_point = const float*, PPS_DEVICE empty) */
  ORC_OBJ_USER = 256,
};

/* f(x, dim, p, data, ndata) of a user objective, x contiguous */
typedef float (*orc_user_fn)(const float* x, int dim, const float* p, const float* data, long long ndata);
/* its gradient (a source that defines PPS_HAS_GRADIENT): g = grad f(x), returns f(x) */
typedef float (*orc_user_grad_fn)(const float* x, int dim, const float* p, const float* data, long long ndata,
                                  float* g);

struct orc_ode_fit;

/* problem description, mirrors pps_problem in include/pps.h */
typedef struct orc_problem {
  int32_t objective;
  int32_t dim;
  const float* lb;      /* dim floats, may hold +-inf */
  const float* ub;      /* dim floats */
  const float* u0;      /* dim floats (unbounded sampler only) */
  float params[8];      /* objective parameters */
  int32_t nparams;
  const struct orc_ode_fit* ode;  /* ORC_OBJ_LV_FIT / ORC_OBJ_FHN_FIT only */
  const float* mlp_data;          /* ORC_OBJ_MLP: S x 16 samples then S targets */
  int32_t mlp_samples;
  /* constraints g_k(x) <= 0, k < ncons <= 4, each c_k + sum_i a_ki x_i + b_ki x_i^2:
   * cons = ncons rows of (c_k, a_k[dim], b_k[dim]) */
  int32_t ncons;
  const float* cons;
  /* ORC_OBJ_USER: the function and its data buffer */
  orc_user_fn user_fn;
  const float* user_data;
  int64_t user_ndata;
  orc_user_grad_fn user_grad;  /* NULL: no gradient */
} orc_problem;

/* structure-of-arrays swarm state: x[d*n + i] */
typedef struct orc_swarm {
  int64_t n;
  int32_t dim;
  float* x;
  float* v;
  float* pbest;
  float* pcost;
  float* cost;
  float* g;       /* dim floats: global best position */
  float gcost;
  int64_t gidx;
  /* Particle-range shard of a larger swarm: local particle i is particle
   * first + i of nglobal (0: nglobal = n, a whole swarm).  Random streams,
   * argmin keys, the penalty's particle index and the Latin-hypercube strata
   * use the global index; g / gcost / gidx then hold the shard's own best
   * (gidx global) until the caller replaces them by the exchanged winner. */
  int64_t first;
  int64_t nglobal;
} orc_swarm;

/* ---- primitives ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]);
float orc_u01(uint32_t bits);
float orc_cos2pi(float x);
float orc_sin2pi(float x);
float orc_exp(float x);
uint64_t orc_argmin_key(float cost, uint32_t idx);

/* objective value with the dims split into `lanes` contiguous slices of
 * even length, each summed in order, the slice sums combined by a balanced
 * pairwise tree (lanes a power of two, 1 = plain sequential sum). */
float orc_objective(const orc_problem* prob, const float* x, int64_t stride, int32_t lanes);
/* calc_penalty (src/utils.jl:320-372) for the registered constraint form at x
 * (stride `stride`), with h = sqrt and the weight's argument `iter`: 1 at init
 * (src/utils.jl:72-74), particle index + 1 (1-based) in the sync and
 * queue-lock steps (src/kernels.jl:77,151 pass the index as `iter`,
 * handle_constraints adds 1, :28-31).  0 without constraints. */
float orc_penalty(const orc_problem* prob, const float* x, int64_t stride, float iter);
/* analytic gradient (Rosenbrock, Rastrigin, Ackley, sphere), sequential sums */
float orc_objective_grad(const orc_problem* prob, const float* x, float* grad);

/* ---- swarm ---- */
/* samplers: uniform_itr (src/utils.jl:1-5,57-84), the unbounded sampler
 * (src/utils.jl:23-55), Latin hypercube (init(...; sampler =
 * LatinHypercubeSample()), src/init.jl:15-34; QuasiMonteCarlo is not
 * vendored, so this restates the published method: per dim a random
 * permutation of the n strata, a uniform draw inside each stratum) */
enum { ORC_SAMPLER_UNIFORM = 0, ORC_SAMPLER_UNBOUNDED = 1, ORC_SAMPLER_LHS = 2 };
/* the Latin-hypercube stratum of particle i (< n) in dim d: a keyed bijection
 * of [0, n) (4-round Feistel network on 2h bits, cycle-walked into [0, n)) */
uint32_t orc_lhs_stratum(uint32_t i, uint32_t n, uint32_t d, uint64_t seed);
enum { ORC_GBEST_FROM_PBEST = 0, ORC_GBEST_FROM_POSITION = 1 };

void orc_init(const orc_problem* prob, orc_swarm* s, uint64_t seed, int32_t sampler);
/* the uniform draws of init (u) and of step t (r1, r2) as [d*n + i] arrays for
 * particles first .. first + n - 1: the random numbers orc_init / orc_sync_run
 * consume, for an independent restatement to consume too */
void orc_init_draws(uint64_t seed, int64_t first, int64_t n, int32_t dim, float* u);
void orc_step_draws(uint64_t seed, int64_t first, int64_t n, int32_t dim, uint32_t t, float* r1, float* r2);
/* argmin of pcost (lowest index on ties), gather g from pbest or position */
void orc_select_gbest(const orc_problem* prob, orc_swarm* s, int32_t gbest_source);
/* `iters` synchronous iterations starting at iteration counter t0.
 * Returns the inertia weight after the last damping step. */
float orc_sync_run(const orc_problem* prob, orc_swarm* s, uint64_t seed, uint32_t t0,
                   int32_t iters, float w, float wdamp, float c1, float c2,
                   int32_t gbest_source, int32_t nthreads);
/* async: every particle runs `iters` iterations against a private global best
 * seeded from s->g; the objective is summed with `lanes` slices. */
float orc_async_run(const orc_problem* prob, orc_swarm* s, uint64_t seed, uint32_t t0,
                    int32_t iters, float w, float wdamp, float c1, float c2,
                    int32_t lanes, int32_t nthreads);
/* how the CUDA async kernel splits D dims over lanes: returns lanes, writes
 * the even slice length */
int32_t orc_async_lanes(int32_t dim, int32_t* slice);

/* ---- HybridPSO local stage ---- */
typedef struct orc_lbfgs_opts {
  int32_t history;     /* m */
  int32_t maxiters;
  float armijo_c1;
  float gtol;
  int32_t max_backtracks;
} orc_lbfgs_opts;
/* projected L-BFGS from each start point (x0[d*n+i]); writes xout, fout */
void orc_lbfgs(const orc_problem* prob, int64_t n, const float* x0, const orc_lbfgs_opts* o,
               float* xout, float* fout, int32_t* iters_out, int32_t nthreads);
/* Broyden quasi-Newton on grad f = 0 (inverse-Jacobian update) */
void orc_broyden(const orc_problem* prob, int64_t n, const float* x0, const orc_lbfgs_opts* o,
                 float* xout, float* fout, int32_t* iters_out, int32_t nthreads);

/* ---- ode_pso ---- */
enum { ORC_ODE_LV = 0, ORC_ODE_FHN = 1 };
typedef struct orc_ode_fit {
  int32_t model;       /* ORC_ODE_LV / ORC_ODE_FHN */
  int32_t nparams;     /* particle dimension */
  float u0[2];
  float dt;
  int32_t nsteps;      /* RK4 steps */
  int32_t save_every;  /* save a point every save_every steps (t=0 included) */
  int32_t nsaves;
  const float* data;   /* nsaves x 2, row major */
  float fixed[4];      /* fixed model constants (FHN: l) */
  int32_t method;      /* ORC_ODE_RK4 (saves every save_every steps), ORC_ODE_TSIT5 or ORC_ODE_TSIT5_ADAPTIVE */
  float save_dt;       /* Tsit5: saves at m * save_dt from the continuous extension */
  float rtol, atol;    /* adaptive Tsit5: tolerances of the step-size control; dt is the first step */
} orc_ode_fit;
enum { ORC_ODE_RK4 = 0, ORC_ODE_TSIT5 = 1, ORC_ODE_TSIT5_ADAPTIVE = 2 };
/* adaptive Tsit5 (parameter_estim_ode!(..., Val(true)), src/ode_pso.jl:54-111):
 * the SSE, and the steps taken (accepted + rejected; 100000 at most, after
 * which, or when a step no longer advances t, the loss is +inf) */
float orc_ode_loss_adaptive(const orc_ode_fit* f, const float* p, int32_t* steps);
/* ln x of the step-size controller (the CUDA kernels' log_f, same bits) */
float orc_log(float x);
/* RK4 or Tsit5 integration + SSE against data (src/ode_pso.jl:47-52) */
float orc_ode_loss(const orc_ode_fit* fit, const float* p);
/* trajectory at the save points: out[nsaves*2] */
void orc_ode_solve(const orc_ode_fit* fit, const float* p, float* out);
/* sum of squared differences per particle: data[m][k] vs us[i][m][k]
 * (the reference's _reduce_losses!, test/regression.jl:345-357) */
void orc_reduce_losses(int32_t m, int32_t ncomp, int64_t n, const float* data,
                       const float* us, float* losses);
/* An ODE fit is a swarm whose objective is ORC_OBJ_LV_FIT / ORC_OBJ_FHN_FIT
 * (orc_problem.ode points at the fit): orc_init + orc_sync_run give the
 * parameter_estim_ode! loop of src/ode_pso.jl:113-170 with an elementwise
 * clamp and RK4 in place of GPUTsit5. */

/* ---- MLP regression objective (tensor-core path) ----
 * particle x (577 floats): W1[i][j] at i*32 + j (16 inputs x 32 hidden),
 * b1 at 512.., w2 at 544.., b2 at 576.  Loss = mean_s (w2 . tanh(W1^T X_s + b1)
 * + b2 - y_s)^2 with X_s and W1 rounded to bfloat16 (the GEMM operands) and
 * everything else in double: the reference value the kernel's BF16 GEMM with
 * FP32 accumulation and approximate tanh is compared against within a
 * tolerance. */
double orc_mlp_loss(const float* x, const float* X, const float* y, int32_t samples);
float orc_bf16_round(float v);

#ifdef __cplusplus
}
#endif
#endif
