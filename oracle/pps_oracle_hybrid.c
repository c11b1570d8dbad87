/*
 * pps_oracle_hybrid.c -- CPU restatement of HybridPSO's local stage (test
 * infrastructure; see pps_oracle.h).
 *
 * Reference: src/hybrid.jl:100-158 launches lbfgs_run! (src/lbfgs.jl:9-21),
 * one SimpleOptimization._lbfgs per particle started from its personal best,
 * then a host findmin keeps the result if it beats the swarm best.
 * SimpleOptimization (compat "2", Project.toml) is not vendored; this is the
 * published algorithm it names: projected L-BFGS with the two-loop recursion
 * (Nocedal & Wright, Numerical Optimization, 2nd ed., Alg. 7.4) and, as the
 * workload asks, a backtracking Armijo line search (c1 = 1e-4) along the
 * projected path.  Dot products are sequential binary32 sums with no fusion;
 * the CUDA kernel performs the same operations in the same order.
 *
 * The BFGS variant (src/hybrid.jl:33-98) solves grad f = 0 with
 * SimpleNonlinearSolve.SimpleBroyden starting from each particle's current
 * position, the gradient replaced by 1e15 outside the box grown by twice its
 * width (BoundedGrad, src/hybrid.jl:15-31).  Restated here as Broyden's
 * "good" method on the inverse Jacobian (Sherman-Morrison update) with a
 * halving backtrack on ||F||^2.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "pps_oracle.h"

#define MAXD 64
#define MAXM 32

static inline float dotf(const float* a, const float* b, int D) {
  float s = 0.0f;
  for (int d = 0; d < D; ++d) s = s + a[d] * b[d];
  return s;
}
static inline float clampf_(float x, float lo, float hi) {
  x = (x < lo) ? lo : x;
  x = (x > hi) ? hi : x;
  return x;
}

/* one projected L-BFGS run; returns iterations used */
static int lbfgs_one(const orc_problem* prob, const float* x0, const orc_lbfgs_opts* o, float* xo,
                     float* fo) {
  const int D = prob->dim;
  const int m = o->history;
  const float* lb = prob->lb;
  const float* ub = prob->ub;
  float x[MAXD], g[MAXD], pg[MAXD], q[MAXD], dir[MAXD], xn[MAXD], gn[MAXD];
  float S[MAXM][MAXD], Y[MAXM][MAXD], rho[MAXM], alpha[MAXM];
  int hist = 0, head = 0;
  for (int d = 0; d < D; ++d) x[d] = clampf_(x0[d], lb[d], ub[d]);
  float f = orc_objective_grad(prob, x, g);
  int it = 0;
  for (; it < o->maxiters; ++it) {
    if (!isfinite(f)) break;
    /* projected gradient: zero components held at an active bound */
    for (int d = 0; d < D; ++d) {
      int hold = (x[d] <= lb[d] && g[d] > 0.0f) || (x[d] >= ub[d] && g[d] < 0.0f);
      pg[d] = hold ? 0.0f : g[d];
    }
    float gn2 = dotf(pg, pg, D);
    if (sqrtf(gn2) <= o->gtol) break;
    /* two-loop recursion, newest pair first */
    for (int d = 0; d < D; ++d) q[d] = pg[d];
    for (int j = 0; j < hist; ++j) {
      int slot = (head - 1 - j + m) % m;
      float a = rho[slot] * dotf(S[slot], q, D);
      alpha[slot] = a;
      for (int d = 0; d < D; ++d) q[d] = q[d] - a * Y[slot][d];
    }
    float gamma = 1.0f;
    if (hist > 0) {
      int nw = (head - 1 + m) % m;
      gamma = dotf(S[nw], Y[nw], D) / dotf(Y[nw], Y[nw], D);
    }
    for (int d = 0; d < D; ++d) q[d] = gamma * q[d];
    for (int j = hist - 1; j >= 0; --j) {
      int slot = (head - 1 - j + m) % m;
      float b = rho[slot] * dotf(Y[slot], q, D);
      for (int d = 0; d < D; ++d) q[d] = q[d] + S[slot][d] * (alpha[slot] - b);
    }
    for (int d = 0; d < D; ++d) {
      float dd = -q[d];
      int hold = (x[d] <= lb[d] && dd < 0.0f) || (x[d] >= ub[d] && dd > 0.0f);
      dir[d] = hold ? 0.0f : dd;
    }
    float gd = dotf(g, dir, D);
    if (!(gd < 0.0f)) {
      /* not a descent direction: restart from steepest descent */
      hist = 0;
      head = 0;
      for (int d = 0; d < D; ++d) dir[d] = -pg[d];
      gd = dotf(g, dir, D);
      if (!(gd < 0.0f)) break;
    }
    float step = 1.0f;
    int ok = 0;
    float fn = f;
    for (int bt = 0; bt < o->max_backtracks; ++bt) {
      for (int d = 0; d < D; ++d) xn[d] = clampf_(x[d] + step * dir[d], lb[d], ub[d]);
      fn = orc_objective(prob, xn, 1, 1);
      float dec = 0.0f;
      for (int d = 0; d < D; ++d) dec = dec + g[d] * (xn[d] - x[d]);
      if (fn <= f + o->armijo_c1 * dec) { ok = 1; break; }
      step = step * 0.5f;
    }
    if (!ok) break;
    fn = orc_objective_grad(prob, xn, gn);
    float sy = 0.0f;
    float sv[MAXD], yv[MAXD];
    for (int d = 0; d < D; ++d) {
      sv[d] = xn[d] - x[d];
      yv[d] = gn[d] - g[d];
      sy = sy + sv[d] * yv[d];
    }
    if (sy > 1e-12f) {
      for (int d = 0; d < D; ++d) { S[head][d] = sv[d]; Y[head][d] = yv[d]; }
      rho[head] = 1.0f / sy;
      head = (head + 1) % m;
      if (hist < m) ++hist;
    }
    for (int d = 0; d < D; ++d) { x[d] = xn[d]; g[d] = gn[d]; }
    f = fn;
  }
  for (int d = 0; d < D; ++d) xo[d] = x[d];
  *fo = isfinite(f) ? f : INFINITY;
  return it;
}

/* BoundedGrad (src/hybrid.jl:23-31) */
static void bounded_grad(const orc_problem* prob, const float* x, float* F) {
  const int D = prob->dim;
  int in_box = 1;
  for (int d = 0; d < D; ++d) {
    float w = prob->ub[d] - prob->lb[d];
    if (!isfinite(x[d]) || x[d] < prob->lb[d] - 2.0f * w || x[d] > prob->ub[d] + 2.0f * w) in_box = 0;
  }
  if (in_box) {
    orc_objective_grad(prob, x, F);
  } else {
    for (int d = 0; d < D; ++d) F[d] = 1.0e15f;
  }
}

static int broyden_one(const orc_problem* prob, const float* x0, const orc_lbfgs_opts* o,
                       float* xo, float* fo) {
  const int D = prob->dim;
  float x[MAXD], F[MAXD], xn[MAXD], Fn[MAXD], dx[MAXD], dF[MAXD], JdF[MAXD], dxJ[MAXD];
  float J[MAXD * MAXD];
  for (int d = 0; d < D; ++d) x[d] = x0[d];
  for (int a = 0; a < D; ++a)
    for (int b = 0; b < D; ++b) J[a * D + b] = (a == b) ? 1.0f : 0.0f;
  bounded_grad(prob, x, F);
  float phi = dotf(F, F, D);
  int it = 0;
  for (; it < o->maxiters; ++it) {
    if (!(sqrtf(phi) > o->gtol)) break;
    float step[MAXD];
    for (int a = 0; a < D; ++a) step[a] = -dotf(&J[a * D], F, D);
    float s = 1.0f;
    float phin = phi;
    int ok = 0;
    for (int bt = 0; bt < o->max_backtracks; ++bt) {
      for (int d = 0; d < D; ++d) xn[d] = x[d] + s * step[d];
      bounded_grad(prob, xn, Fn);
      phin = dotf(Fn, Fn, D);
      if (phin < phi) { ok = 1; break; }
      s = s * 0.5f;
    }
    if (!ok) break;
    for (int d = 0; d < D; ++d) { dx[d] = xn[d] - x[d]; dF[d] = Fn[d] - F[d]; }
    for (int a = 0; a < D; ++a) JdF[a] = dotf(&J[a * D], dF, D);
    /* dxJ = dx^T J */
    for (int b = 0; b < D; ++b) {
      float acc = 0.0f;
      for (int a = 0; a < D; ++a) acc = acc + dx[a] * J[a * D + b];
      dxJ[b] = acc;
    }
    float den = dotf(dx, JdF, D);
    if (den != 0.0f && isfinite(den)) {
      for (int a = 0; a < D; ++a) {
        float c = (dx[a] - JdF[a]) / den;
        for (int b = 0; b < D; ++b) J[a * D + b] = J[a * D + b] + c * dxJ[b];
      }
    }
    for (int d = 0; d < D; ++d) { x[d] = xn[d]; F[d] = Fn[d]; }
    phi = phin;
  }
  for (int d = 0; d < D; ++d) xo[d] = x[d];
  float v = orc_objective(prob, x, 1, 1);
  *fo = isfinite(v) ? v : INFINITY;
  return it;
}

typedef struct {
  const orc_problem* prob;
  int64_t n;
  const float* x0;
  const orc_lbfgs_opts* o;
  float* xout;
  float* fout;
  int32_t* iters;
  int kind;
} hyb_arg;

static void* hyb_worker(void* p) {
  void** pv = (void**)p;
  hyb_arg* a = (hyb_arg*)pv[0];
  int tid = (int)(intptr_t)pv[1], nth = (int)(intptr_t)pv[2];
  const int D = a->prob->dim;
  int64_t b = (a->n * tid) / nth, e = (a->n * (tid + 1)) / nth;
  float x0[MAXD], xo[MAXD];
  for (int64_t i = b; i < e; ++i) {
    for (int d = 0; d < D; ++d) x0[d] = a->x0[d * a->n + i];
    float f;
    int it = a->kind ? broyden_one(a->prob, x0, a->o, xo, &f) : lbfgs_one(a->prob, x0, a->o, xo, &f);
    for (int d = 0; d < D; ++d) a->xout[d * a->n + i] = xo[d];
    a->fout[i] = f;
    if (a->iters) a->iters[i] = it;
  }
  return NULL;
}

static void hyb_run(hyb_arg* a, int nth) {
  if (nth < 1) nth = 1;
  if (nth > 256) nth = 256;
  pthread_t th[256];
  void* args[256][3];
  for (int t = 0; t < nth; ++t) {
    args[t][0] = a;
    args[t][1] = (void*)(intptr_t)t;
    args[t][2] = (void*)(intptr_t)nth;
    if (t) pthread_create(&th[t], NULL, hyb_worker, args[t]);
  }
  hyb_worker(args[0]);
  for (int t = 1; t < nth; ++t) pthread_join(th[t], NULL);
}

void orc_lbfgs(const orc_problem* prob, int64_t n, const float* x0, const orc_lbfgs_opts* o,
               float* xout, float* fout, int32_t* iters_out, int32_t nthreads) {
  if (prob->dim > MAXD || o->history > MAXM || o->history < 1) return;
  hyb_arg a = {prob, n, x0, o, xout, fout, iters_out, 0};
  hyb_run(&a, nthreads);
}

void orc_broyden(const orc_problem* prob, int64_t n, const float* x0, const orc_lbfgs_opts* o,
                 float* xout, float* fout, int32_t* iters_out, int32_t nthreads) {
  if (prob->dim > MAXD) return;
  hyb_arg a = {prob, n, x0, o, xout, fout, iters_out, 1};
  hyb_run(&a, nthreads);
}
