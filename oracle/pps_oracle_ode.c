/*
 * pps_oracle_ode.c -- CPU restatement of the ode_pso objective (test
 * infrastructure; see pps_oracle.h).
 *
 * The reference integrates each particle's ODE with DiffEqGPU's GPUTsit5
 * (src/ode_pso.jl:87,146, third-party, not vendored) and reduces the loss with
 * _reduce_losses! (src/ode_pso.jl:47-52): SSE over save points and states.
 * This build integrates with the classical fixed-step RK4 instead (the
 * workload asks for RK4 with dt = 0.01); the stage arithmetic below is the
 * one the CUDA kernel performs, with fused multiply-adds written as fmaf().
 *
 * Right-hand sides:
 *   Lotka-Volterra  benchmarks/Lotka_Volterra/lotka_volterra.jl:9-13
 *     du1 = p1*u1 - p2*u1*u2,  du2 = -p3*u2 + p4*u1*u2
 *   FitzHugh-Nagumo benchmarks/Fitzhugh_Nagumo/ode_estimation.jl:6-12
 *     dv = v - v^3/3 - w + l,  dw = tinv*(v + a - b*w)   (l held fixed)
 * evaluated in factored form, two roundings per term where the literal
 * form takes four (the RK4 arithmetic is this build's own: the reference
 * integrates with GPUTsit5):
 *     du1 = u1 * fma(-p2, u2, p1)          du2 = u2 * fma(p4, u1, -p3)
 *     dv  = (fma(v*v*v, -1/3, v) - w) + l  dw  = tinv * fma(-b, w, v + a)
 */
#include <math.h>
#include <string.h>

#include "pps_oracle.h"

static inline void rhs(const orc_ode_fit* f, const float* p, float u0, float u1, float* d0,
                       float* d1) {
  if (f->model == ORC_ODE_LV) {
    *d0 = u0 * fmaf(-p[1], u1, p[0]);
    *d1 = u1 * fmaf(p[3], u0, -p[2]);
  } else {
    float v3 = (u0 * u0) * u0;
    *d0 = (fmaf(v3, -0x1.555556p-2f, u0) - u1) + f->fixed[0];
    *d1 = p[2] * fmaf(-p[1], u1, u0 + p[0]);
  }
}

static inline void rk4_step(const orc_ode_fit* f, const float* p, float* u0, float* u1) {
  const float dt = f->dt;
  const float h2 = dt * 0.5f;
  const float h6 = dt / 6.0f;
  float k1a, k1b, k2a, k2b, k3a, k3b, k4a, k4b;
  rhs(f, p, *u0, *u1, &k1a, &k1b);
  rhs(f, p, fmaf(h2, k1a, *u0), fmaf(h2, k1b, *u1), &k2a, &k2b);
  rhs(f, p, fmaf(h2, k2a, *u0), fmaf(h2, k2b, *u1), &k3a, &k3b);
  rhs(f, p, fmaf(dt, k3a, *u0), fmaf(dt, k3b, *u1), &k4a, &k4b);
  float sa = fmaf(2.0f, k2a, k1a);
  sa = fmaf(2.0f, k3a, sa);
  sa = sa + k4a;
  float sb = fmaf(2.0f, k2b, k1b);
  sb = fmaf(2.0f, k3b, sb);
  sb = sb + k4b;
  *u0 = fmaf(h6, sa, *u0);
  *u1 = fmaf(h6, sb, *u1);
}

void orc_ode_solve(const orc_ode_fit* f, const float* p, float* out) {
  float u0 = f->u0[0], u1 = f->u0[1];
  out[0] = u0;
  out[1] = u1;
  int m = 1;
  for (int s = 1; s <= f->nsteps && m < f->nsaves; ++s) {
    rk4_step(f, p, &u0, &u1);
    if (s % f->save_every == 0) {
      out[2 * m] = u0;
      out[2 * m + 1] = u1;
      ++m;
    }
  }
}

float orc_ode_loss(const orc_ode_fit* f, const float* p) {
  float u0 = f->u0[0], u1 = f->u0[1];
  float d0 = f->data[0] - u0, d1 = f->data[1] - u1;
  float acc = (d0 * d0) + (d1 * d1);
  int m = 1;
  for (int s = 1; s <= f->nsteps && m < f->nsaves; ++s) {
    rk4_step(f, p, &u0, &u1);
    if (s % f->save_every == 0) {
      d0 = f->data[2 * m] - u0;
      d1 = f->data[2 * m + 1] - u1;
      acc = acc + ((d0 * d0) + (d1 * d1));
      ++m;
    }
  }
  return acc;
}

/* losses[i] = sum_m sum_k (data[m][k] - us[i][m][k])^2, as
 * sum!(losses, map(x -> sum(x.^2), gpu_data .- us)) */
void orc_reduce_losses(int32_t m, int32_t ncomp, int64_t n, const float* data, const float* us,
                       float* losses) {
  for (int64_t i = 0; i < n; ++i) {
    float acc = 0.0f;
    for (int32_t j = 0; j < m; ++j) {
      float e = 0.0f;
      for (int32_t k = 0; k < ncomp; ++k) {
        float d = data[j * ncomp + k] - us[(i * m + j) * ncomp + k];
        e = e + d * d;
      }
      acc = acc + e;
    }
    losses[i] = acc;
  }
}

/* ---- MLP objective ---- */
float orc_bf16_round(float v) {
  uint32_t b;
  memcpy(&b, &v, 4);
  if ((b & 0x7f800000u) == 0x7f800000u) return v;  /* inf / nan */
  const uint32_t lsb = (b >> 16) & 1u;
  b += 0x7fffu + lsb; /* round to nearest even */
  b &= 0xffff0000u;
  float r;
  memcpy(&r, &b, 4);
  return r;
}

double orc_mlp_loss(const float* x, const float* X, const float* y, int32_t samples) {
  double acc = 0.0;
  for (int s = 0; s < samples; ++s) {
    double o = x[576];
    for (int j = 0; j < 32; ++j) {
      double h = x[512 + j];
      for (int i = 0; i < 16; ++i) h += (double)orc_bf16_round(X[s * 16 + i]) * (double)orc_bf16_round(x[i * 32 + j]);
      o += (double)x[544 + j] * tanh(h);
    }
    const double e = o - (double)y[s];
    acc += e * e;
  }
  return acc / samples;
}
