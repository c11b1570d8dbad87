/*
 * pps_oracle.c -- CPU restatement of ParallelParticleSwarms.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see pps_oracle.h for the contract,
 * the counter layout of the random stream and the reference citations).
 * Compile with -ffp-contract=off: every arithmetic step below is one IEEE
 * binary32 operation, and fmaf() is written out where the CUDA kernels use a
 * fused multiply-add, so the two produce identical bits.
 */
#include "pps_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 and Philox4x64-10 (Salmon et al., SC'11, section 3)         */
/* ------------------------------------------------------------------------ */
#define PH_M0 0xD2511F53u
#define PH_M1 0xCD9E8D57u
#define PH_W0 0x9E3779B9u
#define PH_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PH_M0 * (uint64_t)c0;
    uint64_t p1 = (uint64_t)PH_M1 * (uint64_t)c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += PH_W0;
    k1 += PH_W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* the 64-bit-word member of the family, used only to pin the round
 * structure against an independent implementation (numpy.random.Philox) */
static void mulhilo64(uint64_t a, uint64_t b, uint64_t* hi, uint64_t* lo) {
  unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
  *hi = (uint64_t)(p >> 64);
  *lo = (uint64_t)p;
}
void orc_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]) {
  const uint64_t M0 = 0xD2E7470EE14C6C93ull, M1 = 0xCA5A826395121157ull;
  const uint64_t W0 = 0x9E3779B97F4A7C15ull, W1 = 0xBB67AE8584CAA73Bull;
  uint64_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint64_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t hi0, lo0, hi1, lo1;
    mulhilo64(M0, c0, &hi0, &lo0);
    mulhilo64(M1, c2, &hi1, &lo1);
    uint64_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0;
    k1 += W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

float orc_u01(uint32_t bits) { return (float)(bits >> 8) * 0x1p-24f; }

static inline void philox_step(uint64_t seed, uint32_t i, uint32_t j, uint32_t t, uint32_t tag,
                               uint32_t out[4]) {
  uint32_t ctr[4] = {i, j, t, tag};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

/* ------------------------------------------------------------------------ */
/* cos(2 pi x), sin(2 pi x), exp(x): own implementations from the Taylor      */
/* series of cos/sin/exp (coefficients pi^k/k! and 1/k! rounded to binary32)  */
/* with exact reduction: y = 2x = n + r, |r| <= 1/2, and Cody-Waite reduction */
/* by ln 2 for exp.                                                           */
/* ------------------------------------------------------------------------ */
static const float COS_C1 = -0x1.3bd3ccp+2f;  /* -pi^2/2!  */
static const float COS_C2 = 0x1.03c1f0p+2f;   /*  pi^4/4!  */
static const float COS_C3 = -0x1.55d3c8p+0f;  /* -pi^6/6!  */
static const float COS_C4 = 0x1.e1f506p-3f;   /*  pi^8/8!  */
static const float COS_C5 = -0x1.a6d1f2p-6f;  /* -pi^10/10! */
static const float COS_C6 = 0x1.f9d38ap-10f;  /*  pi^12/12! */
static const float SIN_S0 = 0x1.921fb6p+1f;   /*  pi        */
static const float SIN_S1 = -0x1.4abbcep+2f;  /* -pi^3/3!   */
static const float SIN_S2 = 0x1.466bc6p+1f;   /*  pi^5/5!   */
static const float SIN_S3 = -0x1.32d2ccp-1f;  /* -pi^7/7!   */
static const float SIN_S4 = 0x1.507834p-4f;   /*  pi^9/9!   */
static const float SIN_S5 = -0x1.e30750p-8f;  /* -pi^11/11! */

/* cos(pi a), 0 <= a <= 1/4 */
static inline float cospi_poly(float a) {
  float z = a * a;
  float p = COS_C6;
  p = fmaf(p, z, COS_C5);
  p = fmaf(p, z, COS_C4);
  p = fmaf(p, z, COS_C3);
  p = fmaf(p, z, COS_C2);
  p = fmaf(p, z, COS_C1);
  return fmaf(p, z, 1.0f);
}
/* sin(pi b), 0 <= b <= 1/4 */
static inline float sinpi_poly(float b) {
  float z = b * b;
  float p = SIN_S5;
  p = fmaf(p, z, SIN_S4);
  p = fmaf(p, z, SIN_S3);
  p = fmaf(p, z, SIN_S2);
  p = fmaf(p, z, SIN_S1);
  p = fmaf(p, z, SIN_S0);
  return p * b;
}
static inline int is_odd_integer(float n) { return rintf(n * 0.5f) * 2.0f != n; }

/* cos(2 pi x) = (-1)^n cos(pi a), y = 2x = n + r, n = rint(y), a = |r| <= 1/2,
 * and cos(pi a) = (1/4 - a^2)(4 + z P(z)), z = a^2, P the degree-3 minimax
 * fit of cospi_coefficients.py; 1/4 - a^2 is one fmaf. */
static const float COS_P0 = -0x1.de9e60p+1f, COS_P1 = 0x1.472a8ap+0f, COS_P2 = -0x1.d47d94p-3f,
                   COS_P3 = 0x1.8c391ap-6f;
float orc_cos2pi(float x) {
  const float y = x + x;
  const float n = rintf(y);
  const uint32_t odd = is_odd_integer(n) ? 1u : 0u;
  uint32_t cb;
  const float a = fabsf(y - n);
  const float z = a * a;
  float q = fmaf(COS_P3, z, COS_P2);
  q = fmaf(q, z, COS_P1);
  q = fmaf(q, z, COS_P0);
  const float p = fmaf(-a, a, 0.25f);
  float c = fmaf(p, z * q, 4.0f * p);
  memcpy(&cb, &c, 4);
  cb ^= odd << 31;
  memcpy(&c, &cb, 4);
  return c;
}

float orc_sin2pi(float x) {
  float y = x + x;
  float n = rintf(y);
  float r = y - n;
  float a = fabsf(r);
  float s = (a <= 0.25f) ? sinpi_poly(a) : cospi_poly(0.5f - a);
  if (r < 0.0f) s = -s;
  return is_odd_integer(n) ? -s : s;
}

static const float EXP_LOG2E = 0x1.715476p+0f;
static const float EXP_LN2_HI = 0x1.62e430p-1f;
static const float EXP_LN2_LO = -0x1.05c610p-29f;
static const float EXP_I3 = 0x1.555556p-3f;  /* 1/3! */
static const float EXP_I4 = 0x1.555556p-5f;  /* 1/4! */
static const float EXP_I5 = 0x1.111112p-7f;  /* 1/5! */
static const float EXP_I6 = 0x1.6c16c2p-10f; /* 1/6! */
static const float EXP_I7 = 0x1.a01a02p-13f; /* 1/7! */

static inline float f_from_bits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t bits_from_f(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

float orc_exp(float x) {
  if (x != x) return x;
  if (x > 88.72283f) return INFINITY;
  if (x < -87.33654f) return 0.0f;
  float k = rintf(x * EXP_LOG2E);
  float r = fmaf(-k, EXP_LN2_HI, x);
  r = fmaf(-k, EXP_LN2_LO, r);
  float p = EXP_I7;
  p = fmaf(p, r, EXP_I6);
  p = fmaf(p, r, EXP_I5);
  p = fmaf(p, r, EXP_I4);
  p = fmaf(p, r, EXP_I3);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ki = (int)k;
  if (ki > 127) return (p * f_from_bits(0x7f000000u)) * 2.0f;
  if (ki < -126) return (p * f_from_bits(0x00800000u)) * f_from_bits((uint32_t)(ki + 126 + 127) << 23);
  return p * f_from_bits((uint32_t)(ki + 127) << 23);
}

/* ln x for the adaptive integrator's step-size controller: x = 2^e m, m in
 * (sqrt(1/2), sqrt(2)], ln m = 2 atanh(s) = 2 (s + s^3/3 + ... + s^9/9) with
 * s = (m - 1)/(m + 1), plus e ln 2 (the Cody-Waite split of orc_exp) */
float orc_log(float x) {
  if (!(x > 0.0f)) return (x == 0.0f) ? -INFINITY : NAN;
  if (x == INFINITY) return x;
  int e = 0;
  if (x < 0x1p-126f) {
    x = x * 0x1p+24f;
    e = -24;
  }
  const uint32_t b = bits_from_f(x);
  e += (int)(b >> 23) - 127;
  float m = f_from_bits((b & 0x007fffffu) | 0x3f800000u);
  if (m > 0x1.6a09e6p+0f) {
    m = m * 0.5f;
    e += 1;
  }
  const float sv = (m - 1.0f) / (m + 1.0f);
  const float z = sv * sv;
  float q = 0x1.c71c72p-3f;
  q = fmaf(q, z, 0x1.249250p-2f);
  q = fmaf(q, z, 0x1.99999ap-2f);
  q = fmaf(q, z, 0x1.555556p-1f);
  q = fmaf(q, z, 2.0f);
  const float lm = sv * q;
  const float ef = (float)e;
  return fmaf(ef, EXP_LN2_HI, fmaf(ef, EXP_LN2_LO, lm));
}

/* orderable 32-bit image of a cost: NaN sorts above +inf */
static inline uint32_t ord_cost(float c) {
  if (c != c) return 0xFFFFFFFFu;
  uint32_t b = bits_from_f(c);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
uint64_t orc_argmin_key(float cost, uint32_t idx) {
  return ((uint64_t)ord_cost(cost) << 32) | (uint64_t)idx;
}

/* ------------------------------------------------------------------------ */
/* objectives                                                                */
/* ------------------------------------------------------------------------ */
static inline float prm(const orc_problem* p, int k, float dflt) {
  return (k < p->nparams) ? p->params[k] : dflt;
}

/* per-dim term accumulation for one slice [d0, d1); x indexed x[d*stride].
 * s1 receives the main sum, s2 the second sum (Ackley cosines). */
static void slice_sums(const orc_problem* prob, const float* x, int64_t stride, int d0, int d1,
                       float* s1, float* s2) {
  const int D = prob->dim;
  float a1 = 0.0f, a2 = 0.0f;
  switch (prob->objective) {
    case ORC_OBJ_SPHERE:
      for (int d = d0; d < d1; ++d) { float xi = x[d * stride]; a1 = a1 + xi * xi; }
      break;
    case ORC_OBJ_ROSENBROCK: {
      /* test/regression.jl:12-18: res += p2*(x[i+1]-x[i]^2)^2 + (p1-x[i])^2 */
      float p1 = prm(prob, 0, 1.0f), p2 = prm(prob, 1, 100.0f);
      for (int d = d0; d < d1 && d < D - 1; ++d) {
        float xi = x[d * stride], xn = x[(d + 1) * stride];
        float t = xn - xi * xi;
        float u = p1 - xi;
        a1 = a1 + ((p2 * (t * t)) + (u * u));
      }
      break;
    }
    case ORC_OBJ_RASTRIGIN: {
      float A = prm(prob, 0, 10.0f);
      for (int d = d0; d < d1; ++d) {
        float xi = x[d * stride];
        a1 = a1 + ((xi * xi) - (A * orc_cos2pi(xi)));
      }
      break;
    }
    case ORC_OBJ_SHIFTED_SPHERE:
      for (int d = d0; d < d1; ++d) {
        float t = x[d * stride] - prm(prob, d, 0.0f);
        a1 = a1 + t * t;
      }
      break;
    case ORC_OBJ_ACKLEY: {
      float k = prm(prob, 2, 1.0f);
      for (int d = d0; d < d1; ++d) {
        float xi = x[d * stride];
        a1 = a1 + xi * xi;
        a2 = a2 + orc_cos2pi(k * xi);
      }
      break;
    }
    default:
      /* closed-form objectives: keep x1, x2 */
      if (d0 == 0 && d1 > 0) a1 = x[0];
      if (d0 <= 1 && d1 > 1) a2 = x[stride];
      break;
  }
  *s1 = a1;
  *s2 = a2;
}

static inline float sq(float a) { return a * a; }

/* theta_default / gamma_default (src/utils.jl:320-338).  The reference
 * compares a Float32 with the Float64 literals 0.001 and 0.1; no binary32
 * lies in [0.001, 0.001f) or in (0.1, 0.1f), so q < 0.001 is q < 0.001f and
 * q <= 0.1 is q < 0.1f. */
static inline float theta_default(float q) {
  return q < 0.001f ? 10.0f : (q < 0.1f ? 20.0f : (q <= 1.0f ? 100.0f : 300.0f));
}

float orc_penalty(const orc_problem* prob, const float* x, int64_t stride, float iter) {
  const int D = prob->dim;
  float q[4];
  for (int k = 0; k < prob->ncons; ++k) {
    const float* row = prob->cons + (int64_t)k * (1 + 2 * D);
    float g = row[0];
    for (int d = 0; d < D; ++d) {
      const float xi = x[d * stride];
      g = g + ((row[1 + d] * xi) + (row[1 + D + d] * (xi * xi)));
    }
    q[k] = (g < 0.0f) ? 0.0f : g; /* max.(cons, 0), NaN kept */
  }
  float pen = 0.0f; /* sum(thetaq) */
  for (int k = 0; k < prob->ncons; ++k) pen = pen + theta_default(q[k]);
  for (int k = 0; k < prob->ncons; ++k) {
    const float pw = (q[k] < 1.0f) ? q[k] : q[k] * q[k]; /* q^gamma_default(q) */
    pen = pen + theta_default(q[k]) * pw;
  }
  return sqrtf(iter) * pen; /* h = sqrt */
}

/* closed-form objectives of test/lbfgs.jl:20-26 from (x1, x2) */
static float closed_form(const orc_problem* prob, float x1, float x2) {
  switch (prob->objective) {
    case ORC_OBJ_BEALE: {
      float x22 = sq(x2), x23 = x22 * x2;
      float a = (1.5f - x1) + x1 * x2;
      float b = (2.25f - x1) + x1 * x22;
      float c = (2.625f - x1) + x1 * x23;
      return (sq(a) + sq(b)) + sq(c);
    }
    case ORC_OBJ_BOOTH: {
      float a = (x1 + 2.0f * x2) - 7.0f;
      float b = (2.0f * x1 + x2) - 5.0f;
      return sq(a) + sq(b);
    }
    case ORC_OBJ_HIMMELBLAU: {
      float a = (sq(x1) + x2) - 11.0f;
      float b = (x1 + sq(x2)) - 7.0f;
      return sq(a) + sq(b);
    }
    case ORC_OBJ_QUADRATIC:
      return prm(prob, 0, 1.0f) * sq(x1 - 1.0f) + sq(x2 + 2.0f);
    case ORC_OBJ_BOUNDARY_QUADRATIC:
      return sq(x1 + 1.0f);
    default:
      return 0.0f;
  }
}

static float finalize(const orc_problem* prob, float s1, float s2) {
  const float Df = (float)prob->dim;
  if (prob->objective >= ORC_OBJ_BEALE) return closed_form(prob, s1, s2);
  switch (prob->objective) {
    case ORC_OBJ_RASTRIGIN: {
      float A = prm(prob, 0, 10.0f);
      return (A * Df) + s1;
    }
    case ORC_OBJ_ACKLEY: {
      float a = prm(prob, 0, 20.0f), b = prm(prob, 1, 0.2f);
      float t1 = -a * orc_exp(-b * sqrtf(s1 / Df));
      float t2 = orc_exp(s2 / Df);
      return ((t1 - t2) + a) + 0x1.5bf0a8p+1f;
    }
    default: return s1;
  }
}

/* balanced pairwise tree in natural order: ((v0+v1)+(v2+v3))... */
static float tree_sum(const float* v, int n) {
  if (n == 1) return v[0];
  int h = n / 2;
  return tree_sum(v, h) + tree_sum(v + h, n - h);
}

float orc_objective(const orc_problem* prob, const float* x, int64_t stride, int32_t lanes) {
  const int D = prob->dim;
  if (prob->objective == ORC_OBJ_LV_FIT || prob->objective == ORC_OBJ_FHN_FIT) {
    float p[8];
    for (int d = 0; d < D && d < 8; ++d) p[d] = x[d * stride];
    return orc_ode_loss(prob->ode, p);
  }
  if (prob->objective == ORC_OBJ_USER) {
    /* cost = prob.f(x, p) (src/kernels.jl:33) with f given as C source */
    float buf[4096];
    for (int d = 0; d < D; ++d) buf[d] = x[d * stride];
    return prob->user_fn(buf, D, prob->params, prob->user_data, (long long)prob->user_ndata);
  }
  if (prob->objective == ORC_OBJ_MLP) {
    float p[577];
    for (int d = 0; d < 577; ++d) p[d] = x[d * stride];
    const int S = prob->mlp_samples;
    return (float)orc_mlp_loss(p, prob->mlp_data, prob->mlp_data + (int64_t)S * 16, S);
  }
  if (lanes <= 1) {
    float s1, s2;
    slice_sums(prob, x, stride, 0, D, &s1, &s2);
    return finalize(prob, s1, s2);
  }
  int S = (D + lanes - 1) / lanes;
  S += S & 1;
  float a1[64], a2[64];
  for (int k = 0; k < lanes; ++k) {
    int d0 = k * S, d1 = d0 + S;
    if (d0 > D) d0 = D;
    if (d1 > D) d1 = D;
    slice_sums(prob, x, stride, d0, d1, &a1[k], &a2[k]);
  }
  return finalize(prob, tree_sum(a1, lanes), tree_sum(a2, lanes));
}

float orc_objective_grad(const orc_problem* prob, const float* x, float* g) {
  const int D = prob->dim;
  if (prob->objective == ORC_OBJ_USER && prob->user_grad)
    return prob->user_grad(x, D, prob->params, prob->user_data, (long long)prob->user_ndata, g);
  float f = orc_objective(prob, x, 1, 1);
  switch (prob->objective) {
    case ORC_OBJ_SPHERE:
      for (int d = 0; d < D; ++d) g[d] = 2.0f * x[d];
      break;
    case ORC_OBJ_ROSENBROCK: {
      float p1 = prm(prob, 0, 1.0f), p2 = prm(prob, 1, 100.0f);
      for (int d = 0; d < D; ++d) {
        float gd = 0.0f;
        if (d < D - 1) {
          float t = x[d + 1] - x[d] * x[d];
          gd = ((-4.0f * p2) * x[d]) * t - 2.0f * (p1 - x[d]);
        }
        if (d > 0) {
          float t = x[d] - x[d - 1] * x[d - 1];
          gd = gd + (2.0f * p2) * t;
        }
        g[d] = gd;
      }
      break;
    }
    case ORC_OBJ_RASTRIGIN: {
      float A = prm(prob, 0, 10.0f);
      const float twopiA = A * 0x1.921fb6p+2f;
      for (int d = 0; d < D; ++d) g[d] = 2.0f * x[d] + twopiA * orc_sin2pi(x[d]);
      break;
    }
    case ORC_OBJ_ACKLEY: {
      float a = prm(prob, 0, 20.0f), b = prm(prob, 1, 0.2f), k = prm(prob, 2, 1.0f);
      const float Df = (float)D;
      float s1, s2;
      slice_sums(prob, x, 1, 0, D, &s1, &s2);
      float rms = sqrtf(s1 / Df);
      float e1 = orc_exp(-b * rms);
      float e2 = orc_exp(s2 / Df);
      /* d/dx_i of -a exp(-b rms) = a b exp(-b rms) x_i / (D rms) */
      float c1 = (rms > 0.0f) ? ((a * b) * e1) / (Df * rms) : 0.0f;
      /* d/dx_i of -exp(s2/D) = exp(s2/D) 2 pi k sin(2 pi k x_i) / D */
      float c2 = (e2 * (0x1.921fb6p+2f * k)) / Df;
      for (int d = 0; d < D; ++d) g[d] = c1 * x[d] + c2 * orc_sin2pi(k * x[d]);
      break;
    }
    case ORC_OBJ_BEALE: {
      float x1 = x[0], x2 = x[1], x22 = sq(x2), x23 = x22 * x2;
      float a = (1.5f - x1) + x1 * x2;
      float b = (2.25f - x1) + x1 * x22;
      float c = (2.625f - x1) + x1 * x23;
      g[0] = (2.0f * a * (x2 - 1.0f) + 2.0f * b * (x22 - 1.0f)) + 2.0f * c * (x23 - 1.0f);
      g[1] = (2.0f * a * x1 + 2.0f * b * (2.0f * x1 * x2)) + 2.0f * c * (3.0f * x1 * x22);
      break;
    }
    case ORC_OBJ_BOOTH: {
      float a = (x[0] + 2.0f * x[1]) - 7.0f;
      float b = (2.0f * x[0] + x[1]) - 5.0f;
      g[0] = 2.0f * a + 4.0f * b;
      g[1] = 4.0f * a + 2.0f * b;
      break;
    }
    case ORC_OBJ_HIMMELBLAU: {
      float a = (sq(x[0]) + x[1]) - 11.0f;
      float b = (x[0] + sq(x[1])) - 7.0f;
      g[0] = 4.0f * a * x[0] + 2.0f * b;
      g[1] = 2.0f * a + 4.0f * b * x[1];
      break;
    }
    case ORC_OBJ_QUADRATIC:
      g[0] = 2.0f * prm(prob, 0, 1.0f) * (x[0] - 1.0f);
      if (D > 1) g[1] = 2.0f * (x[1] + 2.0f);
      break;
    case ORC_OBJ_BOUNDARY_QUADRATIC:
      g[0] = 2.0f * (x[0] + 1.0f);
      for (int d = 1; d < D; ++d) g[d] = 0.0f;
      break;
    default:
      for (int d = 0; d < D; ++d) g[d] = 0.0f;
  }
  return f;
}

/* ------------------------------------------------------------------------ */
/* thread pool helper: run fn(arg, tid, nthreads) on nthreads threads        */
/* ------------------------------------------------------------------------ */
typedef void (*par_fn)(void* arg, int tid, int nth);
typedef struct { par_fn fn; void* arg; int tid, nth; } par_job;
static void* par_tramp(void* p) {
  par_job* j = (par_job*)p;
  j->fn(j->arg, j->tid, j->nth);
  return NULL;
}
static void par_run(par_fn fn, void* arg, int nth) {
  if (nth <= 1) { fn(arg, 0, 1); return; }
  pthread_t th[256];
  par_job jobs[256];
  if (nth > 256) nth = 256;
  for (int t = 1; t < nth; ++t) {
    jobs[t].fn = fn; jobs[t].arg = arg; jobs[t].tid = t; jobs[t].nth = nth;
    pthread_create(&th[t], NULL, par_tramp, &jobs[t]);
  }
  fn(arg, 0, nth);
  for (int t = 1; t < nth; ++t) pthread_join(th[t], NULL);
}
static inline void split_range(int64_t n, int tid, int nth, int64_t* b, int64_t* e) {
  *b = (n * tid) / nth;
  *e = (n * (tid + 1)) / nth;
}

/* ------------------------------------------------------------------------ */
/* Latin hypercube strata: McKay, Beckman & Conover (1979) with the          */
/* permutation of each dim as a Feistel bijection cycle-walked into [0, n)   */
/* (Black & Rogaway, CT-RSA 2002); round keys = one Philox draw of (d, seed) */
/* ------------------------------------------------------------------------ */
#define ORC_TAG_LHS 0x4C485331u /* "LHS1" */

static uint32_t lhs_round(uint32_t r, uint32_t key) {
  uint32_t x = r ^ key;
  x *= 0xD2511F53u;
  x ^= x >> 15;
  x *= 0xCD9E8D57u;
  x ^= x >> 13;
  return x;
}

static uint32_t lhs_feistel(uint32_t v, int h, const uint32_t key[4]) {
  const uint32_t mask = (1u << h) - 1u;
  uint32_t L = v >> h, R = v & mask;
  for (int r = 0; r < 4; ++r) {
    const uint32_t nl = R;
    R = L ^ (lhs_round(R, key[r]) & mask);
    L = nl;
  }
  return (L << h) | R;
}

uint32_t orc_lhs_stratum(uint32_t i, uint32_t n, uint32_t d, uint64_t seed) {
  int bits = 0;
  while (bits < 32 && (1ull << bits) < (uint64_t)n) ++bits;
  const int h = bits < 2 ? 1 : (bits + 1) / 2;
  uint32_t key[4];
  philox_step(seed, d, 0u, 0u, ORC_TAG_LHS, key);
  const uint64_t domain = 1ull << (2 * h);
  uint32_t v = i;
  for (uint64_t it = 0; it < domain; ++it) {
    v = lhs_feistel(v, h, key);
    if (v < n) return v;
  }
  return i;
}

/* ------------------------------------------------------------------------ */
/* init (src/utils.jl:23-84, src/init.jl:38-54)                             */
/* ------------------------------------------------------------------------ */
static inline int64_t swarm_nglobal(const orc_swarm* s) { return s->nglobal > 0 ? s->nglobal : s->n; }

void orc_init(const orc_problem* prob, orc_swarm* s, uint64_t seed, int32_t sampler) {
  const int D = prob->dim;
  const int64_t n = s->n, ng = swarm_nglobal(s);
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t gi = (uint32_t)(s->first + i);  /* index in the whole swarm */
    for (int j = 0; j < (D + 3) / 4; ++j) {
      uint32_t o[4];
      philox_step(seed, gi, (uint32_t)j, 0u, ORC_TAG_INIT, o);
      for (int k = 0; k < 4; ++k) {
        int d = 4 * j + k;
        if (d >= D) break;
        float u = orc_u01(o[k]);
        float xv;
        if (sampler == ORC_SAMPLER_UNBOUNDED) {
          float u0 = prob->u0[d];
          float a = fabsf(u0);
          xv = (a > 0.0f) ? (u0 + (u * a)) : u;
        } else if (sampler == ORC_SAMPLER_LHS) {
          /* x = ((stratum + U) / n) (ub - lb) + lb */
          const float t = ((float)orc_lhs_stratum(gi, (uint32_t)ng, (uint32_t)d, seed) + u) / (float)ng;
          xv = (t * (prob->ub[d] - prob->lb[d])) + prob->lb[d];
        } else {
          /* uniform_itr: rand(T) * (ub[i] - lb[i]) + lb[i] */
          xv = (u * (prob->ub[d] - prob->lb[d])) + prob->lb[d];
        }
        s->x[d * n + i] = xv;
        s->v[d * n + i] = 0.0f;
        s->pbest[d * n + i] = xv;
      }
    }
    float c = orc_objective(prob, s->x + i, n, 1);
    if (prob->ncons > 0) c = c + orc_penalty(prob, s->x + i, n, 1.0f);
    s->cost[i] = c;
    s->pcost[i] = c;
  }
  orc_select_gbest(prob, s, ORC_GBEST_FROM_PBEST);
}

/* the uniform draws of init and of step t, exported so that an independent
 * restatement (the float64 one, oracle/pso_f64.py) consumes the same random
 * numbers: u / r1 / r2 [d*n + i] of particle first + i in dim d */
void orc_init_draws(uint64_t seed, int64_t first, int64_t n, int32_t dim, float* u) {
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < (dim + 3) / 4; ++j) {
      uint32_t o[4];
      philox_step(seed, (uint32_t)(first + i), (uint32_t)j, 0u, ORC_TAG_INIT, o);
      for (int k = 0; k < 4 && 4 * j + k < dim; ++k) u[(int64_t)(4 * j + k) * n + i] = orc_u01(o[k]);
    }
}

void orc_step_draws(uint64_t seed, int64_t first, int64_t n, int32_t dim, uint32_t t, float* r1, float* r2) {
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < (dim + 1) / 2; ++j) {
      uint32_t o[4];
      philox_step(seed, (uint32_t)(first + i), (uint32_t)j, t, ORC_TAG_STEP, o);
      for (int h = 0; h < 2 && 2 * j + h < dim; ++h) {
        r1[(int64_t)(2 * j + h) * n + i] = orc_u01(o[2 * h]);
        r2[(int64_t)(2 * j + h) * n + i] = orc_u01(o[2 * h + 1]);
      }
    }
}

void orc_select_gbest(const orc_problem* prob, orc_swarm* s, int32_t gbest_source) {
  const int64_t n = s->n;
  uint64_t best = ~0ull;
  for (int64_t i = 0; i < n; ++i) {
    uint64_t k = orc_argmin_key(s->pcost[i], (uint32_t)(s->first + i));
    if (k < best) best = k;
  }
  int64_t gi = (int64_t)(uint32_t)best, li = gi - s->first;
  const float* src = (gbest_source == ORC_GBEST_FROM_POSITION) ? s->x : s->pbest;
  for (int d = 0; d < prob->dim; ++d) s->g[d] = src[d * n + li];
  s->gcost = s->pcost[li];
  s->gidx = gi;
}

/* ------------------------------------------------------------------------ */
/* the particle update (src/kernels.jl:1-26)                                */
/*   v' = w.*v .+ c1.*r1.*(pbest-x) .+ c2.*r2.*(g-x);  x' = clamp(x+v')      */
/*   cost = f(x');  if cost < pcost: pbest = x', pcost = cost                */
/* ------------------------------------------------------------------------ */
static inline float clamp_lb_ub(float x, float lb, float ub) {
  x = (x < lb) ? lb : x;  /* max.(x, lb) */
  x = (x > ub) ? ub : x;  /* min.(x, ub) */
  return x;
}

static inline void update_dims(const orc_problem* prob, float* x, float* v, const float* p,
                               const float* g, int64_t stride, uint32_t i, uint32_t t, uint64_t seed,
                               float w, float c1, float c2) {
  const int D = prob->dim;
  for (int j = 0; j < (D + 1) / 2; ++j) {
    uint32_t o[4];
    philox_step(seed, i, (uint32_t)j, t, ORC_TAG_STEP, o);
    for (int h = 0; h < 2; ++h) {
      int d = 2 * j + h;
      if (d >= D) break;
      float r1 = orc_u01(o[2 * h]);
      float r2 = orc_u01(o[2 * h + 1]);
      float xd = x[d * stride], vd = v[d * stride], pd = p[d * stride];
      float a = w * vd;
      float b = (c1 * r1) * (pd - xd);
      float c = (c2 * r2) * (g[d] - xd);
      float vn = (a + b) + c;
      float xn = clamp_lb_ub(xd + vn, prob->lb[d], prob->ub[d]);
      v[d * stride] = vn;
      x[d * stride] = xn;
    }
  }
}

typedef struct {
  const orc_problem* prob;
  orc_swarm* s;
  uint64_t seed;
  uint32_t t;
  float w, c1, c2;
} sync_arg;

static void sync_worker(void* a_, int tid, int nth) {
  sync_arg* a = (sync_arg*)a_;
  orc_swarm* s = a->s;
  const int D = a->prob->dim;
  const int64_t n = s->n;
  int64_t b, e;
  split_range(n, tid, nth, &b, &e);
  for (int64_t i = b; i < e; ++i) {
    const int64_t gi = s->first + i;  /* index in the whole swarm */
    update_dims(a->prob, s->x + i, s->v + i, s->pbest + i, s->g, n, (uint32_t)gi, a->t, a->seed,
                a->w, a->c1, a->c2);
    float c = orc_objective(a->prob, s->x + i, n, 1);
    /* the sync step passes the 1-based particle index as iter (src/kernels.jl:151) */
    if (a->prob->ncons > 0) c = c + orc_penalty(a->prob, s->x + i, n, (float)(gi + 2));
    s->cost[i] = c;
    if (c < s->pcost[i]) {
      s->pcost[i] = c;
      for (int d = 0; d < D; ++d) s->pbest[d * n + i] = s->x[d * n + i];
    }
  }
}

float orc_sync_run(const orc_problem* prob, orc_swarm* s, uint64_t seed, uint32_t t0,
                   int32_t iters, float w, float wdamp, float c1, float c2,
                   int32_t gbest_source, int32_t nthreads) {
  for (int32_t it = 0; it < iters; ++it) {
    sync_arg a = {prob, s, seed, t0 + (uint32_t)it, w, c1, c2};
    par_run(sync_worker, &a, nthreads);
    orc_select_gbest(prob, s, gbest_source);
    w = w * wdamp;
  }
  return w;
}

/* ------------------------------------------------------------------------ */
/* async (src/kernels.jl:196-225): each particle loops over all iterations   */
/* against a private best seeded from the swarm best.  The private best is   */
/* either the seed value or, once the particle's own best beat it, the       */
/* particle's own best -- kept as a flag.                                    */
/* ------------------------------------------------------------------------ */
int32_t orc_async_lanes(int32_t dim, int32_t* slice) {
  int lanes = 1;
  if (dim > 16) {
    int need = (dim + 15) / 16;
    while (lanes < need) lanes <<= 1;
    if (lanes > 32) lanes = 32;
  }
  int S = (dim + lanes - 1) / lanes;
  S += S & 1;
  if (slice) *slice = S;
  return lanes;
}

typedef struct {
  const orc_problem* prob;
  orc_swarm* s;
  uint64_t seed;
  uint32_t t0;
  int32_t iters, lanes;
  float w, wdamp, c1, c2;
} async_arg;

static void async_worker(void* a_, int tid, int nth) {
  async_arg* a = (async_arg*)a_;
  orc_swarm* s = a->s;
  const orc_problem* prob = a->prob;
  const int D = prob->dim;
  const int64_t n = s->n;
  int64_t b, e;
  split_range(n, tid, nth, &b, &e);
  float* gp = (float*)malloc(sizeof(float) * (size_t)D);
  for (int64_t i = b; i < e; ++i) {
    int own = 0;
    float w = a->w;
    for (int32_t it = 0; it < a->iters; ++it) {
      for (int d = 0; d < D; ++d) gp[d] = own ? s->pbest[d * n + i] : s->g[d];
      update_dims(prob, s->x + i, s->v + i, s->pbest + i, gp, n, (uint32_t)(s->first + i),
                  a->t0 + (uint32_t)it, a->seed, w, a->c1, a->c2);
      float c = orc_objective(prob, s->x + i, n, a->lanes);
      s->cost[i] = c;
      if (c < s->pcost[i]) {
        s->pcost[i] = c;
        for (int d = 0; d < D; ++d) s->pbest[d * n + i] = s->x[d * n + i];
      }
      if (s->pcost[i] < s->gcost) own = 1;
      w = w * a->wdamp;
    }
  }
  free(gp);
}

float orc_async_run(const orc_problem* prob, orc_swarm* s, uint64_t seed, uint32_t t0,
                    int32_t iters, float w, float wdamp, float c1, float c2,
                    int32_t lanes, int32_t nthreads) {
  async_arg a = {prob, s, seed, t0, iters, lanes, w, wdamp, c1, c2};
  par_run(async_worker, &a, nthreads);
  orc_select_gbest(prob, s, ORC_GBEST_FROM_PBEST);
  for (int32_t it = 0; it < iters; ++it) w = w * wdamp;
  return w;
}
