// pps_ode.cuh -- the ode_pso objective: integrate the model with the
// particle's position as its parameters, SSE against observations.
//
// Reference: parameter_estim_ode! (src/ode_pso.jl:113-170) builds one ODE
// problem per particle (default_prob_func, :43-45), integrates them with
// DiffEqGPU's GPUTsit5 and reduces the loss with _reduce_losses! (:47-52):
//   loss = sum over save points of sum over states (data - u)^2.
// The workload integrates with the classical fixed-step RK4 instead; the
// stage arithmetic below is exactly the CPU restatement's (fused multiply-adds
// where it writes fmaf).
// Right-hand sides (the reference's benchmark models):
//   Lotka-Volterra  benchmarks/Lotka_Volterra/lotka_volterra.jl:9-13
//     du1 = p1 u1 - p2 u1 u2,  du2 = -p3 u2 + p4 u1 u2
//   FitzHugh-Nagumo benchmarks/Fitzhugh_Nagumo/ode_estimation.jl:6-12
//     dv = v - v^3/3 - w + l,  dw = tinv (v + a - b w),  p = (a, b, tinv), l fixed
// evaluated in factored form -- u1 fma(-p2, u2, p1), u2 fma(p4, u1, -p3),
// (fma(v^3, -1/3, v) - w) + l, tinv fma(-b, w, v + a) -- two roundings per
// term and no division, which halves the instructions of an RK4 step.
#pragma once
#include "pps_device.cuh"

namespace pps {

constexpr int kOdeLV = 0;
constexpr int kOdeFHN = 1;
constexpr int kOdeMaxSaves = 4096;

// Fit configuration, packed by the host from pps_problem.params:
// params = [u0_1, u0_2, dt, nsteps, save_every, l (FHN)], data = nsaves x 2.
struct OdeCfg {
  float u0a, u0b, dt, l;
  int nsteps, save_every, nsaves;
};

__host__ __device__ inline OdeCfg ode_cfg(const ObjParams& op, int64_t ndata) {
  OdeCfg c;
  c.u0a = op.p[0];
  c.u0b = op.p[1];
  c.dt = op.p[2];
  c.nsteps = (int)op.p[3];
  c.save_every = (int)op.p[4];
  c.l = op.p[5];
  c.nsaves = (int)(ndata / 2);
  return c;
}

template <int MODEL>
__device__ __forceinline__ void ode_rhs(const float* p, float l, float u0, float u1, float& d0, float& d1) {
  if constexpr (MODEL == kOdeLV) {
    d0 = __fmul_rn(u0, __fmaf_rn(-p[1], u1, p[0]));
    d1 = __fmul_rn(u1, __fmaf_rn(p[3], u0, -p[2]));
  } else {
    const float v3 = __fmul_rn(__fmul_rn(u0, u0), u0);
    d0 = __fadd_rn(__fsub_rn(__fmaf_rn(v3, -0x1.555556p-2f, u0), u1), l);
    d1 = __fmul_rn(p[2], __fmaf_rn(-p[1], u1, __fadd_rn(u0, p[0])));
  }
}

template <int MODEL>
__device__ __forceinline__ void rk4_step(const float* p, float l, float dt, float h2, float h6, float& u0, float& u1) {
  float k1a, k1b, k2a, k2b, k3a, k3b, k4a, k4b;
  ode_rhs<MODEL>(p, l, u0, u1, k1a, k1b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(h2, k1a, u0), __fmaf_rn(h2, k1b, u1), k2a, k2b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(h2, k2a, u0), __fmaf_rn(h2, k2b, u1), k3a, k3b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, k3a, u0), __fmaf_rn(dt, k3b, u1), k4a, k4b);
  float sa = __fmaf_rn(2.0f, k2a, k1a);
  sa = __fmaf_rn(2.0f, k3a, sa);
  sa = __fadd_rn(sa, k4a);
  float sb = __fmaf_rn(2.0f, k2b, k1b);
  sb = __fmaf_rn(2.0f, k3b, sb);
  sb = __fadd_rn(sb, k4b);
  u0 = __fmaf_rn(h6, sa, u0);
  u1 = __fmaf_rn(h6, sb, u1);
}

// SSE of the RK4 trajectory against data[nsaves][2] (t = 0 included)
template <int MODEL>
__device__ __forceinline__ float ode_loss(const float* p, const OdeCfg& c, const float* data) {
  const float dt = c.dt;
  const float h2 = __fmul_rn(dt, 0.5f);
  const float h6 = __fdiv_rn(dt, 6.0f);
  float u0 = c.u0a, u1 = c.u0b;
  float e0 = __fsub_rn(data[0], u0), e1 = __fsub_rn(data[1], u1);
  float acc = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
  int m = 1;
  int next = c.save_every;
  for (int s = 1; s <= c.nsteps && m < c.nsaves; ++s) {
    rk4_step<MODEL>(p, c.l, dt, h2, h6, u0, u1);
    if (s == next) {
      e0 = __fsub_rn(data[2 * m], u0);
      e1 = __fsub_rn(data[2 * m + 1], u1);
      acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
      ++m;
      next += c.save_every;
    }
  }
  return acc;
}

}  // namespace pps
