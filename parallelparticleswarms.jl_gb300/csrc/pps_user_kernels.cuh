// pps_user_kernels.cuh -- init, synchronous step and point evaluation for a
// user objective.  Compiled by NVRTC after pps_user_prelude.cuh and the
// user's source (pps_user.cu); launched through the CUDA runtime's library
// API.  The particle arithmetic is that of the registered kernels
// (pps_sync.cu): the same Philox counters, update order, clamp, strict `<`
// personal-best test, deferred pbest copy and argmin publication, so a user
// objective that spells a registered one's operations reproduces its run bit
// for bit.  What differs is the evaluation: the user's function reads the new
// position back through a pps_point over the SoA column this thread has just
// written (its own writes, so no fence is needed), instead of a streaming
// accumulator.
//
// Reference behaviour restated: update_particle_state (src/kernels.jl:1-26)
// with cost = f(x', p) (:33), the sync step (src/kernels.jl:127-177), init
// (src/utils.jl:23-84), calc_penalty (src/utils.jl:320-372) when the
// problem carries constraints.
#pragma once
#include "pps_publish.cuh"

namespace pps {

constexpr int kUserThreads = 256;
constexpr int kUserSamplerUnbounded = 2;  // PPS_SAMPLER_UNBOUNDED

__device__ __forceinline__ void user_params(float* sp, const ObjParams& op) {
  if (threadIdx.x < 8) sp[threadIdx.x] = (int)threadIdx.x < op.np ? op.p[threadIdx.x] : 0.0f;
}

}  // namespace pps

extern "C" __global__ void __launch_bounds__(pps::kUserThreads)
    pps_user_init(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, unsigned long long seed,
                  int sampler, const float* u0) {
  using namespace pps;
  __shared__ float sp[8];
  user_params(sp, op);
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int D = s.dim;
  unsigned long long key = ~0ull;
  if (i < s.npad) {
    const bool valid = i < s.n;
    ConsAcc ca;
    if (s.ncons > 0) ca.start(s.cons, s.ncons, D);
    for (int j = 0; j < D; j += 4) {
      const Rand4 r = philox4x32_10((uint32_t)i, (uint32_t)(j >> 2), 0u, kTagInit, k0, k1);
      const uint32_t rr[4] = {r.a, r.b, r.c, r.d};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int d = j + h;
        if (d >= D) break;
        const float u = u01(rr[h]);
        float x;
        if (sampler == kUserSamplerUnbounded) {
          const float z = u0 ? u0[d] : 0.0f;
          const float a = fabsf(z);
          x = (a > 0.0f) ? __fadd_rn(z, __fmul_rn(u, a)) : u;
        } else {
          const float lo = s.lb[d], hi = s.ub[d];
          x = __fadd_rn(__fmul_rn(u, __fsub_rn(hi, lo)), lo);  // rand(T) * (ub - lb) + lb
        }
        if (!valid) x = 0.0f;
        const int64_t o = (int64_t)d * s.npad + i;
        s.X[o] = x;
        s.V[o] = 0.0f;
        s.P[o] = x;
        if (s.ncons > 0) ca.add(s.cons, s.ncons, D, d, x);
      }
    }
    float c = __int_as_float(0x7f800000);
    if (valid) {
      c = pps_objective(pps_point{s.X + i, s.npad}, D, sp, data, ndata);
      if (s.ncons > 0) c = __fadd_rn(c, penalty(ca, s.ncons, 1.0f));
      key = argmin_key(c, (uint32_t)i);
    }
    s.cost[i] = c;
    s.pcost[i] = c;
    s.flag[i] = 0;
  }
  if (publish_block_min(key, s.st)) finish_iteration(s, false, 0u, s.st->w);
}

// One thread per particle, a grid of resident blocks striding over the
// swarm.  Dims are walked in pairs, one Philox call per pair.
extern "C" __global__ void __launch_bounds__(pps::kUserThreads)
    pps_user_step(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, pps::PhiloxKeys keys,
                  float c1, float c2, int from_position) {
  using namespace pps;
  extern __shared__ float sm[];
  __shared__ float sp[8];
  const int D = s.dim;
  float* sg = sm;
  float* slb = sm + D;
  float* sub = sm + 2 * D;
  IterState* st = s.st;
  const uint32_t t = st->t;
  const float w = st->w;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    sg[d] = s.g[d];
    slb[d] = s.lb[d];
    sub[d] = s.ub[d];
  }
  user_params(sp, op);
  __syncthreads();
  const int64_t npad = s.npad, n = s.n;
  float* X = s.X;  // not restrict: the objective reads back what this thread stores
  float* V = s.V;
  float* P = s.P;
  unsigned long long best = ~0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool fl = s.flag[i] != 0;
    ConsAcc ca;
    if (s.ncons > 0) ca.start(s.cons, s.ncons, D);
    for (int j = 0; j < D; j += 2) {
      const Rand4 r = philox4x32_10((uint32_t)i, (uint32_t)(j >> 1), t, kTagStep, keys);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int d = j + h;
        if (d >= D) break;
        const int64_t o = (int64_t)d * npad + i;
        float x = X[o], v = V[o], p = P[o];
        if (fl) {  // the personal-best copy deferred from the last step
          p = x;
          P[o] = p;
        }
        v = velocity(x, v, p, sg[d], w, c1, c2, u01(h ? r.c : r.a), u01(h ? r.d : r.b));
        x = clamp_lb_ub(__fadd_rn(x, v), slb[d], sub[d]);
        X[o] = x;
        V[o] = v;
        if (s.ncons > 0) ca.add(s.cons, s.ncons, D, d, x);
      }
    }
    float c = pps_objective(pps_point{X + i, npad}, D, sp, data, ndata);
    if (s.ncons > 0) c = __fadd_rn(c, penalty(ca, s.ncons, __uint2float_rn((uint32_t)(i + 2))));
    float pc = s.pcost[i];
    // if cost < best_cost: best = position (strict <, src/kernels.jl:21-24)
    const bool imp = c < pc;
    if (imp) {
      pc = c;
      s.pcost[i] = c;
    }
    s.cost[i] = c;
    s.flag[i] = imp ? 1 : 0;
    const unsigned long long key = argmin_key(pc, (uint32_t)i);
    best = key < best ? key : best;
  }
  if (publish_block_min(best, st)) finish_iteration(s, from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
}

// f[i] = objective at point i, coordinates x[d * stride + i]
extern "C" __global__ void __launch_bounds__(pps::kUserThreads)
    pps_user_eval(pps::ObjParams op, const float* data, long long ndata, const float* x, long long npts,
                  long long stride, float* f) {
  using namespace pps;
  __shared__ float sp[8];
  user_params(sp, op);
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npts) f[i] = pps_objective(pps_point{x + i, stride}, op.dim, sp, data, ndata);
}
