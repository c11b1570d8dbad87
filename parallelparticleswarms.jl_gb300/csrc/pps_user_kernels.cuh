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
#include "pps_vec.cuh"

// resident blocks each kernel is compiled for (register cap 65536 / (256 x
// blocks)): 4 leaves 64 registers a thread and 32 warps per SM for one or two
// particles per thread, 2 leaves 128 for four.  PPS_USER_MINBLOCKS, when
// defined, sets all of them.
#ifdef PPS_USER_MINBLOCKS
#define PPS_USER_MB4 PPS_USER_MINBLOCKS
#define PPS_USER_MB2 PPS_USER_MINBLOCKS
#else
#define PPS_USER_MB4 4
#define PPS_USER_MB2 2
#endif

namespace pps {

constexpr int kUserThreads = 256;

__device__ __forceinline__ void user_params(float* sp, const ObjParams& op) {
  if (threadIdx.x < 8) sp[threadIdx.x] = (int)threadIdx.x < op.np ? op.p[threadIdx.x] : 0.0f;
}

}  // namespace pps

extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB4)
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
        if (sampler == kSamplerUnbounded) {
          const float z = u0 ? u0[d] : 0.0f;
          const float a = fabsf(z);
          x = (a > 0.0f) ? __fadd_rn(z, __fmul_rn(u, a)) : u;
        } else if (sampler == kSamplerLhs) {
          x = valid ? lhs_position((uint32_t)i, (uint32_t)s.n, (uint32_t)d, u, s.lb[d], s.ub[d], k0, k1) : 0.0f;
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

// Each thread owns PPT consecutive particles (float / float2 / float4 along
// the particle axis, as the registered step kernel), the grid of resident
// blocks strides over the groups.  Dims are walked in pairs, one Philox call
// per particle and pair, the loads of the next pair issued before the current
// pair is computed.  The objective then runs once per particle over the
// column this thread has just written; that read-back mostly misses L2 at
// large swarms (at 2^20 particles x 100 dims about 124 MB of new positions
// are in flight across the GPU).  A source that defines PPS_HAS_STREAM folds
// the objective into registers as each dim moves (pps_stream_add in
// increasing d) and reads nothing back, as the registered kernels do.
namespace pps {

template <int PPT, bool CONS>
__device__ __forceinline__ void user_step(const SwarmDev& s, const ObjParams& op, const float* data, long long ndata,
                                          const PhiloxKeys& keys, float c1, float c2, int from_position) {
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
  const int64_t ngroups = (n + PPT - 1) / PPT;  // the last group may hold padding
  float* X = s.X;  // not restrict: the objective reads back what this thread stores
  float* V = s.V;
  float* P = s.P;
  unsigned long long best = ~0ull;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < ngroups; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i0 = q * PPT;
    uint8_t fl[PPT];
    ldflags<PPT>(fl, s.flag + i0);
    bool anyfl = false;
#pragma unroll
    for (int k = 0; k < PPT; ++k) anyfl |= (fl[k] != 0);
    ConsAcc ca[PPT];
    if constexpr (CONS) {
#pragma unroll
      for (int k = 0; k < PPT; ++k) ca[k].start(s.cons, s.ncons, D);
    }
#ifdef PPS_HAS_STREAM
    pps_stream fs[PPT];  // the objective folded over the dims as they move
#pragma unroll
    for (int k = 0; k < PPT; ++k) pps_stream_start(&fs[k], D, sp, data, ndata);
#endif
    float xa[PPT], va[PPT], pa[PPT], xb[PPT], vb[PPT], pb[PPT];
    ldv<PPT>(xa, X + i0);
    ldv<PPT>(va, V + i0);
    ldv<PPT>(pa, P + i0);
    if (D > 1) {
      ldv<PPT>(xb, X + npad + i0);
      ldv<PPT>(vb, V + npad + i0);
      ldv<PPT>(pb, P + npad + i0);
    }
    for (int j = 0; j < D; j += 2) {
      float nxa[PPT], nva[PPT], npa[PPT], nxb[PPT], nvb[PPT], npb[PPT];
      if (j + 2 < D) {
        const int64_t o = (int64_t)(j + 2) * npad + i0;
        ldv<PPT>(nxa, X + o);
        ldv<PPT>(nva, V + o);
        ldv<PPT>(npa, P + o);
      }
      if (j + 3 < D) {
        const int64_t o = (int64_t)(j + 3) * npad + i0;
        ldv<PPT>(nxb, X + o);
        ldv<PPT>(nvb, V + o);
        ldv<PPT>(npb, P + o);
      }
      Rand4 r[PPT];
#pragma unroll
      for (int k = 0; k < PPT; ++k) r[k] = philox4x32_10((uint32_t)(i0 + k), (uint32_t)(j >> 1), t, kTagStep, keys);
      {  // dim j
        const int64_t o = (int64_t)j * npad + i0;
        if (anyfl) {  // the personal-best copies deferred from the last step
#pragma unroll
          for (int k = 0; k < PPT; ++k) pa[k] = fl[k] ? xa[k] : pa[k];
          stv<PPT>(P + o, pa);
        }
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          va[k] = velocity(xa[k], va[k], pa[k], sg[j], w, c1, c2, u01(r[k].a), u01(r[k].b));
          xa[k] = clamp_lb_ub(__fadd_rn(xa[k], va[k]), slb[j], sub[j]);
          if constexpr (CONS) ca[k].add(s.cons, s.ncons, D, j, xa[k]);
#ifdef PPS_HAS_STREAM
          pps_stream_add(&fs[k], j, xa[k], D, sp, data, ndata);
#endif
        }
        stv<PPT>(X + o, xa);
        stv<PPT>(V + o, va);
      }
      if (j + 1 < D) {  // dim j + 1
        const int64_t o = (int64_t)(j + 1) * npad + i0;
        if (anyfl) {
#pragma unroll
          for (int k = 0; k < PPT; ++k) pb[k] = fl[k] ? xb[k] : pb[k];
          stv<PPT>(P + o, pb);
        }
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          vb[k] = velocity(xb[k], vb[k], pb[k], sg[j + 1], w, c1, c2, u01(r[k].c), u01(r[k].d));
          xb[k] = clamp_lb_ub(__fadd_rn(xb[k], vb[k]), slb[j + 1], sub[j + 1]);
          if constexpr (CONS) ca[k].add(s.cons, s.ncons, D, j + 1, xb[k]);
#ifdef PPS_HAS_STREAM
          pps_stream_add(&fs[k], j + 1, xb[k], D, sp, data, ndata);
#endif
        }
        stv<PPT>(X + o, xb);
        stv<PPT>(V + o, vb);
      }
#pragma unroll
      for (int k = 0; k < PPT; ++k) {
        xa[k] = nxa[k]; va[k] = nva[k]; pa[k] = npa[k];
        xb[k] = nxb[k]; vb[k] = nvb[k]; pb[k] = npb[k];
      }
    }
    float pc[PPT], cc[PPT];
    ldv<PPT>(pc, s.pcost + i0);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const bool valid = i0 + k < n;
      float c = __int_as_float(0x7f800000);
      if (valid) {
#ifdef PPS_HAS_STREAM
        c = pps_stream_finish(&fs[k], D, sp, data, ndata);
#else
        c = pps_objective(pps_point{X + i0 + k, npad}, D, sp, data, ndata);
#endif
        if constexpr (CONS) c = __fadd_rn(c, penalty(ca[k], s.ncons, __uint2float_rn((uint32_t)(i0 + k + 2))));
      }
      cc[k] = c;
      // if cost < best_cost: best = position (strict <, src/kernels.jl:21-24)
      fl[k] = (valid && c < pc[k]) ? 1 : 0;
      pc[k] = fl[k] ? c : pc[k];
      if (valid) {
        const unsigned long long key = argmin_key(pc[k], (uint32_t)(i0 + k));
        best = key < best ? key : best;
      }
    }
    stv<PPT>(s.pcost + i0, pc);
    stv<PPT>(s.cost + i0, cc);
    stflags<PPT>(s.flag + i0, fl);
  }
  if (publish_block_min(best, st)) finish_iteration(s, from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
}

}  // namespace pps

extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB4)
    pps_user_step1(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, pps::PhiloxKeys keys,
                   float c1, float c2, int from_position) {
  pps::user_step<1, false>(s, op, data, ndata, keys, c1, c2, from_position);
}

extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB4)
    pps_user_step2(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, pps::PhiloxKeys keys,
                   float c1, float c2, int from_position) {
  pps::user_step<2, false>(s, op, data, ndata, keys, c1, c2, from_position);
}

// the constrained path: calc_penalty with iter = the 1-based particle index
// (src/kernels.jl:77,151), one particle per thread
extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB4)
    pps_user_step_cons(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata,
                       pps::PhiloxKeys keys, float c1, float c2, int from_position) {
  pps::user_step<1, true>(s, op, data, ndata, keys, c1, c2, from_position);
}

extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB2)
    pps_user_step4(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, pps::PhiloxKeys keys,
                   float c1, float c2, int from_position) {
  pps::user_step<4, false>(s, op, data, ndata, keys, c1, c2, from_position);
}

// ParallelPSOKernel(global_update = false) for a user objective: the whole run
// in one launch (src/kernels.jl:196-225, src/lowerlevel_solve.jl:95-121).
// Each particle runs every iteration against a private global best that
// starts as the swarm's and becomes its own personal best once that beats the
// starting cost (:215-218); w is damped in the kernel (:219); personal-best
// copies are immediate.  The state stays in HBM (one thread per particle,
// grid-stride), as the objective reads the position back; the run ends with
// the argmin over the personal bests (:119-120).
extern "C" __global__ void __launch_bounds__(pps::kUserThreads, PPS_USER_MB4)
    pps_user_async(pps::SwarmDev s, pps::ObjParams op, const float* data, long long ndata, pps::PhiloxKeys keys,
                   int iters, float c1, float c2) {
  using namespace pps;
  extern __shared__ float sm[];
  __shared__ float sp[8];
  const int D = s.dim;
  float* sg = sm;
  float* slb = sm + D;
  float* sub = sm + 2 * D;
  IterState* st = s.st;
  const uint32_t t0 = st->t;
  const float w0 = st->w, wdamp = st->wdamp, gcost0 = st->gcost;
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
    bool own = false;
    float w = w0;
    float pc = s.pcost[i];
    for (int it = 0; it < iters; ++it) {
      const uint32_t t = t0 + (uint32_t)it;
      for (int j = 0; j < D; j += 2) {
        const Rand4 r = philox4x32_10((uint32_t)i, (uint32_t)(j >> 1), t, kTagStep, keys);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int d = j + h;
          if (d >= D) break;
          const int64_t o = (int64_t)d * npad + i;
          const float x = X[o], p = P[o];
          const float gd = own ? p : sg[d];
          const float v = velocity(x, V[o], p, gd, w, c1, c2, u01(h ? r.c : r.a), u01(h ? r.d : r.b));
          X[o] = clamp_lb_ub(__fadd_rn(x, v), slb[d], sub[d]);
          V[o] = v;
        }
      }
      const float c = pps_objective(pps_point{X + i, npad}, D, sp, data, ndata);
      s.cost[i] = c;
      if (c < pc) {  // strict <, src/kernels.jl:21-24
        pc = c;
        for (int d = 0; d < D; ++d) P[(int64_t)d * npad + i] = X[(int64_t)d * npad + i];
      }
      if (pc < gcost0) own = true;
      w = __fmul_rn(w, wdamp);
    }
    s.pcost[i] = pc;
    const unsigned long long key = argmin_key(pc, (uint32_t)i);
    best = key < best ? key : best;
  }
  float wf = w0;  // the inertia after the run, for every block alike
  for (int it = 0; it < iters; ++it) wf = __fmul_rn(wf, wdamp);
  if (publish_block_min(best, st)) finish_iteration(s, false, t0 + (uint32_t)iters, wf);
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

#ifdef PPS_HAS_GRADIENT
// HybridPSO's local stage on a user objective with a gradient: L-BFGS with the
// history in shared memory (dim <= 16) or thread-local memory (dim <= 64),
// Broyden with the inverse Jacobian in shared memory (dim <= 16)
#include "pps_local.cuh"

extern "C" __global__ void __launch_bounds__(pps::kLbfgsThreads)
    pps_user_lbfgs16(const float* X0, int64_t ld, int64_t n, pps::ObjParams op, const float* lbp, const float* ubp,
                     pps::LocalOpts o, float* xout, float* fout, float* itout) {
  pps::lbfgs_run<pps::kUserObjective, 16, true>(X0, ld, n, op, lbp, ubp, o, xout, fout, itout);
}

extern "C" __global__ void __launch_bounds__(128)
    pps_user_lbfgs64(const float* X0, int64_t ld, int64_t n, pps::ObjParams op, const float* lbp, const float* ubp,
                     pps::LocalOpts o, float* xout, float* fout, float* itout) {
  pps::lbfgs_run<pps::kUserObjective, 64, false>(X0, ld, n, op, lbp, ubp, o, xout, fout, itout);
}

extern "C" __global__ void __launch_bounds__(pps::kBroydenThreads)
    pps_user_broyden16(const float* X0, int64_t ld, int64_t n, pps::ObjParams op, const float* lbp, const float* ubp,
                       pps::LocalOpts o, float* xout, float* fout, float* itout) {
  pps::broyden_run<pps::kUserObjective, 16, true>(X0, ld, n, op, lbp, ubp, o, xout, fout, itout);
}
#endif
