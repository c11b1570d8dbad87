// pps_ode.cu -- one ODE-fit swarm at a time: init and the synchronous step
// for the ode_pso objectives (parameter_estim_ode!, src/ode_pso.jl:113-170).
//
// The reference's loop per iteration: ode_update_particle_states! (:1-24),
// a host broadcast that rebuilds every particle's ODE problem, the DiffEqGPU
// solve, _reduce_losses!, ode_update_particle_costs! (:26-41) and a host
// minimum -- about five launches and five synchronisations.  Here the whole
// iteration is one launch: update, RK4 integration, SSE, personal best and
// the argmin publication fused, one thread per particle (two with packed
// RK4 losses for large swarms), observations in shared memory.
//
// The reference clamps with max(position, lb) on whole SVectors
// (src/ode_pso.jl:18-19), which compares lexicographically; this build
// clamps each parameter (max.(x, lb), min.(x, ub)) as the other kernels do.
#include <cmath>

#include <mutex>

#include "pps_internal.h"
#include "pps_ode.cuh"
#include "pps_publish.cuh"

namespace pps {

constexpr int kOdeThreads = 128;
// The step kernel's launch bounds ask for 4 resident blocks per SM: without
// them the assembler sizes the kernel for full occupancy (32 registers),
// which slows the integrators' dependent chains; with them it takes the 36-56
// registers the integrators use.
constexpr int kOdeStepMinBlocks = 4;
constexpr int kOdeMaxDim = 4;

// dynamic shared memory of a launch: the observations (2 floats per save),
// then the fixed-step Tsit5 saves' weight table (8 floats per save)
inline size_t ode_dyn_smem(const OdeCfg& c) {
  return sizeof(float) * (size_t)c.nsaves * (c.method == kOdeTsit5 ? 10 : 2);
}

// the block's dynamic shared memory: the observations at 0, the fixed-step
// Tsit5 save table behind them.  Kernels index it directly so the compiler
// keeps its loads in the shared address space.
extern __shared__ float ode_smem[];

// copies the observations to shared memory and builds the save table
// (fixed-step Tsit5 only); every thread calls it, and it ends in a barrier
template <int METHOD>
__device__ __forceinline__ void ode_smem_fill(const OdeCfg& c, const float* __restrict__ data_g) {
  for (int k = threadIdx.x; k < 2 * c.nsaves; k += blockDim.x) ode_smem[k] = data_g[k];
  if constexpr (METHOD == kOdeTsit5) tsit5_table_build(c, ode_smem + 2 * c.nsaves);
  __syncthreads();
}

// Particles per thread of the step kernel: 1, or 2 for RK4 losses packed in
// f32x2 (ode_loss2).  The packed form issues half the instructions but its
// dependent chain is slower, so it pays only when the launch is
// throughput-bound: a swarm that fills the GPU several times over, or a
// swarm run by the request server beside other launches.  A smaller swarm
// solved alone, whose launch is latency-bound, keeps one particle per thread.
constexpr int64_t kOdePackedMinParticles = (int64_t)1 << 18;

template <int MODEL, int METHOD>
__device__ __forceinline__ float ode_eval(const float (&x)[kOdeMaxDim], const OdeCfg& c, const float* data,
                                          const float* tab) {
  if constexpr (METHOD == kOdeTsit5) return tsit5_loss_tab<MODEL>(x, c, data, tab);
  else if constexpr (METHOD == kOdeTsit5Adaptive) return tsit5a_loss<MODEL>(x, c, data);
  else return ode_loss<MODEL>(x, c, data);
}

template <int MODEL, int METHOD>
__global__ void __launch_bounds__(kOdeThreads) k_init_ode(SwarmDev s, ObjParams op, OdeCfg cfg,
                                                          const float* __restrict__ data_g, uint64_t seed,
                                                          int sampler, const float* __restrict__ u0) {
  ode_smem_fill<METHOD>(cfg, data_g);
  const float* data = ode_smem;
  const float* tab = ode_smem + 2 * cfg.nsaves;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int D = s.dim;
  unsigned long long key = ~0ull;
  if (i < s.npad) {
    const bool valid = i < s.n;
    float x[kOdeMaxDim] = {0.0f, 0.0f, 0.0f, 0.0f};
    const Rand4 r = philox4x32_10((uint32_t)i, 0u, 0u, kTagInit, k0, k1);
    const uint32_t rr[4] = {r.a, r.b, r.c, r.d};
#pragma unroll
    for (int d = 0; d < kOdeMaxDim; ++d) {
      if (d < D) {
        const float u = u01(rr[d]);
        float xv;
        if (sampler == PPS_SAMPLER_UNBOUNDED) {
          const float z = u0 ? u0[d] : 0.0f;
          const float a = fabsf(z);
          xv = (a > 0.0f) ? __fadd_rn(z, __fmul_rn(u, a)) : u;
        } else if (sampler == PPS_SAMPLER_LHS) {
          xv = valid ? lhs_position((uint32_t)i, (uint32_t)s.n, (uint32_t)d, u, s.lb[d], s.ub[d], k0, k1) : 0.0f;
        } else {
          xv = __fadd_rn(__fmul_rn(u, __fsub_rn(s.ub[d], s.lb[d])), s.lb[d]);
        }
        x[d] = valid ? xv : 0.0f;
        const int64_t o = (int64_t)d * s.npad + i;
        s.X[o] = x[d];
        s.V[o] = 0.0f;
        s.P[o] = x[d];
      }
    }
    const float c = valid ? ode_eval<MODEL, METHOD>(x, cfg, data, tab) : __int_as_float(0x7f800000);
    s.cost[i] = c;
    s.pcost[i] = c;
    s.flag[i] = 0;
    if (valid) key = argmin_key(c, (uint32_t)i);
  }
  if (publish_block_min(key, s.st)) finish_iteration(s, false, 0u, s.st->w);
}

template <int MODEL, int METHOD, int PPT>
__global__ void __launch_bounds__(kOdeThreads, kOdeStepMinBlocks) k_sync_step_ode(SwarmDev s, ObjParams op, OdeCfg cfg,
                                                               const float* __restrict__ data_g, uint64_t seed,
                                                               float c1, float c2, int from_position, float one) {
  static_assert(PPT == 1 || (PPT == 2 && METHOD == kOdeRk4), "two particles per thread: RK4 only");
  __shared__ float sg[kOdeMaxDim], slb[kOdeMaxDim], sub[kOdeMaxDim];
  IterState* st = s.st;
  const uint32_t t = st->t;
  const float w = st->w;
  const int D = s.dim;
  if (threadIdx.x < D) {
    sg[threadIdx.x] = s.g[threadIdx.x];
    slb[threadIdx.x] = s.lb[threadIdx.x];
    sub[threadIdx.x] = s.ub[threadIdx.x];
  }
  ode_smem_fill<METHOD>(cfg, data_g);
  const float* data = ode_smem;
  const float* tab = ode_smem + 2 * cfg.nsaves;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  // this thread's particles: i0 (and i0 + blockDim.x) of the block's tile
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x * PPT + threadIdx.x;
  float x[PPT][kOdeMaxDim];
#pragma unroll
  for (int q = 0; q < PPT; ++q) {
    const int64_t i = i0 + (int64_t)q * blockDim.x;
#pragma unroll
    for (int d = 0; d < kOdeMaxDim; ++d) x[q][d] = 0.0f;
    if (i >= s.npad) continue;
    const bool pending = s.flag[i] != 0;
    const Rand4 r0 = philox4x32_10((uint32_t)i, 0u, t, kTagStep, k0, k1);
    const Rand4 r1 = philox4x32_10((uint32_t)i, 1u, t, kTagStep, k0, k1);
    const float ra[4] = {u01(r0.a), u01(r0.c), u01(r1.a), u01(r1.c)};  // r1 draws of dims 0..3
    const float rb[4] = {u01(r0.b), u01(r0.d), u01(r1.b), u01(r1.d)};  // r2 draws
#pragma unroll
    for (int d = 0; d < kOdeMaxDim; ++d) {
      if (d < D) {
        const int64_t o = (int64_t)d * s.npad + i;
        float xd = s.X[o];
        float vd = s.V[o];
        float pd = s.P[o];
        if (pending) {
          pd = xd;
          s.P[o] = pd;
        }
        vd = velocity(xd, vd, pd, sg[d], w, c1, c2, ra[d], rb[d]);
        xd = clamp_lb_ub(__fadd_rn(xd, vd), slb[d], sub[d]);
        s.X[o] = xd;
        s.V[o] = vd;
        x[q][d] = xd;
      }
    }
  }
  float c[PPT];
  if constexpr (PPT == 2) {
    const float2 cc = ode_loss2<MODEL>(x[0], x[1], cfg, data, one);
    c[0] = cc.x;
    c[1] = cc.y;
  } else {
    c[0] = ode_eval<MODEL, METHOD>(x[0], cfg, data, tab);
  }
  unsigned long long key = ~0ull;
#pragma unroll
  for (int q = 0; q < PPT; ++q) {
    const int64_t i = i0 + (int64_t)q * blockDim.x;
    if (i >= s.npad) continue;
    const bool valid = i < s.n;
    float pc = s.pcost[i];
    const bool improved = valid && c[q] < pc;
    pc = improved ? c[q] : pc;
    s.pcost[i] = pc;
    s.cost[i] = c[q];
    s.flag[i] = improved ? 1 : 0;
    if (valid) {
      const unsigned long long k = argmin_key(pc, (uint32_t)i);
      key = k < key ? k : key;
    }
  }
  if (publish_block_min(key, st)) finish_iteration(s, from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
}

// model x integrator
#define PPS_DISPATCH_ODE(obj, method, MACRO)                              \
  do {                                                                    \
    const bool lv_ = (obj) == kLvFit;                                     \
    if ((method) == kOdeTsit5) {                                          \
      if (lv_) MACRO(kOdeLV, kOdeTsit5); else MACRO(kOdeFHN, kOdeTsit5);  \
    } else if ((method) == kOdeTsit5Adaptive) {                           \
      if (lv_) MACRO(kOdeLV, kOdeTsit5Adaptive);                          \
      else MACRO(kOdeFHN, kOdeTsit5Adaptive);                             \
    } else {                                                              \
      if (lv_) MACRO(kOdeLV, kOdeRk4); else MACRO(kOdeFHN, kOdeRk4);      \
    }                                                                     \
  } while (0)

int ode_check(const pps_problem* prob) {
  if (prob->dim < 1 || prob->dim > kOdeMaxDim)
    return set_error(PPS_EINVAL, "ODE fits have at most %d parameters (got %d)", kOdeMaxDim, prob->dim);
  if (prob->objective == kLvFit && prob->dim != 4)
    return set_error(PPS_EINVAL, "the Lotka-Volterra fit has 4 parameters (got %d)", prob->dim);
  if (prob->objective == kFhnFit && prob->dim != 3 && prob->dim != 4)
    return set_error(PPS_EINVAL, "the FitzHugh-Nagumo fit has 3 parameters, or 4 with l (got %d)", prob->dim);
  if (prob->nparams < 5 || !prob->params)
    return set_error(PPS_EINVAL, "ODE fits take params = [u0_1, u0_2, dt, nsteps, save_every(, l)]");
  if (prob->objective == kFhnFit && prob->dim == 3 && prob->nparams < 6)
    return set_error(PPS_EINVAL, "the FitzHugh-Nagumo fit of 3 parameters needs params[5] = l");
  if (!prob->data || prob->ndata < 2 || (prob->ndata & 1) || prob->ndata / 2 > kOdeMaxSaves)
    return set_error(PPS_EINVAL, "ODE fit needs data of 2 * nsaves floats, 1 <= nsaves <= %d", kOdeMaxSaves);
  const float method = prob->nparams > 6 ? prob->params[6] : 0.0f;
  if (method != (float)kOdeRk4 && method != (float)kOdeTsit5 && method != (float)kOdeTsit5Adaptive)
    return set_error(PPS_EINVAL, "ODE fit: params[6] (method) is 0 (RK4), 1 (Tsit5) or 2 (adaptive Tsit5)");
  if (method == (float)kOdeTsit5Adaptive) {
    // params = [u0_1, u0_2, dt (first step), reltol, abstol, l, 2, save_dt]
    const float dt0 = prob->params[2], rtol = prob->params[3], atol = prob->params[4];
    const float save_dt = prob->nparams > 7 ? prob->params[7] : 0.0f;
    if (!(dt0 > 0.0f) || !std::isfinite(dt0) || !(rtol > 0.0f) || !std::isfinite(rtol) || !(atol > 0.0f) ||
        !std::isfinite(atol))
      return set_error(PPS_EINVAL, "adaptive Tsit5 needs a first step dt > 0, reltol > 0 and abstol > 0 (finite)");
    if (!(save_dt > 0.0f) || !std::isfinite(save_dt) || !std::isfinite((prob->ndata / 2 - 1) * save_dt))
      return set_error(PPS_EINVAL, "ODE fit with Tsit5 needs params[7] = save_dt > 0");
    return PPS_OK;
  }
  const float nsteps = prob->params[3], every = prob->params[4];
  if (!(prob->params[2] > 0.0f) || !(nsteps >= 1.0f) || !(every >= 1.0f) || nsteps != (float)(int)nsteps ||
      every != (float)(int)every)
    return set_error(PPS_EINVAL, "ODE fit needs dt > 0 and integral nsteps, save_every >= 1");
  if (method == (float)kOdeTsit5) {
    const float save_dt = prob->nparams > 7 ? prob->params[7] : 0.0f;
    if (!(save_dt > 0.0f) || !std::isfinite(save_dt))
      return set_error(PPS_EINVAL, "ODE fit with Tsit5 needs params[7] = save_dt > 0");
    if ((double)(prob->ndata / 2 - 1) * save_dt > (double)nsteps * prob->params[2] * (1.0 + 1e-6))
      return set_error(PPS_EINVAL, "ODE fit: (nsaves - 1) * save_dt exceeds nsteps * dt");
    return PPS_OK;
  }
  if ((prob->ndata / 2 - 1) * (int64_t)every > (int64_t)nsteps)
    return set_error(PPS_EINVAL, "ODE fit: (nsaves - 1) * save_every exceeds nsteps");
  return PPS_OK;
}

static OdeCfg cfg_of(pps_swarm* s) { return ode_cfg(s->op, s->od.ndata); }

template <int MODEL, int METHOD>
__global__ void k_eval_ode(ObjParams op, OdeCfg cfg, const float* __restrict__ data_g, const float* __restrict__ x,
                           int64_t npts, int64_t stride, float* __restrict__ f);

// The fixed-step Tsit5 kernels' dynamic shared-memory limit is raised once
// per device to the largest observations + save table (init precedes every
// captured run of a swarm, so captured launches need no attribute call); the
// other methods stay within the default 48 KB (2 floats per save).
static int ode_set_smem_limit() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  PPS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(PPS_ENOTSUP, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return PPS_OK;
  const int smem = (int)(sizeof(float) * 10 * kOdeMaxSaves);
#define PPS_ODE_SMEM(M)                                                                                         \
  PPS_CUDA(cudaFuncSetAttribute(k_init_ode<M, kOdeTsit5>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));      \
  PPS_CUDA(cudaFuncSetAttribute(k_sync_step_ode<M, kOdeTsit5, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
  PPS_CUDA(cudaFuncSetAttribute(k_eval_ode<M, kOdeTsit5>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))
  PPS_ODE_SMEM(kOdeLV);
  PPS_ODE_SMEM(kOdeFHN);
#undef PPS_ODE_SMEM
  done[dev] = true;
  return PPS_OK;
}

int launch_init_ode(pps_swarm* s, int sampler, const float* u0_dev) {
  const unsigned blocks = (unsigned)((s->dv.npad + kOdeThreads - 1) / kOdeThreads);
  const OdeCfg c = cfg_of(s);
  const size_t dsm = ode_dyn_smem(c);
  if (c.method == kOdeTsit5) {
    const int rc = ode_set_smem_limit();
    if (rc) return rc;
  }
#define L_INIT_ODE(M, I) \
  k_init_ode<M, I><<<blocks, kOdeThreads, dsm, s->stream>>>(s->dv, s->op, c, s->od.data, s->seed, sampler, u0_dev)
  PPS_DISPATCH_ODE(s->objective, c.method, L_INIT_ODE);
#undef L_INIT_ODE
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_sync_step_ode(pps_swarm* s, float c1, float c2) {
  const OdeCfg c = cfg_of(s);
  const bool served = !s->owns_memory;  // state carved from a server's arena
  const int ppt = (c.method == kOdeRk4 && (s->dv.npad >= kOdePackedMinParticles || served)) ? 2 : 1;
  const int64_t tile = (int64_t)kOdeThreads * ppt;
  const unsigned blocks = (unsigned)((s->dv.npad + tile - 1) / tile);
  const int from_pos = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  const size_t dsm = ode_dyn_smem(c);
  // the last argument, 1.0f, is the packed losses' run-time one
#define L_STEP_ODE(M, I)                                                                                   \
  do {                                                                                                     \
    if (I == kOdeRk4 && ppt == 2)                                                                          \
      k_sync_step_ode<M, kOdeRk4, 2><<<blocks, kOdeThreads, dsm, s->stream>>>(s->dv, s->op, c, s->od.data, \
                                                                              s->seed, c1, c2, from_pos,  \
                                                                              1.0f);                      \
    else                                                                                                   \
      k_sync_step_ode<M, I, 1><<<blocks, kOdeThreads, dsm, s->stream>>>(s->dv, s->op, c, s->od.data,       \
                                                                        s->seed, c1, c2, from_pos, 1.0f);  \
  } while (0)
  PPS_DISPATCH_ODE(s->objective, c.method, L_STEP_ODE);
#undef L_STEP_ODE
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

template <int MODEL, int METHOD>
__global__ void k_eval_ode(ObjParams op, OdeCfg cfg, const float* __restrict__ data_g, const float* __restrict__ x,
                           int64_t npts, int64_t stride, float* __restrict__ f) {
  ode_smem_fill<METHOD>(cfg, data_g);
  const float* data = ode_smem;
  const float* tab = ode_smem + 2 * cfg.nsaves;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  float p[kOdeMaxDim] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int d = 0; d < kOdeMaxDim; ++d)
    if (d < op.dim) p[d] = x[(int64_t)d * stride + i];
  f[i] = ode_eval<MODEL, METHOD>(p, cfg, data, tab);
}

int launch_eval_ode(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                    int64_t stride, float* f, cudaStream_t stream) {
  const unsigned blocks = (unsigned)((npts + 127) / 128);
  const OdeCfg c = ode_cfg(op, od.ndata);
  const size_t dsm = ode_dyn_smem(c);
  if (c.method == kOdeTsit5) {
    const int rc = ode_set_smem_limit();
    if (rc) return rc;
  }
#define L_EVAL_ODE(M, I) k_eval_ode<M, I><<<blocks, 128, dsm, stream>>>(op, c, od.data, x, npts, stride, f)
  PPS_DISPATCH_ODE(objective, c.method, L_EVAL_ODE);
#undef L_EVAL_ODE
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

}  // namespace pps
