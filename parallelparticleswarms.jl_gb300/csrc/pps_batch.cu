// pps_batch.cu -- many independent swarms of uneven dimension and size in one
// persistent launch.
//
// The reference solves one problem per solve() call: every iteration of
// vectorized_solve! is a kernel launch plus a host reduction
// (src/lowerlevel_solve.jl:1-36), and parameter_estim_ode! takes about five
// launches and host synchronisations per iteration (src/ode_pso.jl:113-170).
// Small problems leave the GPU idle.  Here one CTA owns one swarm for its
// whole life -- sampling, every synchronous iteration, the global best -- with
// the argmin a block reduction (no atomics, no host round trip), so a batch of
// thousands of swarms is one launch that keeps every SM busy.
//
// Semantics per swarm are exactly pps_sync_run's (same Philox counters, same
// operation order, global best from the personal best), so a swarm's result
// does not depend on the batch it rides in: bit-identical alone and in a mix.
//
// Scheduling: CTAs are issued longest-estimated-work first (LPT), so the long
// swarms start early and the short ones fill the tail.  The block size and
// particles per thread come from an autotuner that times the candidates on
// the batch itself (a few iterations each) and caches the winner per batch
// shape.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "pps_internal.h"
#include "pps_ode.cuh"
#include "pps_objgrad.cuh"

namespace pps {

constexpr int kBatchMaxDim = 1024;
constexpr int64_t kBatchMaxParticles = 1 << 16;

struct BatchSwarm {
  int objective, dim, maxiters, sampler;
  int64_t n, ld;
  float w, wdamp, c1, c2;
  uint64_t seed;
  ObjParams op;
  int64_t ndata;
  const float* data;
  float *X, *V, *P, *pcost, *cost;
  const float *lb, *ub, *u0;
  float* g;       // dim floats: global best position (out)
  float* result;  // [gcost, gidx as bits, iterations]
};

__device__ __forceinline__ unsigned long long wmin64(unsigned long long k) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, k, off);
    k = o < k ? o : k;
  }
  return k;
}

// block-wide argmin; every thread returns the winning key
__device__ __forceinline__ unsigned long long block_min(unsigned long long key, unsigned long long* red) {
  key = wmin64(key);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // red may still be read from the previous call
  if (lane == 0) red[warp] = key;
  __syncthreads();
  if (warp == 0) {
    unsigned long long k = (lane < (int)(blockDim.x >> 5)) ? red[lane] : ~0ull;
    k = wmin64(k);
    if (lane == 0) red[32] = k;
  }
  __syncthreads();
  return red[32];
}

struct BatchSmem {
  unsigned long long red[33];
  float gcost;
};

// ---------------------------------------------------------------- separable
template <int OBJ, int PPT>
__device__ void run_swarm(const BatchSwarm& sw, BatchSmem& S, float* sg, float* slb, float* sub, uint8_t* flag) {
  const int D = sw.dim;
  const int64_t n = sw.n, ld = sw.ld;
  const uint32_t k0 = (uint32_t)sw.seed, k1 = (uint32_t)(sw.seed >> 32);
  float* __restrict__ X = sw.X;
  float* __restrict__ V = sw.V;
  float* __restrict__ P = sw.P;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    slb[d] = sw.lb[d];
    sub[d] = sw.ub[d];
  }
  for (int64_t i = threadIdx.x; i < ld; i += blockDim.x) flag[i] = 0;  // padding particles included
  __syncthreads();
  // ---- init (gpu_init_particles!, src/utils.jl:23-84)
  unsigned long long best = ~0ull;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    Acc<OBJ> acc;
    for (int j = 0; j < D; j += 4) {
      const Rand4 r = philox4x32_10((uint32_t)i, (uint32_t)(j >> 2), 0u, kTagInit, k0, k1);
      const uint32_t rr[4] = {r.a, r.b, r.c, r.d};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int d = j + h;
        if (d < D) {
          const float u = u01(rr[h]);
          float x;
          if (sw.sampler == PPS_SAMPLER_UNBOUNDED) {
            const float z = sw.u0 ? sw.u0[d] : 0.0f;
            const float a = fabsf(z);
            x = (a > 0.0f) ? __fadd_rn(z, __fmul_rn(u, a)) : u;
          } else {
            x = __fadd_rn(__fmul_rn(u, __fsub_rn(sub[d], slb[d])), slb[d]);
          }
          const int64_t o = (int64_t)d * ld + i;
          X[o] = x;
          V[o] = 0.0f;
          P[o] = x;
          acc.add(sw.op, d, x);
        }
      }
    }
    const float c = finalize<OBJ>(sw.op, acc.s1, acc.s2);
    sw.cost[i] = c;
    sw.pcost[i] = c;
    flag[i] = 0;
    const unsigned long long k = argmin_key(c, (uint32_t)i);
    best = k < best ? k : best;
  }
  unsigned long long win = block_min(best, S.red);
  {
    const uint32_t gi = (uint32_t)win;
    for (int d = threadIdx.x; d < D; d += blockDim.x) sg[d] = P[(int64_t)d * ld + gi];
    if (threadIdx.x == 0) S.gcost = sw.pcost[gi];
  }
  __syncthreads();
  float w = sw.w;
  // ---- synchronous iterations (src/kernels.jl:1-26, src/lowerlevel_solve.jl:1-36)
  for (int it = 0; it < sw.maxiters; ++it) {
    const uint32_t t = (uint32_t)it;
    best = ~0ull;
    for (int64_t i0 = (int64_t)threadIdx.x * PPT; i0 < n; i0 += (int64_t)blockDim.x * PPT) {
      uint8_t fl[PPT];
      bool anyfl = false;
#pragma unroll
      for (int k = 0; k < PPT; ++k) {
        fl[k] = flag[i0 + k];
        anyfl |= fl[k] != 0;
      }
      Acc<OBJ> acc[PPT];
      for (int j = 0; j < D; j += 2) {
        Rand4 r[PPT];
#pragma unroll
        for (int k = 0; k < PPT; ++k) r[k] = philox4x32_10((uint32_t)(i0 + k), (uint32_t)(j >> 1), t, kTagStep, k0, k1);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int d = j + h;
          if (d < D) {
            const int64_t o = (int64_t)d * ld + i0;
            float x[PPT], v[PPT], p[PPT];
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
              x[k] = X[o + k];
              v[k] = V[o + k];
              p[k] = P[o + k];
            }
            if (anyfl) {
#pragma unroll
              for (int k = 0; k < PPT; ++k) {
                p[k] = fl[k] ? x[k] : p[k];
                if (fl[k]) P[o + k] = p[k];
              }
            }
            const float gd = sg[d], lo = slb[d], hi = sub[d];
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
              const float r1 = u01(h ? r[k].c : r[k].a), r2 = u01(h ? r[k].d : r[k].b);
              v[k] = velocity(x[k], v[k], p[k], gd, w, sw.c1, sw.c2, r1, r2);
              x[k] = clamp_lb_ub(__fadd_rn(x[k], v[k]), lo, hi);
              X[o + k] = x[k];
              V[o + k] = v[k];
              acc[k].add(sw.op, d, x[k]);
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < PPT; ++k) {
        const int64_t i = i0 + k;
        const bool valid = i < n;
        const float c = finalize<OBJ>(sw.op, acc[k].s1, acc[k].s2);
        const float pc = sw.pcost[i];
        const bool imp = valid && c < pc;
        const float npc = imp ? c : pc;
        if (valid) {
          sw.pcost[i] = npc;
          sw.cost[i] = c;
          const unsigned long long key = argmin_key(npc, (uint32_t)i);
          best = key < best ? key : best;
        }
        flag[i] = imp ? 1 : 0;
      }
    }
    win = block_min(best, S.red);  // also orders this iteration's writes before the gather
    const uint32_t gi = (uint32_t)win;
    const bool from_x = flag[gi] != 0;
    for (int d = threadIdx.x; d < D; d += blockDim.x) sg[d] = from_x ? X[(int64_t)d * ld + gi] : P[(int64_t)d * ld + gi];
    if (threadIdx.x == 0) S.gcost = sw.pcost[gi];
    __syncthreads();
    w = __fmul_rn(w, sw.wdamp);
  }
  // ---- canonical state and result
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    if (flag[i]) {
      for (int d = 0; d < D; ++d) P[(int64_t)d * ld + i] = X[(int64_t)d * ld + i];
    }
  }
  for (int d = threadIdx.x; d < D; d += blockDim.x) sw.g[d] = sg[d];
  if (threadIdx.x == 0) {
    sw.result[0] = S.gcost;
    sw.result[1] = __uint_as_float((uint32_t)win);
    sw.result[2] = (float)sw.maxiters;
  }
}

// ---------------------------------------------------------------- ODE fits
template <int MODEL>
__device__ void run_swarm_ode(const BatchSwarm& sw, BatchSmem& S, float* sg, float* slb, float* sub, uint8_t* flag,
                              float* data) {
  const int D = sw.dim;
  const int64_t n = sw.n, ld = sw.ld;
  const uint32_t k0 = (uint32_t)sw.seed, k1 = (uint32_t)(sw.seed >> 32);
  const OdeCfg cfg = ode_cfg(sw.op, sw.ndata);
  for (int k = threadIdx.x; k < 2 * cfg.nsaves; k += blockDim.x) data[k] = sw.data[k];
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    slb[d] = sw.lb[d];
    sub[d] = sw.ub[d];
  }
  __syncthreads();
  unsigned long long best = ~0ull;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    float x[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const Rand4 r = philox4x32_10((uint32_t)i, 0u, 0u, kTagInit, k0, k1);
    const uint32_t rr[4] = {r.a, r.b, r.c, r.d};
#pragma unroll
    for (int d = 0; d < 4; ++d) {
      if (d < D) {
        const float u = u01(rr[d]);
        float xv;
        if (sw.sampler == PPS_SAMPLER_UNBOUNDED) {
          const float z = sw.u0 ? sw.u0[d] : 0.0f;
          const float a = fabsf(z);
          xv = (a > 0.0f) ? __fadd_rn(z, __fmul_rn(u, a)) : u;
        } else {
          xv = __fadd_rn(__fmul_rn(u, __fsub_rn(sub[d], slb[d])), slb[d]);
        }
        x[d] = xv;
        const int64_t o = (int64_t)d * ld + i;
        sw.X[o] = xv;
        sw.V[o] = 0.0f;
        sw.P[o] = xv;
      }
    }
    const float c = ode_loss<MODEL>(x, cfg, data);
    sw.cost[i] = c;
    sw.pcost[i] = c;
    flag[i] = 0;
    const unsigned long long k = argmin_key(c, (uint32_t)i);
    best = k < best ? k : best;
  }
  unsigned long long win = block_min(best, S.red);
  {
    const uint32_t gi = (uint32_t)win;
    for (int d = threadIdx.x; d < D; d += blockDim.x) sg[d] = sw.P[(int64_t)d * ld + gi];
    if (threadIdx.x == 0) S.gcost = sw.pcost[gi];
  }
  __syncthreads();
  float w = sw.w;
  for (int it = 0; it < sw.maxiters; ++it) {
    const uint32_t t = (uint32_t)it;
    best = ~0ull;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const bool pending = flag[i] != 0;
      float x[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      const Rand4 r0 = philox4x32_10((uint32_t)i, 0u, t, kTagStep, k0, k1);
      const Rand4 r1 = philox4x32_10((uint32_t)i, 1u, t, kTagStep, k0, k1);
      const float ra[4] = {u01(r0.a), u01(r0.c), u01(r1.a), u01(r1.c)};
      const float rb[4] = {u01(r0.b), u01(r0.d), u01(r1.b), u01(r1.d)};
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        if (d < D) {
          const int64_t o = (int64_t)d * ld + i;
          float xd = sw.X[o], vd = sw.V[o], pd = sw.P[o];
          if (pending) {
            pd = xd;
            sw.P[o] = pd;
          }
          vd = velocity(xd, vd, pd, sg[d], w, sw.c1, sw.c2, ra[d], rb[d]);
          xd = clamp_lb_ub(__fadd_rn(xd, vd), slb[d], sub[d]);
          sw.X[o] = xd;
          sw.V[o] = vd;
          x[d] = xd;
        }
      }
      const float c = ode_loss<MODEL>(x, cfg, data);
      const float pc = sw.pcost[i];
      const bool imp = c < pc;
      const float npc = imp ? c : pc;
      sw.pcost[i] = npc;
      sw.cost[i] = c;
      flag[i] = imp ? 1 : 0;
      const unsigned long long key = argmin_key(npc, (uint32_t)i);
      best = key < best ? key : best;
    }
    win = block_min(best, S.red);
    const uint32_t gi = (uint32_t)win;
    const bool from_x = flag[gi] != 0;
    for (int d = threadIdx.x; d < D; d += blockDim.x) sg[d] = from_x ? sw.X[(int64_t)d * ld + gi] : sw.P[(int64_t)d * ld + gi];
    if (threadIdx.x == 0) S.gcost = sw.pcost[gi];
    __syncthreads();
    w = __fmul_rn(w, sw.wdamp);
  }
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    if (flag[i]) {
      for (int d = 0; d < D; ++d) sw.P[(int64_t)d * ld + i] = sw.X[(int64_t)d * ld + i];
    }
  }
  for (int d = threadIdx.x; d < D; d += blockDim.x) sw.g[d] = sg[d];
  if (threadIdx.x == 0) {
    sw.result[0] = S.gcost;
    sw.result[1] = __uint_as_float((uint32_t)win);
    sw.result[2] = (float)sw.maxiters;
  }
}

// dynamic shared memory: g, lb, ub (3 * maxdim floats), ODE data
// (2 * maxsaves floats), flags (max n bytes)
template <int PPT>
__global__ void k_batch(const BatchSwarm* __restrict__ descs, const int* __restrict__ order, int maxdim,
                        int data_floats) {
  extern __shared__ float dsm[];
  __shared__ BatchSmem S;
  const BatchSwarm sw = descs[order[blockIdx.x]];
  float* sg = dsm;
  float* slb = dsm + maxdim;
  float* sub = dsm + 2 * maxdim;
  float* data = dsm + 3 * maxdim;
  uint8_t* flag = reinterpret_cast<uint8_t*>(data + data_floats);
  switch (sw.objective) {
    case kSphere: run_swarm<kSphere, PPT>(sw, S, sg, slb, sub, flag); break;
    case kRosenbrock: run_swarm<kRosenbrock, PPT>(sw, S, sg, slb, sub, flag); break;
    case kRastrigin: run_swarm<kRastrigin, PPT>(sw, S, sg, slb, sub, flag); break;
    case kAckley: run_swarm<kAckley, PPT>(sw, S, sg, slb, sub, flag); break;
    case kLvFit: run_swarm_ode<kOdeLV>(sw, S, sg, slb, sub, flag, data); break;
    case kFhnFit: run_swarm_ode<kOdeFHN>(sw, S, sg, slb, sub, flag, data); break;
    default: break;
  }
}

}  // namespace pps

// ---------------------------------------------------------------------------
// host side: the batch object, arena, autotuner
// ---------------------------------------------------------------------------
using namespace pps;

struct pps_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int sm_count = 0;
  std::vector<BatchSwarm> descs;        // device pointers filled at run time
  std::vector<std::vector<float>> host;  // per swarm: lb | ub | u0 | data
  std::vector<size_t> offsets;           // per swarm: arena offset (bytes)
  size_t arena_bytes = 0;
  void* arena = nullptr;
  size_t arena_cap = 0;
  BatchSwarm* ddescs = nullptr;
  int* dorder = nullptr;
  size_t dcap = 0;
  int tuned_threads = 0, tuned_ppt = 0;
  int last_threads = 0, last_ppt = 0;
  bool ran = false;
};

namespace {

std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune_cache;

size_t a256(size_t v) { return (v + 255) / 256 * 256; }

size_t swarm_bytes(int D, int64_t ld, int64_t ndata) {
  // X, V, P, pcost, cost, lb, ub, u0, g, result, data
  return a256(sizeof(float) * (size_t)D * ld) * 3 + a256(sizeof(float) * ld) * 2 + a256(sizeof(float) * D) * 4 +
         256 + a256(sizeof(float) * (size_t)ndata);
}

double work_estimate(const BatchSwarm& d) {
  double per = is_ode(d.objective) ? (double)ode_cfg(d.op, d.ndata).nsteps * 12.0 : (double)d.dim;
  return (double)d.n * (double)(d.maxiters + 1) * per;
}

}  // namespace

extern "C" {

int pps_batch_create(pps_batch** out) {
  if (!out) return set_error(PPS_EINVAL, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_error(PPS_ENODEV, "no CUDA device");
  pps_batch* b = new (std::nothrow) pps_batch();
  if (!b) return set_error(PPS_ENOMEM, "host allocation failed");
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess) {
    pps_batch_destroy(b);
    return cuda_error(e, "stream/event creation");
  }
  *out = b;
  return PPS_OK;
}

int pps_batch_destroy(pps_batch* b) {
  if (!b) return PPS_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->arena) cudaFree(b->arena);
  if (b->ddescs) cudaFree(b->ddescs);
  if (b->dorder) cudaFree(b->dorder);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PPS_OK;
}

int pps_batch_add(pps_batch* b, const pps_problem* prob, int64_t n, uint64_t seed, int32_t maxiters, float w,
                  float wdamp, float c1, float c2, int32_t* slot) {
  if (!b || !prob) return set_error(PPS_EINVAL, "NULL argument");
  const int obj = prob->objective;
  if (!(obj == kSphere || obj == kRosenbrock || obj == kRastrigin || obj == kAckley || is_ode(obj)))
    return set_error(PPS_ENOTSUP, "objective %d is not supported in batches", obj);
  if (prob->dim < 1 || prob->dim > kBatchMaxDim)
    return set_error(PPS_EINVAL, "batched swarms have 1 <= dim <= %d (got %d)", kBatchMaxDim, prob->dim);
  if (n < 1 || n > kBatchMaxParticles)
    return set_error(PPS_EINVAL, "batched swarms have 1 <= n <= %lld (got %lld)", (long long)kBatchMaxParticles,
                     (long long)n);
  if (maxiters < 0) return set_error(PPS_EINVAL, "maxiters must be >= 0");
  if (prob->nparams < 0 || prob->nparams > 8 || (prob->nparams > 0 && !prob->params))
    return set_error(PPS_EINVAL, "nparams must be in [0, 8]");
  if (!std::isfinite(w) || !std::isfinite(wdamp) || !std::isfinite(c1) || !std::isfinite(c2))
    return set_error(PPS_EINVAL, "coefficients must be finite");
  if (is_ode(obj)) {
    const int rc = ode_check(prob);
    if (rc) return rc;
  }
  const int D = prob->dim;
  bool all_inf = true;
  for (int d = 0; d < D; ++d) {
    const float lo = prob->lb ? prob->lb[d] : -INFINITY, hi = prob->ub ? prob->ub[d] : INFINITY;
    if (std::isnan(lo) || std::isnan(hi) || lo > hi) return set_error(PPS_EINVAL, "bounds of dim %d are invalid", d);
    if (!(std::isinf(lo) && std::isinf(hi))) all_inf = false;
  }
  int sampler = PPS_SAMPLER_UNIFORM;
  if (all_inf) {
    sampler = PPS_SAMPLER_UNBOUNDED;
  } else {
    for (int d = 0; d < D; ++d) {
      const float lo = prob->lb ? prob->lb[d] : -INFINITY, hi = prob->ub ? prob->ub[d] : INFINITY;
      if (!std::isfinite(lo) || !std::isfinite(hi))
        return set_error(PPS_EINVAL, "uniform sampling needs finite bounds (dim %d)", d);
    }
  }
  BatchSwarm d{};
  d.objective = obj;
  d.dim = D;
  d.maxiters = maxiters;
  d.sampler = sampler;
  d.n = n;
  d.ld = (n + 31) / 32 * 32;
  d.w = w;
  d.wdamp = wdamp;
  d.c1 = c1;
  d.c2 = c2;
  d.seed = seed;
  for (int k = 0; k < prob->nparams; ++k) d.op.p[k] = prob->params[k];
  d.op.np = prob->nparams;
  d.op.dim = D;
  d.ndata = is_ode(obj) ? prob->ndata : 0;
  std::vector<float> h;
  h.reserve((size_t)3 * D + (size_t)d.ndata);
  for (int k = 0; k < D; ++k) h.push_back(prob->lb ? prob->lb[k] : -INFINITY);
  for (int k = 0; k < D; ++k) h.push_back(prob->ub ? prob->ub[k] : INFINITY);
  for (int k = 0; k < D; ++k) h.push_back(prob->u0 ? prob->u0[k] : 0.0f);
  for (int64_t k = 0; k < d.ndata; ++k) h.push_back(prob->data[k]);
  b->offsets.push_back(b->arena_bytes);
  b->arena_bytes += swarm_bytes(D, d.ld, d.ndata);
  b->descs.push_back(d);
  b->host.push_back(std::move(h));
  b->ran = false;
  if (slot) *slot = (int32_t)(b->descs.size() - 1);
  return PPS_OK;
}

}  // extern "C"

namespace {

int prepare(pps_batch* b, std::vector<int>& order, int& maxdim, int& data_floats, int64_t& maxn) {
  const size_t ns = b->descs.size();
  if (b->arena_cap < b->arena_bytes) {
    if (b->arena) cudaFree(b->arena);
    b->arena = nullptr;
    b->arena_cap = 0;
    PPS_CUDA(cudaMalloc(&b->arena, b->arena_bytes));
    b->arena_cap = b->arena_bytes;
  }
  if (b->dcap < ns) {
    if (b->ddescs) cudaFree(b->ddescs);
    if (b->dorder) cudaFree(b->dorder);
    b->ddescs = nullptr;
    b->dorder = nullptr;
    b->dcap = 0;
    PPS_CUDA(cudaMalloc(&b->ddescs, sizeof(BatchSwarm) * ns));
    PPS_CUDA(cudaMalloc(&b->dorder, sizeof(int) * ns));
    b->dcap = ns;
  }
  maxdim = 1;
  data_floats = 0;
  maxn = 1;
  char* base = static_cast<char*>(b->arena);
  for (size_t k = 0; k < ns; ++k) {
    BatchSwarm& d = b->descs[k];
    const int D = d.dim;
    size_t off = b->offsets[k];
    auto take = [&](size_t bytes) {
      char* p = base + off;
      off += a256(bytes);
      return p;
    };
    d.X = reinterpret_cast<float*>(take(sizeof(float) * (size_t)D * d.ld));
    d.V = reinterpret_cast<float*>(take(sizeof(float) * (size_t)D * d.ld));
    d.P = reinterpret_cast<float*>(take(sizeof(float) * (size_t)D * d.ld));
    d.pcost = reinterpret_cast<float*>(take(sizeof(float) * d.ld));
    d.cost = reinterpret_cast<float*>(take(sizeof(float) * d.ld));
    float* lbub = reinterpret_cast<float*>(take(sizeof(float) * D));
    float* ubp = reinterpret_cast<float*>(take(sizeof(float) * D));
    float* u0p = reinterpret_cast<float*>(take(sizeof(float) * D));
    d.g = reinterpret_cast<float*>(take(sizeof(float) * D));
    d.result = reinterpret_cast<float*>(take(256));
    float* datap = reinterpret_cast<float*>(take(sizeof(float) * (size_t)d.ndata));
    d.lb = lbub;
    d.ub = ubp;
    d.u0 = u0p;
    d.data = d.ndata ? datap : nullptr;
    const std::vector<float>& h = b->host[k];
    PPS_CUDA(cudaMemcpyAsync(lbub, h.data(), sizeof(float) * D, cudaMemcpyHostToDevice, b->stream));
    PPS_CUDA(cudaMemcpyAsync(ubp, h.data() + D, sizeof(float) * D, cudaMemcpyHostToDevice, b->stream));
    PPS_CUDA(cudaMemcpyAsync(u0p, h.data() + 2 * D, sizeof(float) * D, cudaMemcpyHostToDevice, b->stream));
    if (d.ndata)
      PPS_CUDA(cudaMemcpyAsync(datap, h.data() + 3 * D, sizeof(float) * (size_t)d.ndata, cudaMemcpyHostToDevice,
                               b->stream));
    maxdim = std::max(maxdim, D);
    data_floats = std::max(data_floats, (int)d.ndata);
    maxn = std::max(maxn, d.ld);
  }
  // longest estimated work first
  order.resize(ns);
  for (size_t k = 0; k < ns; ++k) order[k] = (int)k;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return work_estimate(b->descs[a]) > work_estimate(b->descs[c]); });
  PPS_CUDA(cudaMemcpyAsync(b->ddescs, b->descs.data(), sizeof(BatchSwarm) * ns, cudaMemcpyHostToDevice, b->stream));
  PPS_CUDA(cudaMemcpyAsync(b->dorder, order.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, b->stream));
  return PPS_OK;
}

size_t smem_bytes(int maxdim, int data_floats, int64_t maxn) {
  return sizeof(float) * (3 * (size_t)maxdim + (size_t)data_floats) + (size_t)maxn + 16;
}

int launch_batch(pps_batch* b, int threads, int ppt, int ns, int maxdim, int data_floats, int64_t maxn) {
  const size_t smem = smem_bytes(maxdim, data_floats, maxn);
  cudaError_t e;
  if (ppt == 2) {
    e = cudaFuncSetAttribute(k_batch<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute");
    k_batch<2><<<ns, threads, smem, b->stream>>>(b->ddescs, b->dorder, maxdim, data_floats);
  } else {
    e = cudaFuncSetAttribute(k_batch<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute");
    k_batch<1><<<ns, threads, smem, b->stream>>>(b->ddescs, b->dorder, maxdim, data_floats);
  }
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

std::string shape_key(const pps_batch* b) {
  // objective mix and coarse size buckets
  int cnt[8] = {0};
  double dims = 0, parts = 0, iters = 0;
  for (const auto& d : b->descs) {
    cnt[std::min(d.objective, 7)]++;
    dims += d.dim;
    parts += (double)d.n;
    iters += d.maxiters;
  }
  const double ns = (double)std::max<size_t>(1, b->descs.size());
  char buf[256];
  snprintf(buf, sizeof(buf), "%d,%d,%d,%d,%d,%d|%d|%d|%d|%zu", cnt[0] > 0, cnt[1] > 0, cnt[2] > 0, cnt[3] > 0,
           cnt[4] > 0, cnt[5] > 0, (int)std::log2(1 + dims / ns), (int)std::log2(1 + parts / ns),
           (int)std::log2(1 + iters / ns), (size_t)std::log2(1.0 + ns));
  return buf;
}

}  // namespace

extern "C" {

int pps_batch_run(pps_batch* b, float* device_ms) {
  if (!b) return set_error(PPS_EINVAL, "batch is NULL");
  if (b->descs.empty()) return set_error(PPS_EINVAL, "batch is empty");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) PPS_CUDA(cudaSetDevice(b->device));
  std::vector<int> order;
  int maxdim = 1, data_floats = 0;
  int64_t maxn = 1;
  int rc = prepare(b, order, maxdim, data_floats, maxn);
  if (rc) return rc;
  const int ns = (int)b->descs.size();
  if (smem_bytes(maxdim, data_floats, maxn) > 200 * 1024)
    return set_error(PPS_ENOTSUP, "batch needs more shared memory than a CTA has (dim, data or n too large)");
  // autotune the block shape for this batch shape (cached)
  int threads = b->tuned_threads, ppt = b->tuned_ppt;
  if (!threads) {
    const std::string key = shape_key(b);
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        threads = it->second.first;
        ppt = it->second.second;
      }
    }
    if (!threads) {
      // time each candidate on this batch with a few iterations per swarm
      std::vector<BatchSwarm> saved = b->descs;
      for (auto& d : b->descs) d.maxiters = std::min(d.maxiters, 4);
      PPS_CUDA(cudaMemcpyAsync(b->ddescs, b->descs.data(), sizeof(BatchSwarm) * ns, cudaMemcpyHostToDevice, b->stream));
      const int cand_t[3] = {128, 256, 512};
      const int cand_p[2] = {1, 2};
      float best_ms = 1e30f;
      for (int ct : cand_t) {
        for (int cp : cand_p) {
          if (cp == 2 && data_floats > 0 && maxdim <= 4) continue;  // ODE swarms ignore PPT
          PPS_CUDA(cudaEventRecord(b->ev0, b->stream));
          if ((rc = launch_batch(b, ct, cp, ns, maxdim, data_floats, maxn))) return rc;
          PPS_CUDA(cudaEventRecord(b->ev1, b->stream));
          PPS_CUDA(cudaEventSynchronize(b->ev1));
          float ms = 0.0f;
          PPS_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
          if (ms < best_ms) {
            best_ms = ms;
            threads = ct;
            ppt = cp;
          }
        }
      }
      b->descs = saved;
      PPS_CUDA(cudaMemcpyAsync(b->ddescs, b->descs.data(), sizeof(BatchSwarm) * ns, cudaMemcpyHostToDevice, b->stream));
      std::lock_guard<std::mutex> lock(g_tune_mu);
      g_tune_cache[key] = {threads, ppt};
    }
  }
  PPS_CUDA(cudaEventRecord(b->ev0, b->stream));
  if ((rc = launch_batch(b, threads, ppt, ns, maxdim, data_floats, maxn))) return rc;
  PPS_CUDA(cudaEventRecord(b->ev1, b->stream));
  PPS_CUDA(cudaEventSynchronize(b->ev1));
  if (device_ms) PPS_CUDA(cudaEventElapsedTime(device_ms, b->ev0, b->ev1));
  b->last_threads = threads;
  b->last_ppt = ppt;
  b->ran = true;
  return PPS_OK;
}

int pps_batch_set_shape(pps_batch* b, int32_t threads, int32_t ppt) {
  if (!b) return set_error(PPS_EINVAL, "batch is NULL");
  if (threads == 0 && ppt == 0) {
    b->tuned_threads = b->tuned_ppt = 0;
    return PPS_OK;
  }
  if (!(threads == 128 || threads == 256 || threads == 512) || !(ppt == 1 || ppt == 2))
    return set_error(PPS_EINVAL, "block shape must be threads in {128, 256, 512} and ppt in {1, 2}");
  b->tuned_threads = threads;
  b->tuned_ppt = ppt;
  return PPS_OK;
}

int pps_batch_info(pps_batch* b, int32_t* nswarms, int32_t* threads, int32_t* ppt, uint64_t* device_bytes) {
  if (!b) return set_error(PPS_EINVAL, "batch is NULL");
  if (nswarms) *nswarms = (int32_t)b->descs.size();
  if (threads) *threads = b->last_threads;
  if (ppt) *ppt = b->last_ppt;
  if (device_bytes) *device_bytes = b->arena_bytes;
  return PPS_OK;
}

int pps_batch_result(pps_batch* b, int32_t slot, float* u, float* cost, int64_t* idx) {
  if (!b) return set_error(PPS_EINVAL, "batch is NULL");
  if (slot < 0 || slot >= (int32_t)b->descs.size()) return set_error(PPS_EINVAL, "slot %d out of range", slot);
  if (!b->ran) return set_error(PPS_EINVAL, "batch has not run");
  const BatchSwarm& d = b->descs[slot];
  float res[3];
  PPS_CUDA(cudaMemcpyAsync(res, d.result, sizeof(res), cudaMemcpyDeviceToHost, b->stream));
  if (u) PPS_CUDA(cudaMemcpyAsync(u, d.g, sizeof(float) * d.dim, cudaMemcpyDeviceToHost, b->stream));
  PPS_CUDA(cudaStreamSynchronize(b->stream));
  if (cost) *cost = res[0];
  if (idx) {
    uint32_t bits;
    memcpy(&bits, &res[1], 4);
    *idx = (int64_t)bits;
  }
  return PPS_OK;
}

int pps_batch_get_state(pps_batch* b, int32_t slot, int32_t field, float* out) {
  if (!b || !out) return set_error(PPS_EINVAL, "NULL argument");
  if (slot < 0 || slot >= (int32_t)b->descs.size()) return set_error(PPS_EINVAL, "slot %d out of range", slot);
  if (!b->ran) return set_error(PPS_EINVAL, "batch has not run");
  const BatchSwarm& d = b->descs[slot];
  float* dev;
  int rows;
  switch (field) {
    case PPS_FIELD_POSITION: dev = d.X; rows = d.dim; break;
    case PPS_FIELD_VELOCITY: dev = d.V; rows = d.dim; break;
    case PPS_FIELD_PBEST: dev = d.P; rows = d.dim; break;
    case PPS_FIELD_PCOST: dev = d.pcost; rows = 1; break;
    case PPS_FIELD_COST: dev = d.cost; rows = 1; break;
    default: return set_error(PPS_EINVAL, "unknown field %d", field);
  }
  const size_t wb = sizeof(float) * (size_t)d.n;
  PPS_CUDA(cudaMemcpy2DAsync(out, wb, dev, sizeof(float) * (size_t)d.ld, wb, rows, cudaMemcpyDeviceToHost, b->stream));
  PPS_CUDA(cudaStreamSynchronize(b->stream));
  return PPS_OK;
}

}  // extern "C"
