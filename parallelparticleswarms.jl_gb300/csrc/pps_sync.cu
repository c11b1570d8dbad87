// pps_sync.cu -- swarm initialisation and the synchronous PSO step.
//
// Reference behaviour restated here:
//   gpu_init_particles!            src/utils.jl:23-84 (uniform and unbounded samplers)
//   update_particle_state          src/kernels.jl:1-26
//   sync step + per-block argmin   src/kernels.jl:127-177, host loop src/lowerlevel_solve.jl:1-36
//   CPU-backend gbest quirk        src/lowerlevel_solve.jl:59-60 (PPS_FLAG_GBEST_FROM_POSITION)
//
// GB300 design.  One launch per iteration; each launch streams the SoA state
// once (read x, v, pbest; write x, v), evaluates the objective in registers,
// reduces the (cost, index) argmin per block with warp shuffles and publishes
// it with one 64-bit atomicMin.  The last block to finish (ticket counter)
// gathers the winner's vector into the global-best buffer and advances the
// device-resident iteration state, so no host round trip separates two
// iterations and the loop captures into a CUDA graph.  The personal-best copy
// is deferred by one iteration: a particle that improved sets a flag, and the
// next launch, which reads x anyway, writes pbest = x for flagged particles,
// so an iteration writes pbest only for particles that improved.
#include <cuda_runtime.h>

#include "pps_internal.h"

namespace pps {

constexpr int kSyncThreads = 256;

// ------------------------------------------------------------------ argmin
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long k) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, k, off);
    k = (o < k) ? o : k;
  }
  return k;
}

// Reduce `key` over the block, fold it into st->key, and return true in the
// last block to finish (all other blocks' global writes are then visible).
__device__ __forceinline__ bool publish_block_min(unsigned long long key, IterState* st) {
  __shared__ unsigned long long wmin[32];
  __shared__ int last;
  key = warp_min_u64(key);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wmin[warp] = key;
  __threadfence();  // make this thread's state writes visible device-wide
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    unsigned long long k = (lane < nw) ? wmin[lane] : ~0ull;
    k = warp_min_u64(k);
    if (lane == 0) {
      atomicMin(&st->key, k);
      __threadfence();
      const unsigned int ticket = atomicAdd(&st->count, 1u);
      last = (ticket == gridDim.x - 1) ? 1 : 0;
    }
  }
  __syncthreads();
  if (last) __threadfence();
  return last != 0;
}

// Last block: gather the winner into g, publish cost/index, reset the
// argmin slot and advance (t, w).
__device__ __forceinline__ void finish_iteration(const SwarmDev& s, bool from_position,
                                                 uint32_t t_next, float w_next) {
  IterState* st = s.st;
  const unsigned long long key = atomicAdd(&st->key, 0ull);
  const uint32_t gi = (uint32_t)key;
  const bool use_x = from_position || (__ldcg(s.flag + gi) != 0);
  const float* src = use_x ? s.X : s.P;
  for (int d = threadIdx.x; d < s.dim; d += blockDim.x) s.g[d] = __ldcg(src + (int64_t)d * s.npad + gi);
  if (threadIdx.x == 0) {
    st->gcost = __ldcg(s.pcost + gi);
    st->gidx = gi;
    st->key = ~0ull;
    st->count = 0u;
    st->t = t_next;
    st->w = w_next;
  }
}

// ------------------------------------------------------------------ init
template <int OBJ>
__global__ void __launch_bounds__(kSyncThreads) k_init(SwarmDev s, ObjParams op, uint64_t seed,
                                                        int sampler, const float* __restrict__ u0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int D = s.dim;
  unsigned long long key = ~0ull;
  if (i < s.npad) {
    const bool valid = i < s.n;
    Acc<OBJ> acc;
    for (int j = 0; j < D; j += 4) {
      const Rand4 r = philox4x32_10((uint32_t)i, (uint32_t)(j >> 2), 0u, kTagInit, k0, k1);
      const uint32_t rr[4] = {r.a, r.b, r.c, r.d};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int d = j + h;
        if (d >= D) break;
        const float u = u01(rr[h]);
        float x;
        if (sampler == PPS_SAMPLER_UNBOUNDED) {
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
        acc.add(op, d, x);
      }
    }
    const float c = valid ? finalize<OBJ>(op, acc.s1, acc.s2) : __int_as_float(0x7f800000);
    s.cost[i] = c;
    s.pcost[i] = c;
    s.flag[i] = 0;
    if (valid) key = argmin_key(c, (uint32_t)i);
  }
  if (publish_block_min(key, s.st)) finish_iteration(s, false, 0u, s.st->w);
}

// ------------------------------------------------------------------ step
// Each thread owns four consecutive particles (float4 along the particle
// axis, so a warp touches 512 contiguous bytes per array per dim) and walks
// the dims in pairs: one Philox call per particle and pair yields r1, r2 for
// both dims.  The block owns a contiguous, 32-particle-aligned range.
template <int OBJ>
__global__ void __launch_bounds__(kSyncThreads) k_sync_step(SwarmDev s, ObjParams op, uint64_t seed,
                                                             float c1, float c2, int from_position) {
  extern __shared__ float sm[];
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
  __syncthreads();
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int64_t rq = s.npad >> 2;  // row stride in float4
  const int64_t nchunk = s.npad >> 5;
  const int64_t qb = ((int64_t)blockIdx.x * nchunk / gridDim.x) * 8;
  const int64_t qe = ((int64_t)(blockIdx.x + 1) * nchunk / gridDim.x) * 8;
  float4* X4 = reinterpret_cast<float4*>(s.X);
  float4* V4 = reinterpret_cast<float4*>(s.V);
  float4* P4 = reinterpret_cast<float4*>(s.P);
  unsigned long long best = ~0ull;

  for (int64_t q = qb + threadIdx.x; q < qe; q += blockDim.x) {
    const uint32_t i0 = (uint32_t)(q * 4);
    uchar4 fl = reinterpret_cast<const uchar4*>(s.flag)[q];
    const bool anyfl = (fl.x | fl.y | fl.z | fl.w) != 0;
    Acc<OBJ> a0, a1, a2, a3;
    for (int j = 0; j < D; j += 2) {
      const uint32_t jj = (uint32_t)(j >> 1);
      const Rand4 ra = philox4x32_10(i0 + 0, jj, t, kTagStep, k0, k1);
      const Rand4 rb = philox4x32_10(i0 + 1, jj, t, kTagStep, k0, k1);
      const Rand4 rc = philox4x32_10(i0 + 2, jj, t, kTagStep, k0, k1);
      const Rand4 rd = philox4x32_10(i0 + 3, jj, t, kTagStep, k0, k1);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int d = j + h;
        if (d >= D) break;
        const int64_t o = (int64_t)d * rq + q;
        float4 x = X4[o];
        float4 v = V4[o];
        float4 p = P4[o];
        if (anyfl) {
          p.x = fl.x ? x.x : p.x;
          p.y = fl.y ? x.y : p.y;
          p.z = fl.z ? x.z : p.z;
          p.w = fl.w ? x.w : p.w;
          P4[o] = p;
        }
        const float gd = sg[d], lo = slb[d], hi = sub[d];
        v.x = velocity(x.x, v.x, p.x, gd, w, c1, c2, u01(h ? ra.c : ra.a), u01(h ? ra.d : ra.b));
        v.y = velocity(x.y, v.y, p.y, gd, w, c1, c2, u01(h ? rb.c : rb.a), u01(h ? rb.d : rb.b));
        v.z = velocity(x.z, v.z, p.z, gd, w, c1, c2, u01(h ? rc.c : rc.a), u01(h ? rc.d : rc.b));
        v.w = velocity(x.w, v.w, p.w, gd, w, c1, c2, u01(h ? rd.c : rd.a), u01(h ? rd.d : rd.b));
        x.x = clamp_lb_ub(__fadd_rn(x.x, v.x), lo, hi);
        x.y = clamp_lb_ub(__fadd_rn(x.y, v.y), lo, hi);
        x.z = clamp_lb_ub(__fadd_rn(x.z, v.z), lo, hi);
        x.w = clamp_lb_ub(__fadd_rn(x.w, v.w), lo, hi);
        X4[o] = x;
        V4[o] = v;
        a0.add(op, d, x.x);
        a1.add(op, d, x.y);
        a2.add(op, d, x.z);
        a3.add(op, d, x.w);
      }
    }
    float4 pc = reinterpret_cast<const float4*>(s.pcost)[q];
    float4 cc;
    cc.x = finalize<OBJ>(op, a0.s1, a0.s2);
    cc.y = finalize<OBJ>(op, a1.s1, a1.s2);
    cc.z = finalize<OBJ>(op, a2.s1, a2.s2);
    cc.w = finalize<OBJ>(op, a3.s1, a3.s2);
    const int64_t n = s.n;
    const bool v0 = (int64_t)i0 + 0 < n, v1 = (int64_t)i0 + 1 < n;
    const bool v2 = (int64_t)i0 + 2 < n, v3 = (int64_t)i0 + 3 < n;
    // if cost < best_cost: best = position (strict <, src/kernels.jl:21-24)
    fl.x = (v0 && cc.x < pc.x) ? 1 : 0;
    fl.y = (v1 && cc.y < pc.y) ? 1 : 0;
    fl.z = (v2 && cc.z < pc.z) ? 1 : 0;
    fl.w = (v3 && cc.w < pc.w) ? 1 : 0;
    pc.x = fl.x ? cc.x : pc.x;
    pc.y = fl.y ? cc.y : pc.y;
    pc.z = fl.z ? cc.z : pc.z;
    pc.w = fl.w ? cc.w : pc.w;
    reinterpret_cast<float4*>(s.pcost)[q] = pc;
    reinterpret_cast<float4*>(s.cost)[q] = cc;
    reinterpret_cast<uchar4*>(s.flag)[q] = fl;
    unsigned long long k;
    if (v0) { k = argmin_key(pc.x, i0 + 0); best = k < best ? k : best; }
    if (v1) { k = argmin_key(pc.y, i0 + 1); best = k < best ? k : best; }
    if (v2) { k = argmin_key(pc.z, i0 + 2); best = k < best ? k : best; }
    if (v3) { k = argmin_key(pc.w, i0 + 3); best = k < best ? k : best; }
  }
  if (publish_block_min(best, st)) {
    finish_iteration(s, from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
  }
}

// copy flagged positions into pbest (makes the state canonical: P == pbest)
__global__ void k_materialize(SwarmDev s) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.npad) return;
  if (s.flag[i] == 0) return;
  for (int d = 0; d < s.dim; ++d) {
    const int64_t o = (int64_t)d * s.npad + i;
    s.P[o] = s.X[o];
  }
  s.flag[i] = 0;
}

__global__ void k_set_iter(IterState* st, uint32_t t, float w, float wdamp) {
  st->key = ~0ull;
  st->count = 0u;
  st->t = t;
  st->w = w;
  st->wdamp = wdamp;
}

// objective at npts points, x[d*stride + i]
template <int OBJ>
__global__ void k_eval(ObjParams op, const float* __restrict__ x, int64_t npts, int64_t stride,
                       float* __restrict__ f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  Acc<OBJ> acc;
  for (int d = 0; d < op.dim; ++d) acc.add(op, d, x[(int64_t)d * stride + i]);
  f[i] = finalize<OBJ>(op, acc.s1, acc.s2);
}

// ------------------------------------------------------------------ dispatch
#define PPS_DISPATCH_SEPARABLE(obj, MACRO) \
  switch (obj) {                           \
    case kSphere: MACRO(kSphere); break;   \
    case kRosenbrock: MACRO(kRosenbrock); break; \
    case kRastrigin: MACRO(kRastrigin); break;   \
    case kAckley: MACRO(kAckley); break;   \
    case kBeale: MACRO(kBeale); break;     \
    case kBooth: MACRO(kBooth); break;     \
    case kHimmelblau: MACRO(kHimmelblau); break; \
    case kQuadratic: MACRO(kQuadratic); break;   \
    case kBoundaryQuadratic: MACRO(kBoundaryQuadratic); break; \
    default: return set_error(PPS_ENOTSUP, "objective %d has no streaming kernel", obj); \
  }

int launch_init(pps_swarm* s, int sampler, const float* u0_dev) {
  const int64_t blocks = (s->dv.npad + kSyncThreads - 1) / kSyncThreads;
#define L_INIT(O) k_init<O><<<(unsigned)blocks, kSyncThreads, 0, s->stream>>>(s->dv, s->op, s->seed, sampler, u0_dev)
  PPS_DISPATCH_SEPARABLE(s->objective, L_INIT)
#undef L_INIT
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_set_iter(pps_swarm* s, uint32_t t, float w, float wdamp) {
  k_set_iter<<<1, 1, 0, s->stream>>>(s->dv.st, t, w, wdamp);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int sync_grid(pps_swarm* s) {
  // resident blocks across the GPU, at most one per 32-particle chunk
  static thread_local int cached_obj = -1, cached_blocks = 0, cached_dev = -1;
  int per_sm = 0;
  if (cached_obj == s->objective && cached_dev == s->device) {
    per_sm = cached_blocks;
  } else {
    const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
#define L_OCC(O) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sync_step<O>, kSyncThreads, smem)
    switch (s->objective) {
      case kSphere: L_OCC(kSphere); break;
      case kRosenbrock: L_OCC(kRosenbrock); break;
      case kRastrigin: L_OCC(kRastrigin); break;
      case kAckley: L_OCC(kAckley); break;
      default: L_OCC(kBeale); break;
    }
#undef L_OCC
    if (per_sm < 1) per_sm = 1;
    cached_obj = s->objective;
    cached_blocks = per_sm;
    cached_dev = s->device;
  }
  int64_t grid = (int64_t)per_sm * s->sm_count;
  const int64_t chunks = s->dv.npad / 32;
  if (grid > chunks) grid = chunks;
  if (grid < 1) grid = 1;
  return (int)grid;
}

int launch_sync_step(pps_swarm* s, float c1, float c2) {
  const int grid = sync_grid(s);
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  const int from_pos = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
#define L_STEP(O) k_sync_step<O><<<grid, kSyncThreads, smem, s->stream>>>(s->dv, s->op, s->seed, c1, c2, from_pos)
  PPS_DISPATCH_SEPARABLE(s->objective, L_STEP)
#undef L_STEP
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_materialize(pps_swarm* s) {
  const int64_t blocks = (s->dv.npad + 255) / 256;
  k_materialize<<<(unsigned)blocks, 256, 0, s->stream>>>(s->dv);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_eval(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                int64_t stride, float* f, cudaStream_t stream) {
  (void)od;
  const int64_t blocks = (npts + 255) / 256;
#define L_EVAL(O) k_eval<O><<<(unsigned)blocks, 256, 0, stream>>>(op, x, npts, stride, f)
  PPS_DISPATCH_SEPARABLE(objective, L_EVAL)
#undef L_EVAL
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

}  // namespace pps
