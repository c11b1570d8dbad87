// pps_async.cu -- ParallelPSOKernel(global_update = false): the whole
// iteration loop inside one launch (src/kernels.jl:196-225,
// src/lowerlevel_solve.jl:95-121).
//
// Semantics.  Every particle starts from the swarm's global best and keeps a
// private copy that it replaces whenever its own personal best beats it
// (src/kernels.jl:215-218).  Once that has happened the private copy IS the
// personal best (the personal best only improves from then on and each
// improvement beats the copy again), so the private state is one flag:
// g_private = own ? pbest : g_start.  w is damped in-kernel (:219).  The run
// ends with the argmin over personal bests (src/lowerlevel_solve.jl:119-120).
//
// GB300 design.  A particle's state lives in registers for the whole run: a
// group of `lanes` threads (a power of two dividing 32) shares one particle,
// each lane holding an even-length slice of its dims (x, v, pbest), so
// D = 100 uses 8 lanes of 14 dims and 48 registers of state.  The objective
// is summed per lane in dim order and the lane sums are combined by an XOR
// butterfly, which yields the balanced pairwise tree in dim order on every
// lane (IEEE addition is commutative), so all lanes take the same
// personal-best decision.  Nothing but the start and end state touches HBM.
#include <cuda_runtime.h>

#include "pps_internal.h"
#include "pps_publish.cuh"

namespace pps {

constexpr int kAsyncThreads = 256;

__device__ __forceinline__ unsigned long long warp_min_u64_a(unsigned long long k) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, k, off);
    k = (o < k) ? o : k;
  }
  return k;
}

template <int OBJ, int S>
__global__ void __launch_bounds__(kAsyncThreads) k_async(SwarmDev s, ObjParams op, PhiloxKeys keys,
                                                          int iters, float c1, float c2, int lanes,
                                                          int slice) {
  extern __shared__ float sm[];
  const int D = s.dim;
  float* sg = sm;
  float* slb = sm + D;
  float* sub = sm + 2 * D;
  IterState* st = s.st;
  const uint32_t t0 = st->t;
  const float w0 = st->w;
  const float wdamp = st->wdamp;
  const float gcost0 = st->gcost;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    sg[d] = s.g[d];
    slb[d] = s.lb[d];
    sub[d] = s.ub[d];
  }
  __syncthreads();

  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = gtid / lanes;
  const int lane = (int)(gtid - i * lanes);
  const bool active = i < s.n;
  const int64_t il = active ? i : (s.n - 1);  // inactive threads mirror a real particle
  const uint32_t gil = (uint32_t)(s.first + il);  // its index in the whole swarm (a shard's is offset)
  const int d0 = lane * slice;
  int cnt = D - d0;
  cnt = cnt < 0 ? 0 : (cnt > slice ? slice : cnt);
  float x[S], v[S], p[S];
  const bool pending = s.flag[il] != 0;
#pragma unroll
  for (int k = 0; k < S; ++k) {
    if (k < cnt) {
      const int64_t o = (int64_t)(d0 + k) * s.npad + il;
      x[k] = s.X[o];
      v[k] = s.V[o];
      p[k] = pending ? x[k] : s.P[o];
    }
  }
  float pc = s.pcost[il];
  float cc = s.cost[il];
  bool own = false;
  float w = w0;
  const unsigned full = 0xffffffffu;

  for (int it = 0; it < iters; ++it) {
    const uint32_t t = t0 + (uint32_t)it;
#pragma unroll
    for (int k = 0; k < S; k += 2) {
      if (k < cnt) {
        const Rand4 r = philox4x32_10(gil, (uint32_t)((d0 + k) >> 1), t, kTagStep, keys);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int kk = k + h;
          if (kk < cnt) {
            const int d = d0 + kk;
            const float gd = own ? p[kk] : sg[d];
            const float r1 = u01(h ? r.c : r.a), r2 = u01(h ? r.d : r.b);
            v[kk] = velocity(x[kk], v[kk], p[kk], gd, w, c1, c2, r1, r2);
            x[kk] = clamp_lb_ub(__fadd_rn(x[kk], v[kk]), slb[d], sub[d]);
          }
        }
      }
    }
    // per-lane objective sums in dim order
    Acc<OBJ> acc;
#pragma unroll
    for (int k = 0; k < S; ++k)
      if (k < cnt) acc.add(op, k, x[k]);
    if constexpr (OBJ == kRosenbrock) {
      // the term of the lane's last dim couples to the next lane's first dim
      const float xn = __shfl_down_sync(full, x[0], 1);
      if (cnt > 0 && d0 + cnt < D) acc.add(op, 1, xn);
    }
    float s1 = acc.s1, s2 = acc.s2;
    for (int off = 1; off < lanes; off <<= 1) {
      s1 = __fadd_rn(s1, __shfl_xor_sync(full, s1, off));
      s2 = __fadd_rn(s2, __shfl_xor_sync(full, s2, off));
    }
    cc = finalize<OBJ>(op, s1, s2);
    if (cc < pc) {
      pc = cc;
#pragma unroll
      for (int k = 0; k < S; ++k)
        if (k < cnt) p[k] = x[k];
    }
    own = own || (pc < gcost0);
    w = __fmul_rn(w, wdamp);
  }

  if (active) {
#pragma unroll
    for (int k = 0; k < S; ++k) {
      if (k < cnt) {
        const int64_t o = (int64_t)(d0 + k) * s.npad + i;
        s.X[o] = x[k];
        s.V[o] = v[k];
        s.P[o] = p[k];
      }
    }
    if (lane == 0) {
      s.pcost[i] = pc;
      s.cost[i] = cc;
      s.flag[i] = 0;
    }
  }
  unsigned long long key = (active && lane == 0) ? argmin_key(pc, gil) : ~0ull;

  // block argmin + last-block publication of the final global best
  __shared__ unsigned long long wmin[32];
  __shared__ int last;
  key = warp_min_u64_a(key);
  const int wl = threadIdx.x & 31, wp = threadIdx.x >> 5;
  if (wl == 0) wmin[wp] = key;
  __threadfence();
  __syncthreads();
  if (wp == 0) {
    unsigned long long k = (wl < (int)(blockDim.x >> 5)) ? wmin[wl] : ~0ull;
    k = warp_min_u64_a(k);
    if (wl == 0) {
      atomicMin(&st->key, k);
      __threadfence();
      const unsigned int ticket = atomicAdd(&st->count, 1u);
      last = (ticket == gridDim.x - 1) ? 1 : 0;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // every flag is clear now, so the winner's vector is its personal best
  finish_iteration(s, false, t0 + (uint32_t)iters, w);
}

int async_lanes(int dim, int* slice) {
  int lanes = 1;
  if (dim > 16) {
    const int need = (dim + 15) / 16;
    while (lanes < need) lanes <<= 1;
    if (lanes > 32) lanes = 32;
  }
  int S = (dim + lanes - 1) / lanes;
  S += S & 1;
  if (slice) *slice = S;
  return lanes;
}

template <int OBJ>
static int launch_async_obj(pps_swarm* s, int iters, float c1, float c2, int lanes, int slice) {
  const int64_t threads = s->dv.npad * lanes;
  const int64_t blocks = (threads + kAsyncThreads - 1) / kAsyncThreads;
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  if (slice <= 4)
    k_async<OBJ, 4><<<(unsigned)blocks, kAsyncThreads, smem, s->stream>>>(s->dv, s->op, philox_round_keys(s->seed), iters, c1, c2, lanes, slice);
  else if (slice <= 8)
    k_async<OBJ, 8><<<(unsigned)blocks, kAsyncThreads, smem, s->stream>>>(s->dv, s->op, philox_round_keys(s->seed), iters, c1, c2, lanes, slice);
  else if (slice <= 16)
    k_async<OBJ, 16><<<(unsigned)blocks, kAsyncThreads, smem, s->stream>>>(s->dv, s->op, philox_round_keys(s->seed), iters, c1, c2, lanes, slice);
  else
    k_async<OBJ, 32><<<(unsigned)blocks, kAsyncThreads, smem, s->stream>>>(s->dv, s->op, philox_round_keys(s->seed), iters, c1, c2, lanes, slice);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_async(pps_swarm* s, int iters, float c1, float c2, int* lanes_out) {
  int slice = 0;
  const int lanes = async_lanes(s->dv.dim, &slice);
  if (slice > 32) return set_error(PPS_ENOTSUP, "async run supports dim <= 1024 (got %d)", s->dv.dim);
  if (lanes_out) *lanes_out = lanes;
  switch (s->objective) {
    case kSphere: return launch_async_obj<kSphere>(s, iters, c1, c2, lanes, slice);
    case kRosenbrock: return launch_async_obj<kRosenbrock>(s, iters, c1, c2, lanes, slice);
    case kRastrigin: return launch_async_obj<kRastrigin>(s, iters, c1, c2, lanes, slice);
    case kAckley: return launch_async_obj<kAckley>(s, iters, c1, c2, lanes, slice);
    case kBeale: return launch_async_obj<kBeale>(s, iters, c1, c2, lanes, slice);
    case kBooth: return launch_async_obj<kBooth>(s, iters, c1, c2, lanes, slice);
    case kHimmelblau: return launch_async_obj<kHimmelblau>(s, iters, c1, c2, lanes, slice);
    case kQuadratic: return launch_async_obj<kQuadratic>(s, iters, c1, c2, lanes, slice);
    case kBoundaryQuadratic: return launch_async_obj<kBoundaryQuadratic>(s, iters, c1, c2, lanes, slice);
    case kShiftedSphere: return launch_async_obj<kShiftedSphere>(s, iters, c1, c2, lanes, slice);
    default: return set_error(PPS_ENOTSUP, "objective %d has no async kernel", s->objective);
  }
}

}  // namespace pps
