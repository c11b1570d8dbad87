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
#include <cstdlib>

#include <cuda_runtime.h>

#include "pps_internal.h"
#include "pps_publish.cuh"
#include "pps_vec.cuh"

namespace pps {

constexpr int kSyncThreads = 256;

// ------------------------------------------------------------------ init
// CONS: the penalty of the constrained path is added to the cost
// (src/utils.jl:72-74: calc_penalty with iter = 1 at init)
template <int OBJ, bool CONS = false>
__global__ void __launch_bounds__(kSyncThreads) k_init(SwarmDev s, ObjParams op, uint64_t seed,
                                                        int sampler, const float* __restrict__ u0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int D = s.dim;
  unsigned long long key = ~0ull;
  if (i < s.npad) {
    const bool valid = i < s.n;
    const uint32_t gi = (uint32_t)(s.first + i);  // the particle's index in the whole swarm
    Acc<OBJ> acc;
    ConsAcc ca;
    if constexpr (CONS) ca.start(s.cons, s.ncons, D);
    for (int j = 0; j < D; j += 4) {
      const Rand4 r = philox4x32_10(gi, (uint32_t)(j >> 2), 0u, kTagInit, k0, k1);
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
        } else if (sampler == PPS_SAMPLER_LHS) {
          x = valid ? lhs_position(gi, (uint32_t)s.nglobal, (uint32_t)d, u, s.lb[d], s.ub[d], k0, k1) : 0.0f;
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
        if constexpr (CONS) ca.add(s.cons, s.ncons, D, d, x);
      }
    }
    if constexpr (OBJ != kMlp) {
      float c = valid ? finalize<OBJ>(op, acc.s1, acc.s2) : __int_as_float(0x7f800000);
      if constexpr (CONS) {
        if (valid) c = __fadd_rn(c, penalty(ca, s.ncons, 1.0f));
      }
      s.cost[i] = c;
      s.pcost[i] = c;
      s.flag[i] = 0;
      if (valid) key = argmin_key(c, gi);
    }
  }
  // the MLP objective is evaluated (and published) by the tensor-core kernel
  if constexpr (OBJ != kMlp) {
    if (publish_block_min(key, s.st)) finish_iteration(s, false, 0u, s.st->w);
  }
}

// ------------------------------------------------------------------ step
// Each thread owns PPT consecutive particles (a float/float2/float4 along the
// particle axis, so a warp reads 128*PPT contiguous bytes per array per dim)
// and walks the dims in pairs: one Philox call per particle and pair yields
// r1, r2 for both dims.  The loads of the next pair are issued before the
// current pair is computed (software prefetch), so every warp keeps six
// vector loads in flight while it runs Philox and the objective.  The swarm
// is cut into tiles of blockDim x PPT particles that the resident blocks take
// one at a time from a counter (IterState::tile_next), the next index fetched
// while the current tile runs: blocks on busier SMs or farther from the
// memory take fewer tiles, and all finish within about one tile of each
// other.  A particle's arithmetic does not depend on which block takes it.
// Resident blocks: 2 for PPT = 4 (128 registers), 4 for PPT = 2 (64
// registers, no spill) and PPT = 1: with 32 warps per SM, two
// particles per thread keep the most loads in flight.
// CONS: the constrained path (PPT = 1 only): the cost adds calc_penalty with
// iter = the 1-based particle index, as the reference's sync and queue-lock
// kernels pass it (src/kernels.jl:77,151; handle_constraints adds 1, :28-31).
template <int OBJ, int PPT, bool CONS = false>
__global__ void __launch_bounds__(kSyncThreads, (PPT == 4 ? 2 : 4))
    k_sync_step(SwarmDev s, ObjParams op, PhiloxKeys keys, float c1, float c2, int from_position) {
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
  const int64_t npad = s.npad;
  const int64_t ngroups = npad / PPT;  // groups of PPT particles
  const uint32_t ntiles = (uint32_t)((ngroups + blockDim.x - 1) / blockDim.x);
  float* __restrict__ X = s.X;
  float* __restrict__ V = s.V;
  float* __restrict__ P = s.P;
  const int64_t n = s.n;
  unsigned long long best = ~0ull;
  __shared__ uint32_t s_tile[2];
  if (threadIdx.x == 0) s_tile[0] = atomicAdd(&st->tile_next, 1u);
  __syncthreads();

  for (int slot = 0;; slot ^= 1) {
    const uint32_t tl = s_tile[slot];
    if (tl >= ntiles) break;  // block-uniform
    if (threadIdx.x == 0) s_tile[slot ^ 1] = atomicAdd(&st->tile_next, 1u);  // the next tile, fetched early
    const int64_t q = (int64_t)tl * blockDim.x + threadIdx.x;
    // the tile's last warps may hold fewer groups: the body is conditional,
    // the barrier after it is not (every thread reaches the same barrier)
    if (q < ngroups) {
      const int64_t i0 = q * PPT;
      const uint32_t gi0 = (uint32_t)(s.first + i0);  // index of particle i0 in the whole swarm
      uint8_t fl[PPT];
      ldflags<PPT>(fl, s.flag + i0);
      bool anyfl = false;
#pragma unroll
      for (int k = 0; k < PPT; ++k) anyfl |= (fl[k] != 0);
      Acc<OBJ> acc[PPT];
      ConsAcc ca[PPT];
      if constexpr (CONS) {
#pragma unroll
        for (int k = 0; k < PPT; ++k) ca[k].start(s.cons, s.ncons, D);
      }
      // current pair (dims j, j+1) and the prefetched next pair
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
        for (int k = 0; k < PPT; ++k) r[k] = philox4x32_10(gi0 + (uint32_t)k, (uint32_t)(j >> 1), t, kTagStep, keys);
        {  // dim j
          const int64_t o = (int64_t)j * npad + i0;
          if (anyfl) {
#pragma unroll
            for (int k = 0; k < PPT; ++k) pa[k] = fl[k] ? xa[k] : pa[k];
            stv<PPT>(P + o, pa);
          }
          const float gd = sg[j], lo = slb[j], hi = sub[j];
#pragma unroll
          for (int k = 0; k < PPT; ++k) {
            va[k] = velocity(xa[k], va[k], pa[k], gd, w, c1, c2, u01(r[k].a), u01(r[k].b));
            xa[k] = clamp_lb_ub(__fadd_rn(xa[k], va[k]), lo, hi);
            acc[k].add(op, j, xa[k]);
            if constexpr (CONS) ca[k].add(s.cons, s.ncons, D, j, xa[k]);
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
          const float gd = sg[j + 1], lo = slb[j + 1], hi = sub[j + 1];
#pragma unroll
          for (int k = 0; k < PPT; ++k) {
            vb[k] = velocity(xb[k], vb[k], pb[k], gd, w, c1, c2, u01(r[k].c), u01(r[k].d));
            xb[k] = clamp_lb_ub(__fadd_rn(xb[k], vb[k]), lo, hi);
            acc[k].add(op, j + 1, xb[k]);
            if constexpr (CONS) ca[k].add(s.cons, s.ncons, D, j + 1, xb[k]);
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
        cc[k] = finalize<OBJ>(op, acc[k].s1, acc[k].s2);
        if constexpr (CONS) cc[k] = __fadd_rn(cc[k], penalty(ca[k], s.ncons, __uint2float_rn(gi0 + (uint32_t)(k + 2))));
        const bool valid = i0 + k < n;
        // if cost < best_cost: best = position (strict <, src/kernels.jl:21-24)
        fl[k] = (valid && cc[k] < pc[k]) ? 1 : 0;
        pc[k] = fl[k] ? cc[k] : pc[k];
        if (valid) {
          const unsigned long long key = argmin_key(pc[k], gi0 + (uint32_t)k);
          best = key < best ? key : best;
        }
      }
      stv<PPT>(s.pcost + i0, pc);
      stv<PPT>(s.cost + i0, cc);
      stflags<PPT>(s.flag + i0, fl);
    }
    __syncthreads();  // s_tile[slot ^ 1] written; s_tile[slot] free for the grab after next
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
  st->tile_next = 0u;
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
    case kShiftedSphere: MACRO(kShiftedSphere); break; \
    case kAckley: MACRO(kAckley); break;   \
    case kBeale: MACRO(kBeale); break;     \
    case kBooth: MACRO(kBooth); break;     \
    case kHimmelblau: MACRO(kHimmelblau); break; \
    case kQuadratic: MACRO(kQuadratic); break;   \
    case kBoundaryQuadratic: MACRO(kBoundaryQuadratic); break; \
    default: return set_error(PPS_ENOTSUP, "objective %d has no streaming kernel", obj); \
  }

int launch_init(pps_swarm* s, int sampler, const float* u0_dev) {
  if (is_user(s->objective)) return launch_user_init(s, sampler, u0_dev);
  const int64_t blocks = (s->dv.npad + kSyncThreads - 1) / kSyncThreads;
#define L_INIT(O) k_init<O><<<(unsigned)blocks, kSyncThreads, 0, s->stream>>>(s->dv, s->op, s->seed, sampler, u0_dev)
#define L_INIT_CONS(O) \
  k_init<O, true><<<(unsigned)blocks, kSyncThreads, 0, s->stream>>>(s->dv, s->op, s->seed, sampler, u0_dev)
  if (s->objective == kMlp) {
    L_INIT(kMlp);
  } else if (s->dv.ncons > 0) {
    PPS_DISPATCH_SEPARABLE(s->objective, L_INIT_CONS)
  } else {
    PPS_DISPATCH_SEPARABLE(s->objective, L_INIT)
  }
#undef L_INIT_CONS
#undef L_INIT
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int launch_set_iter(pps_swarm* s, uint32_t t, float w, float wdamp) {
  k_set_iter<<<1, 1, 0, s->stream>>>(s->dv.st, t, w, wdamp);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

// particles per thread of the step kernel: PPS_SYNC_PPT=1|2|4 overrides the
// default of 2 (every variant performs the same work and the same arithmetic).
// Measured on 2^20 x 100-D Rastrigin, ms per iteration (resident blocks):
//   PPT 4: 0.387 (2), 0.401 (3, spills)   PPT 2: 0.393 (3), 0.378 (4), 0.422 (5)
//   PPT 1: 0.464 (6), 0.481 (8)
static int sync_ppt() {
  static int ppt = [] {
    const char* e = getenv("PPS_SYNC_PPT");
    const int v = e ? atoi(e) : 2;
    return (v == 1 || v == 2 || v == 4) ? v : 2;
  }();
  return ppt;
}

template <int OBJ>
static int occupancy_of(int ppt, size_t smem) {
  int per_sm = 0;
  if (ppt == 4)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sync_step<OBJ, 4>, kSyncThreads, smem);
  else if (ppt == 2)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sync_step<OBJ, 2>, kSyncThreads, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sync_step<OBJ, 1>, kSyncThreads, smem);
  return per_sm;
}

// The step kernels keep g, lb and ub (12 bytes per dim) in dynamic shared
// memory.  Without opting in, a block gets 48 kB of static and dynamic shared
// memory together, which 4096 dims (48 kB of dynamic) exceed: above
// kSmemOptIn bytes every step kernel of the objective opts in.  Once per
// objective and size, from sync_grid, which runs before any stream capture.
constexpr size_t kSmemOptIn = 40 << 10;

static int sync_smem_opt_in(const pps_swarm* s) {
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  if (smem <= kSmemOptIn) return PPS_OK;
  // per objective: the size opted in and the device it was set on (function
  // attributes belong to the device's context)
  static thread_local size_t done[kBoundaryQuadratic + 1] = {};
  static thread_local int done_dev[kBoundaryQuadratic + 1] = {};
  if (s->objective < 0 || s->objective > kBoundaryQuadratic) return PPS_OK;
  if (done[s->objective] >= smem && done_dev[s->objective] == s->device) return PPS_OK;
  const int v = (int)smem;
#define OPT_IN(O)                                                                                           \
  do {                                                                                                      \
    PPS_CUDA(cudaFuncSetAttribute(k_sync_step<O, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, v));       \
    PPS_CUDA(cudaFuncSetAttribute(k_sync_step<O, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, v));       \
    PPS_CUDA(cudaFuncSetAttribute(k_sync_step<O, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, v));       \
    PPS_CUDA(cudaFuncSetAttribute(k_sync_step<O, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v)); \
  } while (0)
  PPS_DISPATCH_SEPARABLE(s->objective, OPT_IN)
#undef OPT_IN
  done[s->objective] = smem;
  done_dev[s->objective] = s->device;
  return PPS_OK;
}

int sync_grid(pps_swarm* s) {
  sync_smem_opt_in(s);  // a failure here resurfaces as the launch's own error
  int bulk_blocks = 0;
  sync_bulk_prepare(s, &bulk_blocks);  // the TMA-staged kernel's occupancy, resolved here outside any capture
  // resident blocks of the step kernel per SM (cached per objective, device, dim)
  static thread_local int cached_obj = -1, cached_blocks = 0, cached_dev = -1, cached_dim = -1;
  int per_sm = 0;
  if (cached_obj == s->objective && cached_dev == s->device && cached_dim == s->dv.dim) {
    per_sm = cached_blocks;
  } else {
    const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
    const int ppt = sync_ppt();
    switch (s->objective) {
      case kSphere: per_sm = occupancy_of<kSphere>(ppt, smem); break;
      case kRosenbrock: per_sm = occupancy_of<kRosenbrock>(ppt, smem); break;
      case kRastrigin: per_sm = occupancy_of<kRastrigin>(ppt, smem); break;
      case kAckley: per_sm = occupancy_of<kAckley>(ppt, smem); break;
      default: per_sm = occupancy_of<kBeale>(ppt, smem); break;
    }
    if (per_sm < 1) per_sm = 1;
    cached_obj = s->objective;
    cached_blocks = per_sm;
    cached_dev = s->device;
    cached_dim = s->dv.dim;
  }
  // every resident block, at most one per tile; blocks take tiles dynamically
  const int64_t resident = (int64_t)per_sm * s->sm_count;
  const int64_t tile = (int64_t)kSyncThreads * sync_ppt();
  const int64_t ntiles = (s->dv.npad + tile - 1) / tile;
  int64_t grid = resident < ntiles ? resident : ntiles;
  if (grid < 1) grid = 1;
  return (int)grid;
}

int launch_sync_step(pps_swarm* s, float c1, float c2) {
  if (is_user(s->objective)) return launch_user_step(s, c1, c2);
  if (int rc = sync_smem_opt_in(s)) return rc;
  if (s->dv.ncons == 0) {  // PPS_SYNC_KERNEL=bulk: the TMA-staged kernel where it applies
    bool taken = false;
    const int rc = launch_sync_step_bulk(s, c1, c2, &taken);
    if (rc || taken) return rc;
  }
  const int grid = sync_grid(s);
  const PhiloxKeys keys = philox_round_keys(s->seed);
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  const int from_pos = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  const int ppt = sync_ppt();
#define L_STEP(O)                                                                                       \
  if (ppt == 4)                                                                                         \
    k_sync_step<O, 4><<<grid, kSyncThreads, smem, s->stream>>>(s->dv, s->op, keys, c1, c2, from_pos); \
  else if (ppt == 2)                                                                                    \
    k_sync_step<O, 2><<<grid, kSyncThreads, smem, s->stream>>>(s->dv, s->op, keys, c1, c2, from_pos); \
  else                                                                                                  \
    k_sync_step<O, 1><<<grid, kSyncThreads, smem, s->stream>>>(s->dv, s->op, keys, c1, c2, from_pos)
  if (s->dv.ncons > 0) {
    // constrained path: one particle per thread; tiles of 256 particles,
    // handed out dynamically, so any grid up to 4 blocks per SM is right
    const int64_t ntiles = (s->dv.npad + kSyncThreads - 1) / kSyncThreads;
    const int64_t cgrid = ntiles < 4 * (int64_t)s->sm_count ? ntiles : 4 * (int64_t)s->sm_count;
#define L_STEP_CONS(O) \
  k_sync_step<O, 1, true><<<(unsigned)cgrid, kSyncThreads, smem, s->stream>>>(s->dv, s->op, keys, c1, c2, from_pos)
    PPS_DISPATCH_SEPARABLE(s->objective, L_STEP_CONS)
#undef L_STEP_CONS
  } else {
    PPS_DISPATCH_SEPARABLE(s->objective, L_STEP)
  }
#undef L_STEP
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

// the swarm's result for a host that polls mapped memory: gbest, its cost
// and index, then the done flag after a system-scope fence
__global__ void k_publish_result(SwarmDev s, float* __restrict__ mail, int* done) {
  for (int d = threadIdx.x; d < s.dim; d += blockDim.x) mail[d] = s.g[d];
  if (threadIdx.x == 0) {
    mail[s.dim] = s.st->gcost;
    mail[s.dim + 1] = __uint_as_float(s.st->gidx);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence_system();
    *reinterpret_cast<volatile int*>(done) = 1;
  }
}

int launch_publish_result(pps_swarm* s, float* mail, int* done) {
  k_publish_result<<<1, 256, 0, s->stream>>>(s->dv, mail, done);
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
  if (is_user(objective)) return launch_user_eval(op, od, objective, x, npts, stride, f, stream);
  const int64_t blocks = (npts + 255) / 256;
#define L_EVAL(O) k_eval<O><<<(unsigned)blocks, 256, 0, stream>>>(op, x, npts, stride, f)
  PPS_DISPATCH_SEPARABLE(objective, L_EVAL)
#undef L_EVAL
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

}  // namespace pps
