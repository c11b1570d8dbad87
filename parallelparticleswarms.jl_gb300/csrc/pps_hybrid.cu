// pps_hybrid.cu -- HybridPSO's local stage: one local optimiser per particle.
//
// Reference: src/hybrid.jl:100-158 launches lbfgs_run! (src/lbfgs.jl:9-21),
// one SimpleOptimization._lbfgs per particle started from its personal best,
// then copies result_fx to the host and keeps its findmin if it beats the
// swarm best (:145-150).  The BFGS variant (src/hybrid.jl:33-98) runs
// SimpleNonlinearSolve.SimpleBroyden on grad f = 0 from every particle's
// current position, with the gradient replaced by 1e15 outside the box grown
// by twice its width (BoundedGrad, :15-31).
//
// Algorithms (the published ones the workload names; the third-party code is
// not part of the reference tree):
//   L-BFGS  projected two-loop recursion (Nocedal & Wright, Alg. 7.4), history
//           m, H0 = (s'y / y'y) I, backtracking Armijo (c1) along the projected
//           path, steepest-descent restart when the direction does not descend,
//           stop on ||projected gradient|| <= gtol, maxiters, or a failed search.
//   Broyden inverse-Jacobian ("good") update by Sherman-Morrison, J0 = I, a
//           halving backtrack on ||F||^2, stop on ||F|| <= gtol.
// Every dot product is a sequential binary32 sum (no fusion), the operation
// sequence of the CPU restatement, so results are bit-identical to it.
//
// GB300 design: one thread per particle; vectors of the particle's dimension
// live in registers (compile-time bound MAXD).  Up to 16 dims the L-BFGS
// history (2 m MAXD + 2 m floats per particle) lives in shared memory, particle
// fastest (element (slot, d) of thread t at (slot MAXD + d) 64 + t in blocks of
// 64, so a warp's accesses hit 32 banks at compile-time offsets);
// longer histories stay in thread-local memory.  From 8 dims Broyden's inverse
// Jacobian (D^2 floats) lives in shared memory the same way (blocks of 64).  The
// argmin over the per-particle results (the reference's host findmin) runs on
// the device with the 64-bit (cost, index) key.  The optimisers' device code
// is in pps_local.cuh, which NVRTC also compiles for a user objective with a
// gradient (pps_user.cu); this file holds the registered objectives' kernels
// and the launch logic.
#include <cmath>

#include "pps_internal.h"
#include "pps_local.cuh"

namespace pps {

// the kernels of the registered objectives over the shared device code
template <int OBJ, int MAXD, bool SMEM>
__global__ void __launch_bounds__(SMEM ? kLbfgsThreads : 128)
    k_lbfgs(const float* __restrict__ X0, int64_t ld, int64_t n, ObjParams op, const float* __restrict__ lbp,
            const float* __restrict__ ubp, LocalOpts o, float* __restrict__ xout, float* __restrict__ fout,
            float* __restrict__ itout, unsigned int* next) {
  lbfgs_run<OBJ, MAXD, SMEM>(X0, ld, n, op, lbp, ubp, o, xout, fout, itout, next);
}

template <int OBJ, int MAXD, bool SMEM>
__global__ void __launch_bounds__(SMEM ? kBroydenThreads : 128)
    k_broyden(const float* __restrict__ X0, int64_t ld, int64_t n, ObjParams op, const float* __restrict__ lbp,
              const float* __restrict__ ubp, LocalOpts o, float* __restrict__ xout, float* __restrict__ fout,
              float* __restrict__ itout, unsigned int* next) {
  broyden_run<OBJ, MAXD, SMEM>(X0, ld, n, op, lbp, ubp, o, xout, fout, itout, next);
}

// argmin over the local results (findmin, src/hybrid.jl:145-146) and gather
// of the winner's point; key/count live in the result block
struct ArgminSlot {
  unsigned long long key;
  unsigned int count;
  unsigned int idx;
  float cost;
  unsigned int next;  // the L-BFGS kernel's work counter (particles handed out after the first wave)
  unsigned int pad[58];
};

__global__ void k_reset_slot(ArgminSlot* sl) {
  sl->key = ~0ull;
  sl->count = 0u;
}

__global__ void k_argmin_gather(const float* __restrict__ f, const float* __restrict__ X, int64_t n, int64_t ld, int D,
                                ArgminSlot* sl, float* __restrict__ u) {
  __shared__ unsigned long long wmin[32];
  __shared__ int last;
  unsigned long long key = ~0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = argmin_key(f[i], (uint32_t)i);
    key = k < key ? k : key;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, key, off);
    key = o < key ? o : key;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wmin[warp] = key;
  __syncthreads();
  if (warp == 0) {
    unsigned long long k = (lane < (int)(blockDim.x >> 5)) ? wmin[lane] : ~0ull;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, k, off);
      k = o < k ? o : k;
    }
    if (lane == 0) {
      atomicMin(&sl->key, k);
      __threadfence();
      last = (atomicAdd(&sl->count, 1u) == gridDim.x - 1) ? 1 : 0;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const unsigned long long best = atomicAdd(&sl->key, 0ull);
  const uint32_t gi = (uint32_t)best;
  for (int d = threadIdx.x; d < D; d += blockDim.x) u[d] = __ldcg(X + (int64_t)d * ld + gi);
  if (threadIdx.x == 0) {
    sl->idx = gi;
    sl->cost = __ldcg(f + gi);
  }
}

static int ensure_local_block(pps_swarm* s) {
  if (s->local_block) return PPS_OK;
  const size_t npad = (size_t)s->dv.npad, D = (size_t)s->dv.dim;
  const size_t bytes = sizeof(float) * (D * npad + 2 * npad + 256) + sizeof(ArgminSlot) + 256;
  PPS_CUDA(cudaMalloc(&s->local_block, bytes));
  return PPS_OK;
}

struct LocalBufs {
  float* x;
  float* f;
  float* it;
  float* u;
  ArgminSlot* slot;
};

static LocalBufs local_bufs(pps_swarm* s) {
  const size_t npad = (size_t)s->dv.npad, D = (size_t)s->dv.dim;
  float* b = static_cast<float*>(s->local_block);
  LocalBufs lb;
  lb.x = b;
  lb.f = b + D * npad;
  lb.it = lb.f + npad;
  lb.u = lb.it + npad;  // 256 floats (dim <= 64)
  lb.slot = reinterpret_cast<ArgminSlot*>(lb.u + 256);
  return lb;
}

// L-BFGS: up to 16 dims the history lives in shared memory, blocks of 64
// (m = 10: 56 KB at MAXD 10; the largest, m = 16 at MAXD 16: 136 KB, one
// block per SM); above 16 dims in thread-local memory
// The grid is the resident blocks (at most one thread per particle); the
// particles after the first wave are handed out by the work counter.
template <typename K>
static unsigned resident_blocks(K kernel, int threads, size_t smem, int sm_count, int64_t n) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  const int64_t need = (n + threads - 1) / threads;
  const int64_t resident = (int64_t)per_sm * sm_count;
  return (unsigned)(need < resident ? need : resident);
}

template <int OBJ, int MAXD>
static int launch_local_lbfgs(pps_swarm* s, const float* x0, const LocalOpts& o, const LocalBufs& b) {
  const int64_t n = s->dv.n;
  PPS_CUDA(cudaMemsetAsync(&b.slot->next, 0, sizeof(b.slot->next), s->stream));
  if constexpr (MAXD <= 16) {
    const size_t smem = sizeof(float) * lbfgs_hist_floats(o.history, MAXD) * kLbfgsThreads;
    PPS_CUDA(cudaFuncSetAttribute(k_lbfgs<OBJ, MAXD, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = resident_blocks(k_lbfgs<OBJ, MAXD, true>, kLbfgsThreads, smem, s->sm_count, n);
    k_lbfgs<OBJ, MAXD, true><<<blocks, kLbfgsThreads, smem, s->stream>>>(x0, s->dv.npad, n, s->op, s->dv.lb,
                                                                          s->dv.ub, o, b.x, b.f, b.it, &b.slot->next);
  } else {
    const unsigned blocks = resident_blocks(k_lbfgs<OBJ, MAXD, false>, 128, 0, s->sm_count, n);
    k_lbfgs<OBJ, MAXD, false><<<blocks, 128, 0, s->stream>>>(x0, s->dv.npad, n, s->op, s->dv.lb, s->dv.ub, o, b.x,
                                                              b.f, b.it, &b.slot->next);
  }
  return PPS_OK;
}

// Broyden: from 8 dims the inverse Jacobian (MAXD^2 floats a particle) lives
// in shared memory, blocks of 64 (16 KB at MAXD 8, 25 KB at 10, 64 KB at 16)
template <int OBJ, int MAXD>
static int launch_local_broyden(pps_swarm* s, const float* x0, const LocalOpts& o, const LocalBufs& b) {
  const int64_t n = s->dv.n;
  PPS_CUDA(cudaMemsetAsync(&b.slot->next, 0, sizeof(b.slot->next), s->stream));
  if constexpr (MAXD >= 8) {
    const size_t smem = sizeof(float) * MAXD * MAXD * kBroydenThreads;
    if (smem > (48u << 10))
      PPS_CUDA(cudaFuncSetAttribute(k_broyden<OBJ, MAXD, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = resident_blocks(k_broyden<OBJ, MAXD, true>, kBroydenThreads, smem, s->sm_count, n);
    k_broyden<OBJ, MAXD, true><<<blocks, kBroydenThreads, smem, s->stream>>>(x0, s->dv.npad, n, s->op, s->dv.lb,
                                                                             s->dv.ub, o, b.x, b.f, b.it,
                                                                             &b.slot->next);
  } else {
    const unsigned blocks = resident_blocks(k_broyden<OBJ, MAXD, false>, 128, 0, s->sm_count, n);
    k_broyden<OBJ, MAXD, false><<<blocks, 128, 0, s->stream>>>(x0, s->dv.npad, n, s->op, s->dv.lb, s->dv.ub, o,
                                                                b.x, b.f, b.it, &b.slot->next);
  }
  return PPS_OK;
}

template <int OBJ, int MAXD>
static int launch_local_t(pps_swarm* s, int kind, const float* x0, const LocalOpts& o, const LocalBufs& b) {
  if (kind == 0) return launch_local_lbfgs<OBJ, MAXD>(s, x0, o, b);
  return launch_local_broyden<OBJ, MAXD>(s, x0, o, b);
}

int launch_user_local(pps_swarm* s, int kind, const float* x0, const LocalOpts& o, float* xout, float* fout,
                      float* itout);  // pps_user.cu

template <int OBJ>
static int launch_local_obj(pps_swarm* s, int kind, const float* x0, const LocalOpts& o, const LocalBufs& b) {
  const int D = s->dv.dim;
  if (kind == 1 && D > 16) return set_error(PPS_ENOTSUP, "the Broyden local stage supports dim <= 16 (got %d)", D);
  int rc;
  if constexpr (OBJ >= kBeale) {  // closed forms are defined for dim <= 2
    rc = launch_local_t<OBJ, 2>(s, kind, x0, o, b);
  } else {
    if (D <= 2) rc = launch_local_t<OBJ, 2>(s, kind, x0, o, b);
    else if (D <= 4) rc = launch_local_t<OBJ, 4>(s, kind, x0, o, b);
    else if (D <= 8) rc = launch_local_t<OBJ, 8>(s, kind, x0, o, b);
    else if (D <= 10) rc = kind == 0 ? launch_local_lbfgs<OBJ, 10>(s, x0, o, b)
                                     : launch_local_broyden<OBJ, 10>(s, x0, o, b);
    else if (D <= 16) rc = launch_local_t<OBJ, 16>(s, kind, x0, o, b);
    else if (D <= 32) rc = launch_local_lbfgs<OBJ, 32>(s, x0, o, b);
    else rc = launch_local_lbfgs<OBJ, 64>(s, x0, o, b);
  }
  if (rc) return rc;
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

// kind 0: L-BFGS from personal bests; kind 1: Broyden from positions
int run_local(pps_swarm* s, int kind, const pps_local_opts* opts, float* u_out, float* f_out, int64_t* idx_out,
              float* device_ms) {
  if (!s) return set_error(PPS_EINVAL, "swarm is NULL");
  if (!s->initialized) return set_error(PPS_EINVAL, "swarm is not initialised");
  if (s->shard) return set_error(PPS_ENOTSUP, "the local stage runs on a whole swarm, not on a shard");
  if (!opts) return set_error(PPS_EINVAL, "options are NULL");
  if (kind == 0 && (opts->history < 1 || opts->history > kMaxHistory))
    return set_error(PPS_EINVAL, "history must be in [1, %d] (got %d)", kMaxHistory, opts->history);
  if (opts->maxiters < 0 || opts->max_backtracks < 1)
    return set_error(PPS_EINVAL, "maxiters must be >= 0 and max_backtracks >= 1");
  if (!(opts->gtol >= 0.0f) || !std::isfinite(opts->armijo_c1))
    return set_error(PPS_EINVAL, "gtol must be >= 0 and armijo_c1 finite");
  if (s->dv.dim > 64) return set_error(PPS_ENOTSUP, "the local stage supports dim <= 64 (got %d)", s->dv.dim);
  if (is_ode(s->objective)) return set_error(PPS_ENOTSUP, "ODE-fit objectives have no analytic gradient here");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != s->device) PPS_CUDA(cudaSetDevice(s->device));
  int rc = ensure_local_block(s);
  if (rc) return rc;
  const LocalBufs b = local_bufs(s);
  LocalOpts o{opts->history, opts->maxiters, opts->armijo_c1, opts->gtol, opts->max_backtracks};
  const float* x0 = (kind == 0) ? s->dv.P : s->dv.X;
  PPS_CUDA(cudaEventRecord(s->ev0, s->stream));
  switch (s->objective) {
    case kSphere: rc = launch_local_obj<kSphere>(s, kind, x0, o, b); break;
    case kRosenbrock: rc = launch_local_obj<kRosenbrock>(s, kind, x0, o, b); break;
    case kRastrigin: rc = launch_local_obj<kRastrigin>(s, kind, x0, o, b); break;
    case kAckley: rc = launch_local_obj<kAckley>(s, kind, x0, o, b); break;
    case kBeale: rc = launch_local_obj<kBeale>(s, kind, x0, o, b); break;
    case kBooth: rc = launch_local_obj<kBooth>(s, kind, x0, o, b); break;
    case kHimmelblau: rc = launch_local_obj<kHimmelblau>(s, kind, x0, o, b); break;
    case kQuadratic: rc = launch_local_obj<kQuadratic>(s, kind, x0, o, b); break;
    case kBoundaryQuadratic: rc = launch_local_obj<kBoundaryQuadratic>(s, kind, x0, o, b); break;
    default:
      if (!is_user(s->objective)) return set_error(PPS_ENOTSUP, "objective %d has no gradient", s->objective);
      rc = launch_user_local(s, kind, x0, o, b.x, b.f, b.it);  // its source's gradient, compiled at run time
  }
  if (rc) return rc;
  k_reset_slot<<<1, 1, 0, s->stream>>>(b.slot);
  k_argmin_gather<<<s->sm_count, 256, 0, s->stream>>>(b.f, b.x, s->dv.n, s->dv.npad, s->dv.dim, b.slot, b.u);
  PPS_CUDA(cudaGetLastError());
  PPS_CUDA(cudaEventRecord(s->ev1, s->stream));
  ArgminSlot slot;
  PPS_CUDA(cudaMemcpyAsync(&slot, b.slot, sizeof(slot), cudaMemcpyDeviceToHost, s->stream));
  if (u_out) PPS_CUDA(cudaMemcpyAsync(u_out, b.u, sizeof(float) * s->dv.dim, cudaMemcpyDeviceToHost, s->stream));
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  if (device_ms) PPS_CUDA(cudaEventElapsedTime(device_ms, s->ev0, s->ev1));
  if (f_out) *f_out = slot.cost;
  if (idx_out) *idx_out = (int64_t)slot.idx;
  s->local_valid = 1;
  return PPS_OK;
}

int local_field(pps_swarm* s, int32_t field, float** dev, int* rows) {
  if (!s->local_block || !s->local_valid) return set_error(PPS_EINVAL, "no local-stage results yet");
  const LocalBufs b = local_bufs(s);
  switch (field) {
    case PPS_FIELD_LOCAL_X: *dev = b.x; *rows = s->dv.dim; return PPS_OK;
    case PPS_FIELD_LOCAL_F: *dev = b.f; *rows = 1; return PPS_OK;
    case PPS_FIELD_LOCAL_ITERS: *dev = b.it; *rows = 1; return PPS_OK;
    default: return set_error(PPS_EINVAL, "unknown field %d", field);
  }
}

}  // namespace pps

using namespace pps;

extern "C" int pps_hybrid_lbfgs(pps_swarm* s, const pps_local_opts* o, float* u, float* f, int64_t* idx,
                                float* device_ms) {
  return run_local(s, 0, o, u, f, idx, device_ms);
}

extern "C" int pps_hybrid_bfgs(pps_swarm* s, const pps_local_opts* o, float* u, float* f, int64_t* idx,
                               float* device_ms) {
  return run_local(s, 1, o, u, f, idx, device_ms);
}
