// pps_noalloc.cu -- pps_sync_run_noalloc: the synchronous PSO run on swarm
// arrays that the caller owns, with no allocation by this library.
//
// Who needs it.  A caller whose device memory belongs to someone else cannot
// let a library call cudaMalloc behind its back: a Julia program whose
// arrays live in CUDA.jl's pooled allocator (a hidden cudaMalloc can fail
// while the pool holds the memory, and it synchronises the device), a host
// framework that hands every buffer to its plugins from its own arena, or a
// latency-bound loop where the implicit synchronisation of cudaMalloc and
// cudaFree is not acceptable.  Such a caller passes its own x, v, pbest,
// costs, bounds and global-best buffers, plus a stream, and this entry point
// runs the same kernels as pps_sync_run on them.
//
// Scratch.  The step kernel needs memory beyond its inputs and outputs: the
// iteration state (argmin slot, block ticket, t, w) and one byte per particle
// that defers the personal-best copy.  Here that scratch is the file-scope
// array g_noalloc_scratch below, sized for kNoAllocMaxParticles particles
// (1 MiB + 256 bytes).  Every GPU that loads the library holds it until the
// process exits.  Its address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call on that
// device; make that first call before any stream capture begins.
//
// Concurrency.  Every call shares the one array, which keeps the contents of
// the last call (each call clears the flags and resets the iteration state it
// needs).  Calls whose work overlaps on the GPU -- on different streams, or
// from several host threads without ordering -- race on it and give wrong
// results; serialise them.
#include <cmath>
#include <cstddef>
#include <mutex>

#include "pps_internal.h"

namespace pps {

constexpr int64_t kNoAllocMaxParticles = int64_t(1) << 20;
constexpr size_t kNoAllocStateBytes = 256;  // IterState padded to 256 B
static_assert(sizeof(IterState) <= kNoAllocStateBytes, "iteration state outgrew its slot");

// [0, 256): IterState; [256, 256 + kNoAllocMaxParticles): personal-best flags
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocStateBytes + kNoAllocMaxParticles];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_addr[kMaxDevices] = {};

// host-side address of this device's copy of g_noalloc_scratch
static int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return set_error(PPS_ENOTSUP, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_addr[device];
  return PPS_OK;
}

// argmin of pcost (lowest index on ties) and gather of the winner into g:
// the global best the run starts from
__global__ void k_noalloc_select(SwarmDev s, int from_position) {
  __shared__ unsigned long long wmin[32];
  __shared__ int last;
  IterState* st = s.st;
  unsigned long long key = ~0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = argmin_key(s.pcost[i], (uint32_t)i);
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
      atomicMin(&st->key, k);
      __threadfence();
      last = (atomicAdd(&st->count, 1u) == gridDim.x - 1) ? 1 : 0;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const unsigned long long best = atomicAdd(&st->key, 0ull);
  const uint32_t gi = (uint32_t)best;
  const float* src = from_position ? s.X : s.P;
  for (int d = threadIdx.x; d < s.dim; d += blockDim.x) s.g[d] = __ldcg(src + (int64_t)d * s.npad + gi);
  if (threadIdx.x == 0) {
    st->gcost = __ldcg(s.pcost + gi);
    st->gidx = gi;
    st->key = ~0ull;
    st->count = 0u;
  }
}

// the global best of a swarm whose personal bests were just set.  The argmin
// slot and the block ticket are reset first: a swarm that was created but
// never initialised holds zeros there (a zero key would make particle 0 the
// winner whatever its cost); t and w are left as they are.
int launch_select_gbest(pps_swarm* s) {
  static_assert(offsetof(IterState, key) == 0 && offsetof(IterState, count) == 8, "IterState layout");
  PPS_CUDA(cudaMemsetAsync(&s->dv.st->key, 0xFF, sizeof(s->dv.st->key), s->stream));
  PPS_CUDA(cudaMemsetAsync(&s->dv.st->count, 0, sizeof(s->dv.st->count), s->stream));
  k_noalloc_select<<<s->sm_count, 256, 0, s->stream>>>(s->dv, (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace pps

using namespace pps;

extern "C" int pps_sync_run_noalloc(int32_t objective, const float* params, int32_t nparams,
                                    const pps_device_swarm* sw, uint64_t seed, uint32_t iteration,
                                    int32_t maxiters, float w, float wdamp, float c1, float c2,
                                    uint32_t flags, void* stream, float* gcost_out, int64_t* gidx_out) {
  if (!sw) return set_error(PPS_EINVAL, "device swarm is NULL");
  if (sw->n < 1 || sw->n > kNoAllocMaxParticles)
    return set_error(PPS_EINVAL, "pps_sync_run_noalloc supports 1 <= n <= %lld particles (got %lld)",
                     (long long)kNoAllocMaxParticles, (long long)sw->n);
  if (sw->ld < sw->n || sw->ld % 32 != 0 || sw->ld > kNoAllocMaxParticles)
    return set_error(PPS_EINVAL, "ld must be a multiple of 32 with n <= ld <= %lld (got ld=%lld, n=%lld)",
                     (long long)kNoAllocMaxParticles, (long long)sw->ld, (long long)sw->n);
  if (sw->dim < 1 || sw->dim > 4096) return set_error(PPS_EINVAL, "dim must be in [1, 4096] (got %d)", sw->dim);
  if (nparams < 0 || nparams > 8 || (nparams > 0 && !params))
    return set_error(PPS_EINVAL, "nparams must be in [0, 8] with params set");
  if (maxiters < 0) return set_error(PPS_EINVAL, "maxiters must be >= 0");
  if (!std::isfinite(w) || !std::isfinite(wdamp) || !std::isfinite(c1) || !std::isfinite(c2))
    return set_error(PPS_EINVAL, "coefficients must be finite");
  // the Philox counters of an iteration include its number: a wrapped counter repeats draws
  if ((uint64_t)iteration + (uint64_t)maxiters > 0xFFFFFFFFull)
    return set_error(PPS_EINVAL, "iteration counter would overflow (iteration %u + maxiters %d)", iteration, maxiters);
  const void* ptrs[]= {sw->x, sw->v, sw->pbest, sw->pcost, sw->cost, sw->lb, sw->ub, sw->g};
  for (const void* p : ptrs) {
    if (!p) return set_error(PPS_EINVAL, "a device buffer of the swarm is NULL");
    if (!aligned16(p)) return set_error(PPS_EINVAL, "device buffers must be 16-byte aligned");
  }
  switch (objective) {
    case kSphere: case kRosenbrock: case kRastrigin: case kAckley: case kBeale: case kBooth:
    case kHimmelblau: case kQuadratic: case kBoundaryQuadratic: case kShiftedSphere:
      break;
    default:
      return set_error(PPS_ENOTSUP, "objective %d is not supported by pps_sync_run_noalloc", objective);
  }
  if (objective >= kBeale && sw->dim > 2) return set_error(PPS_EINVAL, "objective %d is defined for dim <= 2", objective);

  int device = 0;
  PPS_CUDA(cudaGetDevice(&device));
  unsigned char* scratch = nullptr;
  int rc = scratch_address(device, &scratch);
  if (rc) return rc;

  // a handle on the host stack that points at the caller's buffers and the
  // static scratch; the existing launchers run on it unchanged
  pps_swarm h;
  h.device = device;
  h.stream = static_cast<cudaStream_t>(stream);
  PPS_CUDA(cudaDeviceGetAttribute(&h.sm_count, cudaDevAttrMultiProcessorCount, device));
  h.dv.X = sw->x;
  h.dv.V = sw->v;
  h.dv.P = sw->pbest;
  h.dv.pcost = sw->pcost;
  h.dv.cost = sw->cost;
  h.dv.flag = scratch + kNoAllocStateBytes;
  h.dv.g = sw->g;
  h.dv.lb = const_cast<float*>(sw->lb);
  h.dv.ub = const_cast<float*>(sw->ub);
  h.dv.st = reinterpret_cast<IterState*>(scratch);
  h.dv.n = sw->n;
  h.dv.npad = sw->ld;
  h.dv.dim = sw->dim;
  for (int k = 0; k < nparams; ++k) h.op.p[k] = params[k];
  h.op.np = nparams;
  h.op.dim = sw->dim;
  h.objective = objective;
  h.seed = seed;
  h.flags = flags & PPS_FLAG_GBEST_FROM_POSITION;

  PPS_CUDA(cudaMemsetAsync(h.dv.flag, 0, (size_t)sw->ld, h.stream));
  PPS_CUDA(cudaMemsetAsync(&h.dv.st->status, 0, sizeof(h.dv.st->status), h.stream));
  if ((rc = launch_set_iter(&h, iteration, w, wdamp))) return rc;
  k_noalloc_select<<<h.sm_count, 256, 0, h.stream>>>(h.dv, (h.flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0);
  PPS_CUDA(cudaGetLastError());
  for (int32_t k = 0; k < maxiters; ++k)
    if ((rc = launch_sync_step(&h, c1, c2))) return rc;
  if ((rc = launch_materialize(&h))) return rc;
  if (gcost_out || gidx_out) {
    IterState st;
    PPS_CUDA(cudaMemcpyAsync(&st, h.dv.st, sizeof(st), cudaMemcpyDeviceToHost, h.stream));
    PPS_CUDA(cudaStreamSynchronize(h.stream));
    if (st.status & 4u) return set_error(PPS_ETIMEOUT, "the step kernel timed out waiting for a bulk copy");
    if (gcost_out) *gcost_out = st.gcost;
    if (gidx_out) *gidx_out = (int64_t)st.gidx;
  }
  return PPS_OK;
}
