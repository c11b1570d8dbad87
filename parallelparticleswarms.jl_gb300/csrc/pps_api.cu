// pps_api.cu -- the C ABI of include/pps.h: swarm lifetime, runs, results.
//
// Reference entry points this layer replaces (all on the host side of the
// reference, which calls KernelAbstractions kernels from Julia):
//   init(prob, ParallelPSOKernel | ParallelSyncPSOKernel)   src/init.jl:56-115
//   reinit!(cache)                                          src/init.jl:117-141
//   solve!(cache) -> vectorized_solve!                      src/solve.jl:11-59,
//                                                           src/lowerlevel_solve.jl:1-121
//   sol.objective = prob.f(gbest.position, prob.p)          src/solve.jl:54-57
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <vector>

#include "pps_internal.h"

namespace pps {

static thread_local char g_err[4096] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  return set_error(e == cudaErrorMemoryAllocation ? PPS_ENOMEM : PPS_ECUDA, "%s: %s (%s)", what,
                   cudaGetErrorString(e), cudaGetErrorName(e));
}

static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static bool supported_objective(int obj) {
  switch (obj) {
    case kSphere:
    case kRosenbrock:
    case kRastrigin:
    case kAckley:
    case kBeale:
    case kBooth:
    case kHimmelblau:
    case kQuadratic:
    case kBoundaryQuadratic:
    case kLvFit:
    case kFhnFit:
    case kMlp:
    case kShiftedSphere:
      return true;
    default:
      return is_user(obj);
  }
}

static int check_problem(const pps_problem* prob) {
  if (!prob) return set_error(PPS_EINVAL, "problem is NULL");
  if (prob->dim < 1 || prob->dim > 4096)
    return set_error(PPS_EINVAL, "dim must be in [1, 4096] (got %d)", prob->dim);
  if (prob->nparams < 0 || prob->nparams > 8)
    return set_error(PPS_EINVAL, "nparams must be in [0, 8] (got %d)", prob->nparams);
  if (prob->nparams > 0 && !prob->params) return set_error(PPS_EINVAL, "params is NULL");
  if (!supported_objective(prob->objective))
    return set_error(PPS_ENOTSUP, "objective %d is not supported by this entry point", prob->objective);
  if (prob->objective >= kBeale && prob->objective <= kBoundaryQuadratic && prob->dim > 2)
    return set_error(PPS_EINVAL, "objective %d is defined for dim <= 2", prob->objective);
  if (is_ode(prob->objective)) {
    const int rc = ode_check(prob);
    if (rc) return rc;
  }
  if (prob->objective == kMlp) {
    const int rc = mlp_check(prob);
    if (rc) return rc;
  }
  if (is_user(prob->objective) && prob->ndata != 0 && (prob->ndata < 0 || !prob->data))
    return set_error(PPS_EINVAL, "data is NULL or ndata is negative");
  if (prob->ncons < 0 || prob->ncons > kMaxCons)
    return set_error(PPS_EINVAL, "ncons must be in [0, %d] (got %d)", kMaxCons, prob->ncons);
  if (prob->ncons > 0) {
    if (!prob->cons) return set_error(PPS_EINVAL, "cons is NULL");
    if (is_ode(prob->objective) || prob->objective == kMlp)
      return set_error(PPS_ENOTSUP, "constraints apply to the registered closed-form objectives only");
    for (int64_t k = 0; k < (int64_t)prob->ncons * (1 + 2 * (int64_t)prob->dim); ++k)
      if (!std::isfinite(prob->cons[k])) return set_error(PPS_EINVAL, "constraint coefficients must be finite");
  }
  for (int d = 0; d < prob->dim; ++d) {
    const float lo = prob->lb ? prob->lb[d] : -INFINITY;
    const float hi = prob->ub ? prob->ub[d] : INFINITY;
    if (std::isnan(lo) || std::isnan(hi) || lo > hi)
      return set_error(PPS_EINVAL, "bounds of dim %d are invalid (lb=%g ub=%g)", d, lo, hi);
  }
  return PPS_OK;
}

static ObjParams make_params(const pps_problem* prob) {
  ObjParams op{};
  for (int k = 0; k < prob->nparams; ++k) op.p[k] = prob->params[k];
  op.np = prob->nparams;
  op.dim = prob->dim;
  return op;
}

// IterState::status: bit 1, a bounded wait of the tensor-core kernel gave up;
// bit 2, a bounded wait of the TMA-staged step kernel gave up
int check_device_status(pps_swarm* s) {
  if (s->objective != kMlp && !s->bounded_waits) return PPS_OK;
  unsigned int status = 0;
  PPS_CUDA(cudaMemcpy(&status, &s->dv.st->status, sizeof(status), cudaMemcpyDeviceToHost));
  if (status & 2u) return set_error(PPS_ETIMEOUT, "the MLP tensor-core kernel timed out waiting for an MMA");
  if (status & 4u) return set_error(PPS_ETIMEOUT, "the step kernel timed out waiting for a bulk copy");
  return PPS_OK;
}

}  // namespace pps

using namespace pps;

extern "C" {

int32_t pps_version(void) { return PPS_VERSION; }

const char* pps_last_error(void) { return g_err; }

int pps_device_count(int32_t* count) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (count) *count = (e == cudaSuccess) ? c : 0;
  if (e != cudaSuccess) return set_error(PPS_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
  return PPS_OK;
}

int pps_set_device(int32_t device) {
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess || c < 1) return set_error(PPS_ENODEV, "no CUDA device");
  if (device < 0 || device >= c) return set_error(PPS_EINVAL, "device %d out of range [0, %d)", device, c);
  PPS_CUDA(cudaSetDevice(device));
  return PPS_OK;
}

}  // extern "C"

namespace pps {

// One device block per swarm, carved into 256-byte-aligned arrays.
struct SwarmLayout {
  size_t oX, oV, oP, oPc, oC, oF, oG, oLb, oUb, oU0, oSt, oData, oMlpA, oCons, oRec, bytes;
  int64_t npad;
  int mlp_samples;
};

static SwarmLayout swarm_layout(const pps_problem* prob, int64_t n, bool shard = false) {
  SwarmLayout L{};
  const int D = prob->dim;
  L.npad = (int64_t)align_up((size_t)n, 64);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  L.oX = take(sizeof(float) * D * L.npad);
  L.oV = take(sizeof(float) * D * L.npad);
  L.oP = take(sizeof(float) * D * L.npad);
  L.oPc = take(sizeof(float) * L.npad);
  L.oC = take(sizeof(float) * L.npad);
  L.oF = take(L.npad);
  L.oG = take(sizeof(float) * D);
  L.oLb = take(sizeof(float) * D);
  L.oUb = take(sizeof(float) * D);
  L.oU0 = take(sizeof(float) * D);
  L.oSt = take(sizeof(IterState));
  L.oData = take(sizeof(float) * (prob->data ? (size_t)prob->ndata : 0));
  L.mlp_samples = prob->objective == kMlp ? (int)(prob->ndata / 17) : 0;
  L.oMlpA = take(L.mlp_samples ? mlp_a_bytes(L.mlp_samples) : 0);
  L.oCons = take(sizeof(float) * (size_t)(prob->ncons > 0 ? prob->ncons : 0) * (1 + 2 * (size_t)D));
  L.oRec = take(shard ? (size_t)shard_record_bytes(D) : 0);
  L.bytes = off;
  return L;
}

int swarm_check(const pps_problem* prob, int64_t n) {
  const int rc = check_problem(prob);
  if (rc) return rc;
  if (n < 1 || n > (int64_t)0xFFFFFF00LL)
    return set_error(PPS_EINVAL, "n must be in [1, 2^32-256] (got %lld)", (long long)n);
  return PPS_OK;
}

size_t swarm_device_bytes(const pps_problem* prob, int64_t n) { return swarm_layout(prob, n).bytes; }

// Points the swarm at device block `b` (layout L), copies the bounds, start
// point and data asynchronously on s->stream and zeroes the rest.  Host
// buffers are pageable, so each copy has left them when the call returns.
static int swarm_setup(pps_swarm* s, const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags, char* b,
                       const SwarmLayout& L) {
  const int D = prob->dim;
  s->bytes = L.bytes;
  s->dv.X = reinterpret_cast<float*>(b + L.oX);
  s->dv.V = reinterpret_cast<float*>(b + L.oV);
  s->dv.P = reinterpret_cast<float*>(b + L.oP);
  s->dv.pcost = reinterpret_cast<float*>(b + L.oPc);
  s->dv.cost = reinterpret_cast<float*>(b + L.oC);
  s->dv.flag = reinterpret_cast<uint8_t*>(b + L.oF);
  s->dv.g = reinterpret_cast<float*>(b + L.oG);
  s->dv.lb = reinterpret_cast<float*>(b + L.oLb);
  s->dv.ub = reinterpret_cast<float*>(b + L.oUb);
  s->dv.st = reinterpret_cast<IterState*>(b + L.oSt);
  s->u0_dev = reinterpret_cast<float*>(b + L.oU0);
  s->data_dev = reinterpret_cast<float*>(b + L.oData);
  s->od.data = s->data_dev;
  s->od.ndata = prob->data ? prob->ndata : 0;
  if (L.mlp_samples) s->mlp_a_dev = b + L.oMlpA;
  s->dv.n = n;
  s->dv.npad = L.npad;
  s->dv.first = 0;
  s->dv.nglobal = n;
  s->dv.xrec = nullptr;
  s->dv.dim = D;
  s->dv.ncons = prob->ncons > 0 ? prob->ncons : 0;
  s->dv.cons = s->dv.ncons ? reinterpret_cast<const float*>(b + L.oCons) : nullptr;
  s->op = make_params(prob);
  s->op.data = s->od.data;  // the local optimisers of a user objective read it through the parameters
  s->op.ndata = s->od.ndata;
  s->objective = prob->objective;
  s->seed = seed;
  s->flags = flags;
  s->host_lb = static_cast<float*>(malloc(sizeof(float) * 3 * D));
  if (!s->host_lb) return set_error(PPS_ENOMEM, "host allocation failed");
  s->host_ub = s->host_lb + D;
  s->host_u0 = s->host_lb + 2 * D;
  for (int d = 0; d < D; ++d) {
    s->host_lb[d] = prob->lb ? prob->lb[d] : -INFINITY;
    s->host_ub[d] = prob->ub ? prob->ub[d] : INFINITY;
    s->host_u0[d] = prob->u0 ? prob->u0[d] : 0.0f;
  }
  PPS_CUDA(cudaMemsetAsync(b, 0, L.bytes, s->stream));
  PPS_CUDA(cudaMemcpyAsync(s->dv.lb, s->host_lb, sizeof(float) * D, cudaMemcpyHostToDevice, s->stream));
  PPS_CUDA(cudaMemcpyAsync(s->dv.ub, s->host_ub, sizeof(float) * D, cudaMemcpyHostToDevice, s->stream));
  PPS_CUDA(cudaMemcpyAsync(s->u0_dev, s->host_u0, sizeof(float) * D, cudaMemcpyHostToDevice, s->stream));
  if (prob->data && prob->ndata > 0)
    PPS_CUDA(cudaMemcpyAsync(s->data_dev, prob->data, sizeof(float) * (size_t)prob->ndata, cudaMemcpyHostToDevice,
                             s->stream));
  if (s->dv.ncons)
    PPS_CUDA(cudaMemcpyAsync(b + L.oCons, prob->cons, sizeof(float) * (size_t)s->dv.ncons * (1 + 2 * (size_t)D),
                             cudaMemcpyHostToDevice, s->stream));
  if (L.mlp_samples) {
    std::vector<uint8_t> packed(mlp_a_bytes(L.mlp_samples));
    mlp_pack_a(prob->data, L.mlp_samples, packed.data());
    PPS_CUDA(cudaMemcpyAsync(s->mlp_a_dev, packed.data(), packed.size(), cudaMemcpyHostToDevice, s->stream));
  }
  return PPS_OK;
}

// A swarm over caller-owned device memory (at least swarm_device_bytes) and
// a caller-owned stream: used by the server, which carves swarms from its
// arena.  Nothing is synchronised.
int swarm_attach(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags, void* mem, cudaStream_t stream,
                 pps_swarm** out) {
  *out = nullptr;
  int rc = swarm_check(prob, n);
  if (rc) return rc;
  pps_swarm* s = new (std::nothrow) pps_swarm();
  if (!s) return set_error(PPS_ENOMEM, "host allocation failed");
  s->owns_memory = false;
  cudaGetDevice(&s->device);
  const cudaError_t ea = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (ea != cudaSuccess) {
    delete s;
    return cuda_error(ea, "cudaDeviceGetAttribute(multiprocessor count)");
  }
  s->stream = stream;
  if ((rc = swarm_setup(s, prob, n, seed, flags, static_cast<char*>(mem), swarm_layout(prob, n)))) {
    swarm_detach(s);
    return rc;
  }
  *out = s;
  return PPS_OK;
}

// releases what an attached swarm owns on the host (its graph included);
// the caller makes sure its stream has finished with it
void swarm_detach(pps_swarm* s) {
  if (!s) return;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  free(s->host_lb);
  delete s;
}

}  // namespace pps

extern "C" {

}  // extern "C"

namespace pps {

// pps_swarm_create, and for a shard (nglobal > 0) pps_shard_create: the
// swarm holds n particles, particles first .. first + n - 1 of nglobal
int swarm_create(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags, int64_t first,
                 int64_t nglobal, pps_swarm** out) {
  if (!out) return set_error(PPS_EINVAL, "out is NULL");
  *out = nullptr;
  int rc = swarm_check(prob, n);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_error(PPS_ENODEV, "no CUDA device");
  pps_swarm* s = new (std::nothrow) pps_swarm();
  if (!s) return set_error(PPS_ENOMEM, "host allocation failed");
  cudaGetDevice(&s->device);
  cudaError_t ea = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (ea != cudaSuccess) {
    delete s;
    return cuda_error(ea, "cudaDeviceGetAttribute(multiprocessor count)");
  }
  const bool shard = nglobal > 0;
  const SwarmLayout L = swarm_layout(prob, n, shard);
  cudaError_t e = cudaMalloc(&s->block, L.bytes);
  if (e != cudaSuccess) {
    delete s;
    return cuda_error(e, "cudaMalloc(swarm state)");
  }
  rc = PPS_OK;
  do {
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
      rc = cuda_error(e, "cudaStreamCreate");
      break;
    }
    if ((e = cudaEventCreate(&s->ev0)) != cudaSuccess || (e = cudaEventCreate(&s->ev1)) != cudaSuccess) {
      rc = cuda_error(e, "cudaEventCreate");
      break;
    }
    if ((rc = swarm_setup(s, prob, n, seed, flags, static_cast<char*>(s->block), L))) break;
    if (shard) {
      s->shard = 1;
      s->dv.first = first;
      s->dv.nglobal = nglobal;
      s->dv.xrec = static_cast<unsigned char*>(s->block) + L.oRec;
      s->shard_records = s->dv.xrec;  // until pps_shard_bind: a lone shard exchanges with itself
      s->shard_nrecords = 1;
    }
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) rc = cuda_error(e, "cudaStreamSynchronize");
  } while (0);
  if (rc) {
    pps_swarm_destroy(s);
    return rc;
  }
  *out = s;
  return PPS_OK;
}

}  // namespace pps

extern "C" {

int pps_swarm_create(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags,
                     pps_swarm** out) {
  return swarm_create(prob, n, seed, flags, 0, 0, out);
}

int pps_swarm_destroy(pps_swarm* s) {
  if (!s) return PPS_OK;
  if (!s->owns_memory) return set_error(PPS_EINVAL, "swarm belongs to a server");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != s->device) cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->block) cudaFree(s->block);
  if (s->local_block) cudaFree(s->local_block);
  free(s->host_lb);
  if (dev >= 0 && dev != s->device) cudaSetDevice(dev);
  delete s;
  return PPS_OK;
}

static int use_device(pps_swarm* s) {
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != s->device) PPS_CUDA(cudaSetDevice(s->device));
  return PPS_OK;
}

int pps_swarm_init(pps_swarm* s, int32_t sampler) {
  if (!s) return set_error(PPS_EINVAL, "swarm is NULL");
  int rc = use_device(s);
  if (rc) return rc;
  const int D = s->dv.dim;
  if (sampler == PPS_SAMPLER_AUTO) {
    bool all_inf = true;
    for (int d = 0; d < D; ++d)
      if (!(std::isinf(s->host_lb[d]) && std::isinf(s->host_ub[d]))) all_inf = false;
    sampler = all_inf ? PPS_SAMPLER_UNBOUNDED : PPS_SAMPLER_UNIFORM;
  }
  if (sampler != PPS_SAMPLER_UNIFORM && sampler != PPS_SAMPLER_UNBOUNDED && sampler != PPS_SAMPLER_LHS)
    return set_error(PPS_EINVAL, "unknown sampler %d", sampler);
  if (sampler == PPS_SAMPLER_UNIFORM || sampler == PPS_SAMPLER_LHS) {
    for (int d = 0; d < D; ++d)
      if (!std::isfinite(s->host_lb[d]) || !std::isfinite(s->host_ub[d]))
        return set_error(PPS_EINVAL, "%s sampler needs finite bounds (dim %d)",
                         sampler == PPS_SAMPLER_LHS ? "Latin hypercube" : "uniform", d);
  }
  if ((rc = launch_set_iter(s, 0u, 0.7298f, 1.0f))) return rc;
  if ((rc = is_ode(s->objective) ? launch_init_ode(s, sampler, s->u0_dev) : launch_init(s, sampler, s->u0_dev)))
    return rc;
  if (s->objective == kMlp && (rc = launch_mlp_init_eval(s))) return rc;
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  if ((rc = check_device_status(s))) return rc;
  s->t = 0;
  s->initialized = 1;
  s->local_valid = 0;
  return PPS_OK;
}

int pps_swarm_info_get(pps_swarm* s, pps_swarm_info* info) {
  if (!s || !info) return set_error(PPS_EINVAL, "NULL argument");
  info->n = s->dv.n;
  info->dim = s->dv.dim;
  info->objective = s->objective;
  info->iteration = s->t;
  int slice = 0;
  info->async_lanes = async_lanes(s->dv.dim, &slice);
  info->async_slice = slice;
  info->device = s->device;
  info->seed = s->seed;
  info->device_bytes = s->bytes;
  return PPS_OK;
}

static int check_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2) {
  if (!s) return set_error(PPS_EINVAL, "swarm is NULL");
  if (!s->initialized) return set_error(PPS_EINVAL, "swarm is not initialised (call pps_swarm_init)");
  if (s->shard)
    return set_error(PPS_ENOTSUP, "a shard runs through pps_shard_step / pps_shard_async and the global-best exchange");
  if (maxiters < 0) return set_error(PPS_EINVAL, "maxiters must be >= 0");
  if (!std::isfinite(w) || !std::isfinite(wdamp) || !std::isfinite(c1) || !std::isfinite(c2))
    return set_error(PPS_EINVAL, "coefficients must be finite");
  if ((uint64_t)s->t + (uint64_t)maxiters > 0xFFFFFFFFull)
    return set_error(PPS_EINVAL, "iteration counter would overflow");
  return use_device(s);
}

static int finish_timing(pps_swarm* s, float* device_ms) {
  PPS_CUDA(cudaEventSynchronize(s->ev1));
  if (device_ms) {
    float ms = 0.0f;
    PPS_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    *device_ms = ms;
  }
  return PPS_OK;
}

static constexpr int kGraphChunk = 32;

static int step_once(pps_swarm* s, float c1, float c2) {
  if (is_ode(s->objective)) return launch_sync_step_ode(s, c1, c2);
  if (s->objective == kMlp) return launch_mlp_step(s, c1, c2);
  return launch_sync_step(s, c1, c2);
}

// the run's flags for the duration of a run, the swarm's own again on every return
struct RunFlags {
  pps_swarm* s;
  uint32_t saved;
  RunFlags(pps_swarm* sw, uint32_t f) : s(sw), saved(sw->flags) { s->flags = f; }
  ~RunFlags() { s->flags = saved; }
};

static int run_steps(pps_swarm* s, int32_t maxiters, float c1, float c2, uint32_t run_flags) {
  int rc;
  RunFlags scoped(s, run_flags);
  // resolve occupancy (and load a user objective's kernels) outside any capture
  if (is_user(s->objective)) {
    if ((rc = user_prepare(s))) return rc;
  } else if (!is_ode(s->objective)) {
    sync_grid(s);
  }
  if (maxiters >= kGraphChunk) {
    const bool stale = !s->graph || s->graph_len != kGraphChunk || s->graph_async_lanes != (int)run_flags ||
                       s->graph_c1 != c1 || s->graph_c2 != c2;
    if (stale) {
      if (s->graph) cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
      cudaGraph_t g = nullptr;
      PPS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < kGraphChunk; ++k) {
        if ((rc = step_once(s, c1, c2))) {
          cudaStreamEndCapture(s->stream, &g);
          if (g) cudaGraphDestroy(g);
          return rc;
        }
      }
      PPS_CUDA(cudaStreamEndCapture(s->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        s->graph = nullptr;  // unspecified after a failed instantiation
        return cuda_error(e, "cudaGraphInstantiate");
      }
      s->graph_len = kGraphChunk;
      s->graph_async_lanes = (int)run_flags;
      s->graph_c1 = c1;
      s->graph_c2 = c2;
    }
  }
  int32_t left = maxiters;
  while (left >= kGraphChunk) {
    cudaError_t e = cudaGraphLaunch(s->graph, s->stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
    left -= kGraphChunk;
  }
  for (; left > 0; --left) {
    if ((rc = step_once(s, c1, c2))) return rc;
  }
  return PPS_OK;
}

static int sync_like_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                         float* device_ms, uint32_t run_flags) {
  int rc = check_run(s, maxiters, w, wdamp, c1, c2);
  if (rc) return rc;
  if ((rc = launch_set_iter(s, s->t, w, wdamp))) return rc;
  PPS_CUDA(cudaEventRecord(s->ev0, s->stream));
  if ((rc = run_steps(s, maxiters, c1, c2, run_flags))) return rc;
  PPS_CUDA(cudaEventRecord(s->ev1, s->stream));
  if ((rc = launch_materialize(s))) return rc;
  if ((rc = finish_timing(s, device_ms))) return rc;
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  s->t += (uint32_t)maxiters;
  return check_device_status(s);
}

int pps_sync_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                 float* device_ms) {
  return sync_like_run(s, maxiters, w, wdamp, c1, c2, device_ms,
                       s ? (s->flags & PPS_FLAG_GBEST_FROM_POSITION) : 0u);
}

int pps_queue_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                  float* device_ms) {
  // block bests are (pbest, pbest cost) pairs (src/kernels.jl:85-91)
  return sync_like_run(s, maxiters, w, wdamp, c1, c2, device_ms, 0u);
}

int pps_async_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2,
                  float* device_ms) {
  int rc = check_run(s, maxiters, w, wdamp, c1, c2);
  if (rc) return rc;
  if (is_ode(s->objective))
    return set_error(PPS_ENOTSUP, "ODE fits run synchronously (parameter_estim_ode!); use pps_sync_run");
  if (s->objective == kMlp)
    return set_error(PPS_ENOTSUP, "the MLP objective runs synchronously (tensor-core evaluation); use pps_sync_run");
  if (s->dv.ncons > 0)
    return set_error(PPS_ENOTSUP, "constrained problems run with pps_sync_run / pps_queue_run");
  if ((rc = launch_set_iter(s, s->t, w, wdamp))) return rc;
  PPS_CUDA(cudaEventRecord(s->ev0, s->stream));
  int lanes = 0;
  if ((rc = is_user(s->objective) ? launch_user_async(s, maxiters, c1, c2) : launch_async(s, maxiters, c1, c2, &lanes)))
    return rc;
  PPS_CUDA(cudaEventRecord(s->ev1, s->stream));
  if ((rc = finish_timing(s, device_ms))) return rc;
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  s->t += (uint32_t)maxiters;
  return PPS_OK;
}

int pps_get_gbest(pps_swarm* s, float* u, float* cost, int64_t* idx) {
  if (!s) return set_error(PPS_EINVAL, "swarm is NULL");
  if (!s->initialized) return set_error(PPS_EINVAL, "swarm is not initialised");
  int rc = use_device(s);
  if (rc) return rc;
  IterState st;
  PPS_CUDA(cudaMemcpyAsync(&st, s->dv.st, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
  if (u) PPS_CUDA(cudaMemcpyAsync(u, s->dv.g, sizeof(float) * s->dv.dim, cudaMemcpyDeviceToHost, s->stream));
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  if (cost) *cost = st.gcost;
  if (idx) *idx = (int64_t)st.gidx;
  return PPS_OK;
}

static int field_ptr(pps_swarm* s, int32_t field, float** dev, int* rows) {
  switch (field) {
    case PPS_FIELD_POSITION: *dev = s->dv.X; *rows = s->dv.dim; return PPS_OK;
    case PPS_FIELD_VELOCITY: *dev = s->dv.V; *rows = s->dv.dim; return PPS_OK;
    case PPS_FIELD_PBEST: *dev = s->dv.P; *rows = s->dv.dim; return PPS_OK;
    case PPS_FIELD_PCOST: *dev = s->dv.pcost; *rows = 1; return PPS_OK;
    case PPS_FIELD_COST: *dev = s->dv.cost; *rows = 1; return PPS_OK;
    case PPS_FIELD_LOCAL_X:
    case PPS_FIELD_LOCAL_F:
    case PPS_FIELD_LOCAL_ITERS:
      return local_field(s, field, dev, rows);
    default: return set_error(PPS_EINVAL, "unknown field %d", field);
  }
}

}  // extern "C"

namespace pps {

// Device -> pageable host copies of swarm state (hundreds of MB for the
// particle positions of a large swarm) go through two pinned staging
// buffers of kStageBytes, allocated once per device: the copy engine fills
// one while the host copies the other out, instead of the driver's slower
// staging of a pageable destination.
constexpr size_t kStageBytes = (size_t)32 << 20;

struct HostStage {
  std::mutex mu;
  char* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool ready = false;
};

static HostStage& host_stage(int device) {
  static HostStage stages[64];
  return stages[device & 63];
}

// rows x row_bytes from dev (pitch src_pitch bytes) to the contiguous host
// array out, on stream
int copy_rows_to_host(int device, cudaStream_t stream, char* out, const char* dev, size_t src_pitch,
                      size_t row_bytes, size_t rows) {
  const size_t total = row_bytes * rows;
  if (total < ((size_t)4 << 20) || device < 0 || device >= 64) {
    PPS_CUDA(cudaMemcpy2DAsync(out, row_bytes, dev, src_pitch, row_bytes, rows, cudaMemcpyDeviceToHost, stream));
    PPS_CUDA(cudaStreamSynchronize(stream));
    return PPS_OK;
  }
  HostStage& hs = host_stage(device);
  std::lock_guard<std::mutex> lock(hs.mu);
  if (!hs.ready) {
    for (int k = 0; k < 2; ++k) {
      PPS_CUDA(cudaMallocHost(&hs.buf[k], kStageBytes));
      PPS_CUDA(cudaEventCreateWithFlags(&hs.ev[k], cudaEventDisableTiming));
    }
    hs.ready = true;
  }
  // pieces: whole rows when a row fits a buffer, else segments of one row
  struct Piece {
    size_t src_off, dst_off, rows, bytes;  // bytes per row of the piece
  };
  std::vector<Piece> pieces;
  if (row_bytes <= kStageBytes) {
    const size_t per = kStageBytes / row_bytes;
    for (size_t r = 0; r < rows; r += per) {
      const size_t nr = (rows - r) < per ? (rows - r) : per;
      pieces.push_back({r * src_pitch, r * row_bytes, nr, row_bytes});
    }
  } else {
    for (size_t r = 0; r < rows; ++r)
      for (size_t c = 0; c < row_bytes; c += kStageBytes) {
        const size_t nb = (row_bytes - c) < kStageBytes ? (row_bytes - c) : kStageBytes;
        pieces.push_back({r * src_pitch + c, r * row_bytes + c, 1, nb});
      }
  }
  for (size_t k = 0; k <= pieces.size(); ++k) {
    if (k < pieces.size()) {  // copy engine: piece k into buffer k % 2
      const Piece& p = pieces[k];
      PPS_CUDA(cudaMemcpy2DAsync(hs.buf[k & 1], p.bytes, dev + p.src_off, src_pitch, p.bytes, p.rows,
                                 cudaMemcpyDeviceToHost, stream));
      PPS_CUDA(cudaEventRecord(hs.ev[k & 1], stream));
    }
    if (k >= 1) {  // host: piece k - 1 out of its buffer while piece k is in flight
      const Piece& p = pieces[k - 1];
      PPS_CUDA(cudaEventSynchronize(hs.ev[(k - 1) & 1]));
      if (p.rows == 1 || p.bytes == row_bytes) {
        memcpy(out + p.dst_off, hs.buf[(k - 1) & 1], p.bytes * p.rows);
      } else {
        for (size_t r = 0; r < p.rows; ++r) memcpy(out + p.dst_off + r * row_bytes, hs.buf[(k - 1) & 1] + r * p.bytes, p.bytes);
      }
    }
  }
  return PPS_OK;
}

}  // namespace pps

extern "C" {

int pps_get_state(pps_swarm* s, int32_t field, float* out) {
  if (!s || !out) return set_error(PPS_EINVAL, "NULL argument");
  int rc = use_device(s);
  if (rc) return rc;
  float* dev = nullptr;
  int rows = 0;
  if ((rc = field_ptr(s, field, &dev, &rows))) return rc;
  const size_t w = sizeof(float) * (size_t)s->dv.n;
  return copy_rows_to_host(s->device, s->stream, reinterpret_cast<char*>(out), reinterpret_cast<const char*>(dev),
                           sizeof(float) * (size_t)s->dv.npad, w, (size_t)rows);
}

int pps_set_state(pps_swarm* s, int32_t field, const float* in) {
  if (!s || !in) return set_error(PPS_EINVAL, "NULL argument");
  if (field > PPS_FIELD_COST) return set_error(PPS_EINVAL, "field %d is read-only", field);
  int rc = use_device(s);
  if (rc) return rc;
  float* dev = nullptr;
  int rows = 0;
  if ((rc = field_ptr(s, field, &dev, &rows))) return rc;
  const size_t w = sizeof(float) * (size_t)s->dv.n;
  PPS_CUDA(cudaMemcpy2DAsync(dev, sizeof(float) * (size_t)s->dv.npad, in, w, w, rows,
                             cudaMemcpyHostToDevice, s->stream));
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  return PPS_OK;
}

// A device snapshot of a state field, as the reference's sol.original =
// get_pos.(particles) is a new device array (src/solve.jl:51-56): the
// swarm may be re-run or destroyed while the snapshot lives.
struct pps_field_copy {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ready = nullptr;
  float* dev = nullptr;
  int rows = 0;
  int64_t n = 0;
};

int pps_field_copy_create(pps_swarm* s, int32_t field, pps_field_copy** out) {
  if (!s || !out) return set_error(PPS_EINVAL, "NULL argument");
  int rc = use_device(s);
  if (rc) return rc;
  float* src = nullptr;
  int rows = 0;
  if ((rc = field_ptr(s, field, &src, &rows))) return rc;
  pps_field_copy* c = new (std::nothrow) pps_field_copy();
  if (!c) return set_error(PPS_ENOMEM, "host allocation failed");
  c->device = s->device;
  c->rows = rows;
  c->n = s->dv.n;
  const size_t w = sizeof(float) * (size_t)s->dv.n;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ready, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&c->dev), w * (size_t)rows, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(c->dev, w, src, sizeof(float) * (size_t)s->dv.npad, w, (size_t)rows,
                          cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ready, s->stream);
  if (e != cudaSuccess) {
    pps_field_copy_destroy(c);
    return cuda_error(e, "pps_field_copy_create");
  }
  *out = c;
  return PPS_OK;
}

int pps_field_copy_read(pps_field_copy* c, float* out) {
  if (!c || !out) return set_error(PPS_EINVAL, "NULL argument");
  PPS_CUDA(cudaSetDevice(c->device));
  PPS_CUDA(cudaStreamWaitEvent(c->stream, c->ready, 0));
  const size_t w = sizeof(float) * (size_t)c->n;
  return copy_rows_to_host(c->device, c->stream, reinterpret_cast<char*>(out), reinterpret_cast<const char*>(c->dev),
                           w, w, (size_t)c->rows);
}

int pps_field_copy_destroy(pps_field_copy* c) {
  if (!c) return PPS_OK;
  cudaSetDevice(c->device);
  if (c->dev) {
    if (c->stream) cudaStreamWaitEvent(c->stream, c->ready, 0);
    cudaFreeAsync(c->dev, c->stream);
  }
  if (c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  if (c->ready) cudaEventDestroy(c->ready);
  delete c;
  return PPS_OK;
}

int pps_eval_objective(const pps_problem* prob, int64_t npoints, const float* x, float* f) {
  int rc = check_problem(prob);
  if (rc) return rc;
  if (npoints < 0 || (npoints > 0 && (!x || !f))) return set_error(PPS_EINVAL, "bad points");
  if (npoints == 0) return PPS_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_error(PPS_ENODEV, "no CUDA device");
  const int D = prob->dim;
  float* dx = nullptr;
  cudaStream_t st = nullptr;
  PPS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  // device layout x[d * stride + i]; the stride is padded to 64 points
  const int64_t stride = (int64_t)align_up((size_t)npoints, 64);
  const size_t bx = sizeof(float) * (size_t)D * (size_t)stride;
  cudaError_t e = cudaMallocAsync(&dx, bx + sizeof(float) * (size_t)stride, st);
  if (e != cudaSuccess) {
    cudaStreamDestroy(st);
    return cuda_error(e, "cudaMallocAsync");
  }
  float* df = dx + (size_t)D * (size_t)stride;
  ObjParams op = make_params(prob);
  ObjData od{};
  float* ddata = nullptr;
  rc = PPS_OK;
  if (is_ode(prob->objective) || (is_user(prob->objective) && prob->ndata > 0)) {
    if ((e = cudaMallocAsync(&ddata, sizeof(float) * (size_t)prob->ndata, st)) != cudaSuccess) rc = cuda_error(e, "cudaMallocAsync");
    if (!rc && (e = cudaMemcpyAsync(ddata, prob->data, sizeof(float) * (size_t)prob->ndata, cudaMemcpyHostToDevice, st)) != cudaSuccess)
      rc = cuda_error(e, "cudaMemcpy");
    od.data = ddata;
    od.ndata = prob->ndata;
  }
  uint8_t* da = nullptr;  // MLP: packed samples followed by the status word
  std::vector<uint8_t> packed;
  if (!rc && prob->objective == kMlp) {
    const int S = (int)(prob->ndata / 17);
    packed.resize(mlp_a_bytes(S));
    mlp_pack_a(prob->data, S, packed.data());
    if ((e = cudaMallocAsync(&ddata, sizeof(float) * (size_t)prob->ndata, st)) != cudaSuccess ||
        (e = cudaMallocAsync(&da, packed.size() + 256, st)) != cudaSuccess)
      rc = cuda_error(e, "cudaMallocAsync");
    if (!rc && ((e = cudaMemcpyAsync(ddata, prob->data, sizeof(float) * (size_t)prob->ndata, cudaMemcpyHostToDevice,
                                     st)) != cudaSuccess ||
                (e = cudaMemcpyAsync(da, packed.data(), packed.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
                (e = cudaMemsetAsync(da + packed.size(), 0, 256, st)) != cudaSuccess))
      rc = cuda_error(e, "cudaMemcpy");
    od.data = ddata;
    od.ndata = prob->ndata;
  }
  if (!rc && (e = cudaMemsetAsync(dx, 0, bx, st)) != cudaSuccess) rc = cuda_error(e, "cudaMemset");
  if (!rc && (e = cudaMemcpy2DAsync(dx, sizeof(float) * (size_t)stride, x, sizeof(float) * (size_t)npoints,
                                    sizeof(float) * (size_t)npoints, (size_t)D, cudaMemcpyHostToDevice, st)) !=
                 cudaSuccess)
    rc = cuda_error(e, "cudaMemcpy");
  unsigned int status = 0;
  if (!rc) {
    if (prob->objective == kMlp) {
      unsigned int* dstatus = reinterpret_cast<unsigned int*>(da + packed.size());
      rc = launch_mlp_points(ddata, prob->ndata, da, dx, npoints, stride, df, dstatus, st);
      if (!rc && (e = cudaMemcpyAsync(&status, dstatus, sizeof(status), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        rc = cuda_error(e, "cudaMemcpy");
    } else if (is_ode(prob->objective)) {
      rc = launch_eval_ode(op, od, prob->objective, dx, npoints, stride, df, st);
    } else {
      rc = launch_eval(op, od, prob->objective, dx, npoints, stride, df, st);
    }
  }
  if (!rc && (e = cudaMemcpyAsync(f, df, sizeof(float) * npoints, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    rc = cuda_error(e, "cudaMemcpy");
  cudaFreeAsync(dx, st);
  if (ddata) cudaFreeAsync(ddata, st);
  if (da) cudaFreeAsync(da, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess && !rc) rc = cuda_error(e, "cudaStreamSynchronize");
  cudaStreamDestroy(st);
  if (!rc && (status & 2u)) rc = set_error(PPS_ETIMEOUT, "the MLP tensor-core kernel timed out waiting for an MMA");
  return rc;
}

}  // extern "C"

namespace pps {

int swarm_enqueue_init(pps_swarm* s) {
  int sampler = PPS_SAMPLER_UNIFORM;
  bool all_inf = true;
  for (int d = 0; d < s->dv.dim; ++d)
    if (!(std::isinf(s->host_lb[d]) && std::isinf(s->host_ub[d]))) all_inf = false;
  if (all_inf) sampler = PPS_SAMPLER_UNBOUNDED;
  for (int d = 0; sampler == PPS_SAMPLER_UNIFORM && d < s->dv.dim; ++d)
    if (!std::isfinite(s->host_lb[d]) || !std::isfinite(s->host_ub[d]))
      return set_error(PPS_EINVAL, "uniform sampler needs finite bounds (dim %d)", d);
  int rc;
  if ((rc = launch_set_iter(s, 0u, 0.7298f, 1.0f))) return rc;
  if ((rc = is_ode(s->objective) ? launch_init_ode(s, sampler, s->u0_dev) : launch_init(s, sampler, s->u0_dev)))
    return rc;
  if (s->objective == kMlp && (rc = launch_mlp_init_eval(s))) return rc;
  s->t = 0;
  s->initialized = 1;
  return PPS_OK;
}

int swarm_enqueue_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2) {
  int rc = check_run(s, maxiters, w, wdamp, c1, c2);
  if (rc) return rc;
  if ((rc = launch_set_iter(s, s->t, w, wdamp))) return rc;
  if ((rc = run_steps(s, maxiters, c1, c2, s->flags & PPS_FLAG_GBEST_FROM_POSITION))) return rc;
  s->t += (uint32_t)maxiters;
  return PPS_OK;
}

}  // namespace pps
