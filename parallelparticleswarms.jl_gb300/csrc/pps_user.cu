// pps_user.cu -- user objectives: CUDA C source compiled at run time.
//
// The reference compiles any isbits Julia closure into its kernels
// (cost = prob.f(x, p), src/kernels.jl:33; the ODE and hybrid paths alike).
// A C ABI cannot take a closure, so a user objective arrives as source text:
// pps_objective_register() compiles it with NVRTC, together with the
// library's own init / step / evaluation kernels (pps_user_kernels.cuh and
// the device headers, embedded in the library at build time), into a cubin
// for the current device, and returns an objective id to put in
// pps_problem.objective.  The cubin is loaded through the CUDA runtime's
// library API on first use and launched with cudaLaunchKernel, so the
// graph-replayed run loop, the server's own-swarm path and the point
// evaluation treat it like a registered objective.
//
// NVRTC is opened with dlopen on the first registration: the library loads
// and every registered objective runs on a machine without it, and
// registration then fails with PPS_ENOTSUP.
#include <dlfcn.h>
#include <nvrtc.h>

#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "pps_internal.h"
#include "pps_local.cuh"
#include "pps_rtc_sources.inc"  // kRtcHeaderNames[], kRtcHeaderTexts[], kRtcHeaderCount (generated)

namespace pps {
namespace {

struct NvrtcApi {
  void* handle = nullptr;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) error_string = nullptr;
};

const NvrtcApi& nvrtc() {
  static NvrtcApi api = [] {
    NvrtcApi a;
    std::vector<std::string> cand = {"libnvrtc.so.13", "libnvrtc.so"};
    for (const char* env : {"CUDA_HOME", "CUDA_PATH"}) {
      const char* v = getenv(env);
      if (v && *v) cand.push_back(std::string(v) + "/lib64/libnvrtc.so.13");
    }
    cand.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    for (const auto& c : cand) {
      a.handle = dlopen(c.c_str(), RTLD_NOW | RTLD_LOCAL);
      if (a.handle) break;
    }
    if (!a.handle) {
      a.why = "libnvrtc.so.13 not found (set CUDA_HOME or LD_LIBRARY_PATH)";
      return a;
    }
    bool ok = true;
    auto sym = [&](auto& fn, const char* name) {
      fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(a.handle, name));
      ok = ok && fn != nullptr;
    };
    sym(a.create, "nvrtcCreateProgram");
    sym(a.compile, "nvrtcCompileProgram");
    sym(a.log_size, "nvrtcGetProgramLogSize");
    sym(a.log, "nvrtcGetProgramLog");
    sym(a.cubin_size, "nvrtcGetCUBINSize");
    sym(a.cubin, "nvrtcGetCUBIN");
    sym(a.destroy, "nvrtcDestroyProgram");
    sym(a.error_string, "nvrtcGetErrorString");
    if (!ok) {
      a.why = "libnvrtc lacks an entry point";
      dlclose(a.handle);
      a.handle = nullptr;
    }
    return a;
  }();
  return api;
}

struct UserObjective {
  std::string source;
  std::vector<char> cubin;
  int arch = 0;  // compute capability compiled for (major * 10 + minor)
  std::mutex load_mu;
  std::atomic<bool> loaded{false};
  cudaLibrary_t lib = nullptr;
  cudaKernel_t k_init = nullptr, k_eval = nullptr;
  cudaKernel_t k_step[3] = {};  // 1, 2, 4 particles per thread
  cudaKernel_t k_step_cons = nullptr;
  cudaKernel_t k_async = nullptr;
  // HybridPSO's local stage, when the source has a gradient (else NULL)
  cudaKernel_t k_lbfgs16 = nullptr, k_lbfgs64 = nullptr, k_broyden16 = nullptr;
};

constexpr int kMaxUser = 4096;
std::atomic<UserObjective*> g_table[kMaxUser];
std::atomic<int> g_count{0};
std::mutex g_register_mu;

UserObjective* lookup(int objective) {
  const int k = objective - PPS_OBJ_USER_BASE;
  if (k < 0 || k >= g_count.load(std::memory_order_acquire)) return nullptr;
  return g_table[k].load(std::memory_order_acquire);
}

// compute capability of the current device; 10.3 (GB300) without one
int current_arch() {
  int count = 0, dev = 0, major = 0, minor = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    return 103;
  }
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) ||
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev)) {
    cudaGetLastError();
    return 103;
  }
  return major * 10 + minor;
}

int compile(const std::string& user, int arch, std::vector<char>* out) {
  const NvrtcApi& api = nvrtc();
  if (!api.handle) return set_error(PPS_ENOTSUP, "user objectives need NVRTC: %s", api.why.c_str());
  const std::string src = "#include \"pps_user_prelude.cuh\"\n#line 1 \"objective\"\n" + user +
                          "\n#line 1 \"pps_user_kernels.cuh\"\n#include \"pps_user_kernels.cuh\"\n";
  nvrtcProgram prog = nullptr;
  nvrtcResult r = api.create(&prog, src.c_str(), "pps_user.cu", kRtcHeaderCount, kRtcHeaderTexts, kRtcHeaderNames);
  if (r != NVRTC_SUCCESS) return set_error(PPS_ECUDA, "nvrtcCreateProgram: %s", api.error_string(r));
  // sm_103a for GB300 (the architecture-specific target the library is built
  // for); the plain target of any other device
  const std::string target =
      "--gpu-architecture=sm_" + std::to_string(arch) + (arch >= 90 ? "a" : "");
  // PPS_USER_MINBLOCKS=N overrides the resident blocks the step kernel is
  // compiled for (register cap); the default is the header's
  std::string minblocks;
  if (const char* mb = getenv("PPS_USER_MINBLOCKS")) {
    const int v = atoi(mb);
    if (v >= 1 && v <= 8) minblocks = "-DPPS_USER_MINBLOCKS=" + std::to_string(v);
  }
  std::vector<const char*> opts = {target.c_str(), "-std=c++17", "--fmad=false", "-lineinfo"};
  if (!minblocks.empty()) opts.push_back(minblocks.c_str());
  r = api.compile(prog, (int)opts.size(), opts.data());
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    std::string log;
    if (api.log_size(prog, &n) == NVRTC_SUCCESS && n > 1) {
      log.resize(n);
      api.log(prog, &log[0]);
    }
    api.destroy(&prog);
    return set_error(PPS_EINVAL, "the objective source does not compile (%s):\n%s", api.error_string(r),
                     log.c_str());
  }
  size_t n = 0;
  if ((r = api.cubin_size(prog, &n)) != NVRTC_SUCCESS || n == 0) {
    api.destroy(&prog);
    return set_error(PPS_ECUDA, "nvrtcGetCUBINSize: %s", api.error_string(r));
  }
  out->resize(n);
  r = api.cubin(prog, out->data());
  api.destroy(&prog);
  if (r != NVRTC_SUCCESS) return set_error(PPS_ECUDA, "nvrtcGetCUBIN: %s", api.error_string(r));
  return PPS_OK;
}

int ensure_loaded(UserObjective* u) {
  if (u->loaded.load(std::memory_order_acquire)) return PPS_OK;
  std::lock_guard<std::mutex> lk(u->load_mu);
  if (u->loaded.load(std::memory_order_relaxed)) return PPS_OK;
  PPS_CUDA(cudaLibraryLoadData(&u->lib, u->cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_init, u->lib, "pps_user_init"));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_step[0], u->lib, "pps_user_step1"));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_step[1], u->lib, "pps_user_step2"));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_step[2], u->lib, "pps_user_step4"));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_step_cons, u->lib, "pps_user_step_cons"));
  PPS_CUDA(cudaLibraryGetKernel(&u->k_async, u->lib, "pps_user_async"));
  if (cudaLibraryGetKernel(&u->k_lbfgs16, u->lib, "pps_user_lbfgs16") != cudaSuccess) {
    cudaGetLastError();  // no gradient in the source: no local stage
    u->k_lbfgs16 = nullptr;
  } else {
    PPS_CUDA(cudaLibraryGetKernel(&u->k_lbfgs64, u->lib, "pps_user_lbfgs64"));
    PPS_CUDA(cudaLibraryGetKernel(&u->k_broyden16, u->lib, "pps_user_broyden16"));
  }
  PPS_CUDA(cudaLibraryGetKernel(&u->k_eval, u->lib, "pps_user_eval"));
  u->loaded.store(true, std::memory_order_release);
  return PPS_OK;
}

UserObjective* loaded_or_error(int objective, int* rc) {
  UserObjective* u = lookup(objective);
  if (!u) {
    *rc = set_error(PPS_EINVAL, "objective %d is not a registered user objective", objective);
    return nullptr;
  }
  *rc = ensure_loaded(u);
  return *rc ? nullptr : u;
}

constexpr int kUserThreads = 256;

// particles per thread of the unconstrained step kernel; PPS_USER_PPT=1|2|4
// overrides the default
int user_step_ppt() {
  static const int ppt = [] {
    const char* e = getenv("PPS_USER_PPT");
    const int v = e ? atoi(e) : 2;
    return (v == 1 || v == 2 || v == 4) ? v : 2;
  }();
  return ppt;
}

}  // namespace

bool is_user(int objective) { return lookup(objective) != nullptr; }

int user_prepare(pps_swarm* s) {
  int rc;
  UserObjective* u = loaded_or_error(s->objective, &rc);
  if (!u) return rc;
  if (s->user_grid > 0) return PPS_OK;
  int ppt = 1;
  const void* k = reinterpret_cast<const void*>(u->k_step_cons);
  if (s->dv.ncons == 0) {
    ppt = user_step_ppt();
    k = reinterpret_cast<const void*>(u->k_step[ppt == 1 ? 0 : (ppt == 2 ? 1 : 2)]);
  }
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  // g, lb, ub in dynamic shared memory: beyond 40 kB (3414 dims) the kernel
  // opts in to more than the default 48 kB of static + dynamic
  if (smem > ((size_t)40 << 10))
    PPS_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kUserThreads, smem));
  if (per_sm < 1) return set_error(PPS_EINVAL, "the objective's step kernel cannot be resident (dim %d)", s->dv.dim);
  const int64_t groups = (s->dv.n + ppt - 1) / ppt;
  const int64_t blocks = (groups + kUserThreads - 1) / kUserThreads;
  const int64_t resident = (int64_t)per_sm * s->sm_count;
  s->user_step_kernel = k;
  s->user_grid = (int)(blocks < resident ? blocks : resident);
  return PPS_OK;
}

int launch_user_init(pps_swarm* s, int sampler, const float* u0_dev) {
  int rc;
  UserObjective* u = loaded_or_error(s->objective, &rc);
  if (!u) return rc;
  const int64_t blocks = (s->dv.npad + kUserThreads - 1) / kUserThreads;
  const float* data = s->od.data;
  long long ndata = (long long)s->od.ndata;
  unsigned long long seed = s->seed;
  void* args[] = {&s->dv, &s->op, &data, &ndata, &seed, &sampler, &u0_dev};
  PPS_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(u->k_init), dim3((unsigned)blocks), dim3(kUserThreads), args,
                            0, s->stream));
  return PPS_OK;
}

int launch_user_step(pps_swarm* s, float c1, float c2) {
  int rc;
  if ((rc = user_prepare(s))) return rc;
  PhiloxKeys keys = philox_round_keys(s->seed);
  const float* data = s->od.data;
  long long ndata = (long long)s->od.ndata;
  int from_pos = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  void* args[] = {&s->dv, &s->op, &data, &ndata, &keys, &c1, &c2, &from_pos};
  PPS_CUDA(cudaLaunchKernel(s->user_step_kernel, dim3((unsigned)s->user_grid), dim3(kUserThreads), args,
                            3 * sizeof(float) * (size_t)s->dv.dim, s->stream));
  return PPS_OK;
}

int launch_user_async(pps_swarm* s, int iters, float c1, float c2) {
  int rc;
  UserObjective* u = loaded_or_error(s->objective, &rc);
  if (!u) return rc;
  const size_t smem = 3 * sizeof(float) * (size_t)s->dv.dim;
  if (smem > ((size_t)40 << 10))
    PPS_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(u->k_async),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(u->k_async),
                                                         kUserThreads, smem));
  if (per_sm < 1) return set_error(PPS_EINVAL, "the objective's async kernel cannot be resident (dim %d)", s->dv.dim);
  const int64_t blocks = (s->dv.n + kUserThreads - 1) / kUserThreads;
  const int64_t resident = (int64_t)per_sm * s->sm_count;
  const unsigned grid = (unsigned)(blocks < resident ? blocks : resident);
  PhiloxKeys keys = philox_round_keys(s->seed);
  const float* data = s->od.data;
  long long ndata = (long long)s->od.ndata;
  void* args[] = {&s->dv, &s->op, &data, &ndata, &keys, &iters, &c1, &c2};
  PPS_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(u->k_async), dim3(grid), dim3(kUserThreads), args, smem,
                            s->stream));
  return PPS_OK;
}

int launch_user_local(pps_swarm* s, int kind, const float* x0, const LocalOpts& o, float* xout, float* fout,
                      float* itout) {
  int rc;
  UserObjective* u = loaded_or_error(s->objective, &rc);
  if (!u) return rc;
  if (!u->k_lbfgs16)
    return set_error(PPS_ENOTSUP, "the HybridPSO local stage needs a gradient: define PPS_HAS_GRADIENT and "
                                  "pps_gradient in the objective's source");
  const int D = s->dv.dim;
  const int64_t n = s->dv.n;
  int64_t ld = s->dv.npad, nn = n;
  ObjParams op = s->op;
  LocalOpts oo = o;
  const float *lb = s->dv.lb, *ub = s->dv.ub;
  void* args[] = {&x0, &ld, &nn, &op, &lb, &ub, &oo, &xout, &fout, &itout};
  const void* k;
  int threads;
  size_t smem = 0;
  if (kind == 1) {
    if (D > 16) return set_error(PPS_ENOTSUP, "the Broyden local stage supports dim <= 16 (got %d)", D);
    k = reinterpret_cast<const void*>(u->k_broyden16);
    threads = kBroydenThreads;
    smem = sizeof(float) * 16 * 16 * kBroydenThreads;
  } else if (D <= 16) {
    k = reinterpret_cast<const void*>(u->k_lbfgs16);
    threads = kLbfgsThreads;
    smem = sizeof(float) * lbfgs_hist_floats(o.history, 16) * kLbfgsThreads;
  } else {
    k = reinterpret_cast<const void*>(u->k_lbfgs64);
    threads = 128;
  }
  if (smem > ((size_t)48 << 10))
    PPS_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned blocks = (unsigned)((n + threads - 1) / threads);
  PPS_CUDA(cudaLaunchKernel(k, dim3(blocks), dim3(threads), args, smem, s->stream));
  return PPS_OK;
}

int launch_user_eval(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                     int64_t stride, float* f, cudaStream_t stream) {
  int rc;
  UserObjective* u = loaded_or_error(objective, &rc);
  if (!u) return rc;
  ObjParams p = op;
  const float* data = od.data;
  long long ndata = (long long)od.ndata, n = (long long)npts, ld = (long long)stride;
  void* args[] = {&p, &data, &ndata, &x, &n, &ld, &f};
  const int64_t blocks = (npts + kUserThreads - 1) / kUserThreads;
  PPS_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(u->k_eval), dim3((unsigned)blocks), dim3(kUserThreads), args,
                            0, stream));
  return PPS_OK;
}

}  // namespace pps

extern "C" int pps_objective_register(const char* source, int32_t* objective) {
  using namespace pps;
  if (!source || !objective) return set_error(PPS_EINVAL, "NULL argument");
  const size_t len = strnlen(source, (size_t)1 << 20);
  if (len == 0 || len >= ((size_t)1 << 20)) return set_error(PPS_EINVAL, "objective source must be 1 B .. 1 MiB");
  const std::string text(source, len);
  const int arch = current_arch();
  {
    const int count = g_count.load(std::memory_order_acquire);
    for (int k = 0; k < count; ++k) {
      UserObjective* u = g_table[k].load(std::memory_order_acquire);
      if (u->arch == arch && u->source == text) {
        *objective = PPS_OBJ_USER_BASE + k;
        return PPS_OK;
      }
    }
  }
  auto u = std::make_unique<UserObjective>();
  u->source = text;
  u->arch = arch;
  int rc = compile(text, arch, &u->cubin);  // outside the lock: NVRTC takes a while
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_register_mu);
  const int count = g_count.load(std::memory_order_relaxed);
  for (int k = 0; k < count; ++k) {  // registered by another thread meanwhile
    UserObjective* v = g_table[k].load(std::memory_order_relaxed);
    if (v->arch == arch && v->source == text) {
      *objective = PPS_OBJ_USER_BASE + k;
      return PPS_OK;
    }
  }
  if (count >= kMaxUser) return set_error(PPS_ENOMEM, "at most %d user objectives per process", kMaxUser);
  g_table[count].store(u.release(), std::memory_order_release);
  g_count.store(count + 1, std::memory_order_release);
  *objective = PPS_OBJ_USER_BASE + count;
  return PPS_OK;
}
