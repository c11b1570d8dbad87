// pps_internal.h -- host-side structures shared by the translation units of
// libpps_cuda.so.  Not part of the public C ABI (include/pps.h is).
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/pps.h"
#include "pps_device.cuh"
#include "pps_state.cuh"

namespace pps {

static_assert(kSamplerUniform == PPS_SAMPLER_UNIFORM && kSamplerUnbounded == PPS_SAMPLER_UNBOUNDED &&
                  kSamplerLhs == PPS_SAMPLER_LHS,
              "device sampler ids follow include/pps.h");

struct ObjData {
  const float* data;  // device copy of the objective's data (ODE obs, MLP set)
  int64_t ndata;
};

}  // namespace pps

struct pps_swarm {
  int device = 0;
  cudaStream_t stream = nullptr;
  void* block = nullptr;  // the single device allocation
  size_t bytes = 0;
  pps::SwarmDev dv{};
  pps::ObjParams op{};
  pps::ObjData od{};
  float* data_dev = nullptr;
  int objective = 0;
  uint64_t seed = 0;
  uint32_t flags = 0;
  uint32_t t = 0;  // host mirror of the iteration counter
  int initialized = 0;
  float* host_lb = nullptr;
  float* host_ub = nullptr;
  float* host_u0 = nullptr;
  float* u0_dev = nullptr;
  cudaGraphExec_t graph = nullptr;  // captured chunk of step launches
  int graph_len = 0;
  int graph_async_lanes = 0;  // run flags the graph was captured with
  float graph_c1 = 0.0f, graph_c2 = 0.0f;
  int sm_count = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void* local_block = nullptr;  // HybridPSO local-stage results (allocated on first use)
  int local_valid = 0;
  void* mlp_a_dev = nullptr;  // MLP objective: the samples as bf16 tensor-core tiles
  bool owns_memory = true;    // false: device block and stream belong to a server
  int user_grid = 0;          // user objective: blocks of its step kernel (0: not resolved yet)
  const void* user_step_kernel = nullptr;  // user objective: the step kernel variant in use
  int shard = 0;              // 1: a particle-range shard (pps_shard_create); dv.xrec is its exchange record
  const unsigned char* shard_records = nullptr;  // shard: every shard's record after the exchange
  int shard_nrecords = 0;
  int bounded_waits = 0;      // 1: a kernel with bounded mbarrier waits ran (a timeout sets IterState::status)
};

namespace pps {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

#define PPS_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return pps::cuda_error(e_, #call); \
  } while (0)

// kernel launchers (pps_sync.cu, pps_async.cu)
int launch_init(pps_swarm* s, int sampler, const float* u0_dev);
int launch_set_iter(pps_swarm* s, uint32_t t, float w, float wdamp);
int launch_sync_step(pps_swarm* s, float c1, float c2);
int launch_materialize(pps_swarm* s);
int launch_async(pps_swarm* s, int iters, float c1, float c2, int* lanes_out);
int launch_eval(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                int64_t stride, float* f, cudaStream_t stream);
int async_lanes(int dim, int* slice);
int sync_grid(pps_swarm* s);
// the TMA-staged step (pps_sync_bulk.cu): resident blocks per SM where it
// applies (0 where it does not), resolved outside any stream capture; the
// launch, *taken false where the caller launches k_sync_step instead
int sync_bulk_prepare(pps_swarm* s, int* blocks_per_sm);
// PPS_ETIMEOUT if a bounded wait of a kernel of this swarm gave up (reads
// IterState::status after the swarm's stream is idle), else PPS_OK
int check_device_status(pps_swarm* s);
int launch_sync_step_bulk(pps_swarm* s, float c1, float c2, bool* taken);
int local_field(pps_swarm* s, int32_t field, float** dev, int* rows);
// ODE-fit objectives (pps_ode.cu)
int ode_check(const pps_problem* prob);
int launch_init_ode(pps_swarm* s, int sampler, const float* u0_dev);
int launch_sync_step_ode(pps_swarm* s, float c1, float c2);
int launch_eval_ode(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                    int64_t stride, float* f, cudaStream_t stream);
inline bool is_ode(int objective) { return objective == kLvFit || objective == kFhnFit; }
// MLP-regression objective on the tensor cores (pps_mlp.cu): one kernel per
// iteration moves the particles, evaluates them, updates the personal bests
// and publishes the argmin
int mlp_check(const pps_problem* prob);
size_t mlp_a_bytes(int samples);
void mlp_pack_a(const float* X, int samples, uint8_t* out);
int launch_mlp_init_eval(pps_swarm* s);
int launch_mlp_step(pps_swarm* s, float c1, float c2);
// swarms over caller-owned memory and streams (pps_api.cu), for the server:
// nothing below synchronises
int swarm_check(const pps_problem* prob, int64_t n);
size_t swarm_device_bytes(const pps_problem* prob, int64_t n);
int swarm_attach(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags, void* mem, cudaStream_t stream,
                 pps_swarm** out);
void swarm_detach(pps_swarm* s);
int swarm_enqueue_init(pps_swarm* s);
int swarm_enqueue_run(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2);
// gbest (dim floats), its cost and index into mail, then done = 1, visible to the host
int launch_publish_result(pps_swarm* s, float* mail, int* done);
// rows x row_bytes of device memory (pitch src_pitch) to a pageable host
// array through pinned staging buffers, on stream (pps_api.cu)
int copy_rows_to_host(int device, cudaStream_t stream, char* out, const char* dev, size_t src_pitch,
                      size_t row_bytes, size_t rows);
// pps_swarm_create / pps_shard_create (pps_api.cu)
int swarm_create(const pps_problem* prob, int64_t n, uint64_t seed, uint32_t flags, int64_t first, int64_t nglobal,
                 pps_swarm** out);
// argmin of pcost into the global best (pps_noalloc.cu)
int launch_select_gbest(pps_swarm* s);
// user objectives compiled at run time (pps_user.cu)
bool is_user(int objective);
int user_prepare(pps_swarm* s);  // loads the kernels and sizes the grid; call outside stream capture
int launch_user_init(pps_swarm* s, int sampler, const float* u0_dev);
int launch_user_step(pps_swarm* s, float c1, float c2);
int launch_user_async(pps_swarm* s, int iters, float c1, float c2);
int launch_user_eval(const ObjParams& op, const ObjData& od, int objective, const float* x, int64_t npts,
                     int64_t stride, float* f, cudaStream_t stream);
int launch_mlp_points(const float* data_dev, int64_t ndata, const uint8_t* a_dev, const float* x, int64_t npts,
                      int64_t stride, float* f, unsigned int* status, cudaStream_t stream);

}  // namespace pps
