// pps_shard.cu -- one swarm split into particle-range shards, with one
// global-best exchange per iteration.
//
// The synchronous loop couples the particles only through its global best:
// each iteration ends with block bests and their minimum
// (src/kernels.jl:156-171, src/lowerlevel_solve.jl:23-33).  So a swarm shards
// by particle ranges: shard r holds particles first_r .. first_r + count_r - 1
// and steps them exactly as the whole swarm would (the kernels take the
// particle's global index for its random stream, its argmin key and the
// penalty's index).  The one exchange per iteration:
//
//   1. each shard's step (or init) writes an exchange record instead of
//      publishing a global best: its best particle's argmin key (orderable
//      cost << 32 | global index), cost and vector (16 + 4 dim bytes);
//   2. the caller gathers every shard's record (an all-gather over ranks,
//      e.g. ncclAllGather of the fixed-size records, or plain device copies
//      when the shards share a process);
//   3. pps_shard_apply makes the record with the lowest key the global best
//      of every shard: the lowest cost, ties to the lowest global index, as
//      the whole swarm's argmin.
//
// Steps 1-3 of every shard reproduce the whole swarm's iteration bit for bit.
// The async run exchanges once, after its last iteration: its private global
// bests start from the exchanged init best (src/kernels.jl:196-225).
#include <cmath>
#include <cstdint>

#include "pps_internal.h"

namespace pps {

// the global best = the record with the lowest key
__global__ void k_shard_apply(SwarmDev s, const unsigned char* __restrict__ recs, int nrec, int64_t rec_bytes) {
  __shared__ int win;
  __shared__ unsigned long long wkey;
  if (threadIdx.x == 0) {
    unsigned long long best = ~0ull;
    int w = 0;
    for (int r = 0; r < nrec; ++r) {
      const unsigned long long k = *reinterpret_cast<const unsigned long long*>(recs + (int64_t)r * rec_bytes);
      if (k < best) {
        best = k;
        w = r;
      }
    }
    win = w;
    wkey = best;
  }
  __syncthreads();
  const unsigned char* rec = recs + (int64_t)win * rec_bytes;
  const float* v = reinterpret_cast<const float*>(rec + 16);
  for (int d = threadIdx.x; d < s.dim; d += blockDim.x) s.g[d] = v[d];
  if (threadIdx.x == 0) {
    s.st->gcost = reinterpret_cast<const float*>(rec)[2];
    s.st->gidx = (uint32_t)wkey;
  }
}

static bool shardable(int objective) {
  switch (objective) {
    case kSphere: case kRosenbrock: case kRastrigin: case kAckley: case kBeale: case kBooth:
    case kHimmelblau: case kQuadratic: case kBoundaryQuadratic: case kShiftedSphere:
      return true;
    default:
      return false;
  }
}

static int check_shard(pps_swarm* s) {
  if (!s) return set_error(PPS_EINVAL, "swarm is NULL");
  if (!s->shard) return set_error(PPS_EINVAL, "the swarm is not a shard (pps_shard_create)");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != s->device) PPS_CUDA(cudaSetDevice(s->device));
  return PPS_OK;
}

static int check_coefficients(pps_swarm* s, int64_t iters, float w, float wdamp, float c1, float c2) {
  if (!s->initialized) return set_error(PPS_EINVAL, "shard is not initialised (call pps_swarm_init)");
  if (iters < 0) return set_error(PPS_EINVAL, "maxiters must be >= 0");
  if (!std::isfinite(w) || !std::isfinite(wdamp) || !std::isfinite(c1) || !std::isfinite(c2))
    return set_error(PPS_EINVAL, "coefficients must be finite");
  if ((uint64_t)s->t + (uint64_t)iters > 0xFFFFFFFFull) return set_error(PPS_EINVAL, "iteration counter would overflow");
  return PPS_OK;
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace pps

using namespace pps;

extern "C" {

int pps_shard_create(const pps_problem* prob, int64_t n_global, int64_t first, int64_t count, uint64_t seed,
                     uint32_t flags, pps_swarm** out) {
  if (!out) return set_error(PPS_EINVAL, "out is NULL");
  *out = nullptr;
  if (!prob) return set_error(PPS_EINVAL, "problem is NULL");
  if (n_global < 1 || n_global > (int64_t)0xFFFFFF00LL)
    return set_error(PPS_EINVAL, "n_global must be in [1, 2^32-256] (got %lld)", (long long)n_global);
  if (first < 0 || count < 1 || first > n_global - count)
    return set_error(PPS_EINVAL, "shard [%lld, %lld + %lld) is not a non-empty range of [0, %lld)", (long long)first,
                     (long long)first, (long long)count, (long long)n_global);
  if (!shardable(prob->objective))
    return set_error(PPS_ENOTSUP, "objective %d does not shard (registered closed-form objectives only)",
                     prob->objective);
  return swarm_create(prob, count, seed, flags, first, n_global, out);
}

int pps_shard_record(pps_swarm* s, void** record, int64_t* bytes, void** stream) {
  int rc = check_shard(s);
  if (rc) return rc;
  if (record) *record = s->dv.xrec;
  if (bytes) *bytes = shard_record_bytes(s->dv.dim);
  if (stream) *stream = s->stream;
  return PPS_OK;
}

int pps_shard_bind(pps_swarm* s, void* record, const void* records, int32_t nrecords) {
  int rc = check_shard(s);
  if (rc) return rc;
  if (!record || !records) return set_error(PPS_EINVAL, "record buffers are NULL");
  if (!aligned16(record) || !aligned16(records)) return set_error(PPS_EINVAL, "record buffers must be 16-byte aligned");
  if (nrecords < 1 || nrecords > 65536) return set_error(PPS_EINVAL, "nrecords must be in [1, 65536] (got %d)", nrecords);
  cudaPointerAttributes a{};
  for (const void* p : {static_cast<const void*>(record), records}) {
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return set_error(PPS_EINVAL, "record buffers must be device memory");
    }
  }
  s->dv.xrec = static_cast<unsigned char*>(record);
  s->shard_records = static_cast<const unsigned char*>(records);
  s->shard_nrecords = nrecords;
  return PPS_OK;
}

int pps_shard_step(pps_swarm* s, int32_t begin, float w, float wdamp, float c1, float c2) {
  int rc = check_shard(s);
  if (rc) return rc;
  if ((rc = check_coefficients(s, 1, w, wdamp, c1, c2))) return rc;
  if (begin && (rc = launch_set_iter(s, s->t, w, wdamp))) return rc;
  if ((rc = launch_sync_step(s, c1, c2))) return rc;
  s->t += 1;
  return PPS_OK;
}

int pps_shard_async(pps_swarm* s, int32_t maxiters, float w, float wdamp, float c1, float c2) {
  int rc = check_shard(s);
  if (rc) return rc;
  if ((rc = check_coefficients(s, maxiters, w, wdamp, c1, c2))) return rc;
  if (s->dv.ncons > 0) return set_error(PPS_ENOTSUP, "constrained problems run synchronously");
  if ((rc = launch_set_iter(s, s->t, w, wdamp))) return rc;
  int lanes = 0;
  if ((rc = launch_async(s, maxiters, c1, c2, &lanes))) return rc;
  s->t += (uint32_t)maxiters;
  return PPS_OK;
}

int pps_shard_apply(pps_swarm* s) {
  int rc = check_shard(s);
  if (rc) return rc;
  k_shard_apply<<<1, 256, 0, s->stream>>>(s->dv, s->shard_records, s->shard_nrecords, shard_record_bytes(s->dv.dim));
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

int pps_shard_finish(pps_swarm* s) {
  int rc = check_shard(s);
  if (rc) return rc;
  if ((rc = launch_materialize(s))) return rc;
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  return check_device_status(s);
}

}  // extern "C"
