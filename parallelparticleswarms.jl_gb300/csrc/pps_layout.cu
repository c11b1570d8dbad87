// pps_layout.cu -- the swarm as the reference's particle array.
//
// The reference keeps a swarm as a vector of SPSOParticle{position, velocity,
// cost, best_position, best_cost} records (src/ParallelParticleSwarms.jl:34-44),
// 3 D + 2 floats each.  pps_get_particles / pps_set_particles move the
// structure-of-arrays state in and out in that record layout (AoS), so a
// Julia caller can wrap the buffer as Vector{SPSOParticle} with no host-side
// conversion, or field by field (SoA).  The transposition runs on the device
// through shared-memory tiles: a block reads T particles of every field row
// with one coalesced load per row and writes them back as one contiguous chunk
// of T records (or the reverse).
#include <algorithm>

#include "pps_internal.h"

namespace pps {

// field row f of the record (position 0..D-1, velocity D..2D-1, cost 2D,
// best_position 2D+1..3D, best_cost 3D+1) as a particle-fastest array
__device__ __forceinline__ float* record_row(const SwarmDev& s, int f) {
  const int D = s.dim;
  if (f < D) return s.X + (int64_t)f * s.npad;
  if (f < 2 * D) return s.V + (int64_t)(f - D) * s.npad;
  if (f == 2 * D) return s.cost;
  if (f <= 3 * D) return s.P + (int64_t)(f - 2 * D - 1) * s.npad;
  return s.pcost;
}

// odd row stride of a tile: the lanes of a warp write 32 different banks
__host__ __device__ inline int tile_stride(int F) { return (F & 1) ? F : F + 1; }

template <bool TO_AOS>
__global__ void k_records(SwarmDev s, float* __restrict__ rec, int T) {
  extern __shared__ float tile[];
  const int F = 3 * s.dim + 2, ld = tile_stride(F);
  const int64_t p0 = (int64_t)blockIdx.x * T;
  const int np = (int)((s.n - p0) < T ? (s.n - p0) : T);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (TO_AOS) {
    for (int f = warp; f < F; f += nw) {
      const float* row = record_row(s, f);
      for (int p = lane; p < np; p += 32) tile[p * ld + f] = row[p0 + p];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < np * F; k += blockDim.x) {
      const int p = k / F;
      rec[p0 * F + k] = tile[p * ld + (k - p * F)];
    }
  } else {
    for (int k = threadIdx.x; k < np * F; k += blockDim.x) {
      const int p = k / F;
      tile[p * ld + (k - p * F)] = rec[p0 * F + k];
    }
    __syncthreads();
    for (int f = warp; f < F; f += nw) {
      float* row = record_row(s, f);
      for (int p = lane; p < np; p += 32) row[p0 + p] = tile[p * ld + f];
    }
  }
}

// particles per tile: 32, fewer for wide records (at most 96 KB of tile)
static int tile_particles(int F) {
  const size_t per = sizeof(float) * (size_t)tile_stride(F);
  const size_t fit = ((size_t)96 << 10) / per;
  return (int)std::max<size_t>(1, std::min<size_t>(32, fit));
}

static int launch_records(pps_swarm* s, float* rec, bool to_aos) {
  const int F = 3 * s->dv.dim + 2, T = tile_particles(F);
  const size_t smem = sizeof(float) * (size_t)tile_stride(F) * (size_t)T;
  const unsigned blocks = (unsigned)((s->dv.n + T - 1) / T);
  if (to_aos) {
    PPS_CUDA(cudaFuncSetAttribute(k_records<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 << 10));
    k_records<true><<<blocks, 256, smem, s->stream>>>(s->dv, rec, T);
  } else {
    PPS_CUDA(cudaFuncSetAttribute(k_records<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 << 10));
    k_records<false><<<blocks, 256, smem, s->stream>>>(s->dv, rec, T);
  }
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

}  // namespace pps

using namespace pps;

extern "C" {

int pps_get_particles(pps_swarm* s, int32_t layout, float* out) {
  if (!s || !out) return set_error(PPS_EINVAL, "NULL argument");
  if (layout != PPS_LAYOUT_AOS && layout != PPS_LAYOUT_SOA) return set_error(PPS_EINVAL, "unknown layout %d", layout);
  if (!s->initialized) return set_error(PPS_EINVAL, "swarm is not initialised");
  const int D = s->dv.dim;
  const int64_t n = s->dv.n;
  if (layout == PPS_LAYOUT_SOA) {  // the record's fields one after another, each particle-fastest
    const int32_t fields[5] = {PPS_FIELD_POSITION, PPS_FIELD_VELOCITY, PPS_FIELD_COST, PPS_FIELD_PBEST, PPS_FIELD_PCOST};
    const int64_t rows[5] = {D, D, 1, D, 1};
    float* dst = out;
    for (int k = 0; k < 5; ++k) {
      const int rc = pps_get_state(s, fields[k], dst);
      if (rc) return rc;
      dst += rows[k] * n;
    }
    return PPS_OK;
  }
  PPS_CUDA(cudaSetDevice(s->device));
  const size_t F = 3 * (size_t)D + 2, bytes = sizeof(float) * F * (size_t)n;
  float* rec = nullptr;
  PPS_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rec), bytes, s->stream));
  int rc = launch_records(s, rec, true);
  if (!rc)
    rc = copy_rows_to_host(s->device, s->stream, reinterpret_cast<char*>(out), reinterpret_cast<const char*>(rec),
                           sizeof(float) * F, sizeof(float) * F, (size_t)n);
  cudaFreeAsync(rec, s->stream);
  return rc;
}

int pps_set_particles(pps_swarm* s, int32_t layout, const float* in) {
  if (!s || !in) return set_error(PPS_EINVAL, "NULL argument");
  if (s->shard) return set_error(PPS_ENOTSUP, "the particles of a shard are set through pps_set_state");
  if (layout != PPS_LAYOUT_AOS && layout != PPS_LAYOUT_SOA) return set_error(PPS_EINVAL, "unknown layout %d", layout);
  const int D = s->dv.dim;
  const int64_t n = s->dv.n;
  PPS_CUDA(cudaSetDevice(s->device));
  int rc = PPS_OK;
  if (layout == PPS_LAYOUT_SOA) {
    const int32_t fields[5] = {PPS_FIELD_POSITION, PPS_FIELD_VELOCITY, PPS_FIELD_COST, PPS_FIELD_PBEST, PPS_FIELD_PCOST};
    const int64_t rows[5] = {D, D, 1, D, 1};
    const float* src = in;
    for (int k = 0; k < 5 && !rc; ++k) {
      rc = pps_set_state(s, fields[k], src);
      src += rows[k] * n;
    }
  } else {
    const size_t F = 3 * (size_t)D + 2, bytes = sizeof(float) * F * (size_t)n;
    float* rec = nullptr;
    PPS_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rec), bytes, s->stream));
    cudaError_t e = cudaMemcpyAsync(rec, in, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) rc = cuda_error(e, "pps_set_particles");
    if (!rc) rc = launch_records(s, rec, false);
    cudaFreeAsync(rec, s->stream);
  }
  if (rc) return rc;
  // the personal bests are now P itself (no deferred copies); the global best
  // is the argmin of best_cost, as init computes it (src/init.jl:49-51)
  PPS_CUDA(cudaMemsetAsync(s->dv.flag, 0, (size_t)s->dv.npad, s->stream));
  if ((rc = launch_select_gbest(s))) return rc;
  PPS_CUDA(cudaStreamSynchronize(s->stream));
  s->initialized = 1;
  return PPS_OK;
}

}  // extern "C"
