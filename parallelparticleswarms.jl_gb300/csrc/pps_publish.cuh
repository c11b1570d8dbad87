// pps_publish.cuh -- the argmin publication shared by the step kernels.
//
// Each block reduces its (orderable cost << 32 | particle) key with warp
// shuffles and folds it into IterState::key with one 64-bit atomicMin; the
// block that takes the last ticket sees every other block's writes and
// gathers the winner's vector into the global-best buffer.  No block ever
// waits for another.
#pragma once
#include "pps_state.cuh"

namespace pps {

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
// argmin slot and advance (t, w).  A shard writes its winner to its exchange
// record instead; the global best is then set by the exchange.
__device__ __forceinline__ void finish_iteration(const SwarmDev& s, bool from_position,
                                                 uint32_t t_next, float w_next) {
  IterState* st = s.st;
  const unsigned long long key = atomicAdd(&st->key, 0ull);
  const uint32_t gi = (uint32_t)key;                  // global particle index
  const int64_t li = (int64_t)gi - s.first;           // its column in this swarm
  const bool found = key != ~0ull;
  const bool use_x = found && (from_position || (__ldcg(s.flag + li) != 0));
  const float* src = use_x ? s.X : s.P;
  float* dst = s.xrec ? reinterpret_cast<float*>(s.xrec + 16) : s.g;
  if (found)
    for (int d = threadIdx.x; d < s.dim; d += blockDim.x) dst[d] = __ldcg(src + (int64_t)d * s.npad + li);
  if (threadIdx.x == 0) {
    const float c = found ? __ldcg(s.pcost + li) : __int_as_float(0x7f800000);
    if (s.xrec) {
      *reinterpret_cast<unsigned long long*>(s.xrec) = key;
      reinterpret_cast<float*>(s.xrec)[2] = c;
      reinterpret_cast<unsigned int*>(s.xrec)[3] = 0u;
    } else {
      st->gcost = c;
      st->gidx = gi;
    }
    st->key = ~0ull;
    st->count = 0u;
    st->tile_next = 0u;  // every block has taken its last tile
    st->t = t_next;
    st->w = w_next;
  }
}

}  // namespace pps
