// pps_sync_bulk.cu -- the synchronous PSO step with the swarm state streamed
// through shared memory by the Tensor Memory Accelerator (cp.async.bulk).
//
// The iteration is k_sync_step's (src/kernels.jl:127-177): velocity and
// position update in Julia's broadcast order, objective, personal best with
// strict <, the block argmin folded into IterState::key and the last block's
// publication (src/lowerlevel_solve.jl:23-33); the same Philox counters, the
// same binary32 operations, the same deferred personal-best copy, so a
// particle's bits do not depend on which kernel moved it.  Only the memory
// path differs.
//
// The step reads X, V and P and writes X and V: about 2 kB per 100-D particle
// and no reuse, so it is bound by HBM bandwidth, and the bandwidth a block
// draws is the bytes it keeps in flight.  In k_sync_step those are the
// registers of the warps' software prefetch (one dim pair ahead).  Here a
// block is kBulkWarps consumer warps (two particles per thread, a tile of
// kBulkTile = 512 consecutive particles) and one producer warp.  Lane 0 of the
// producer takes tiles from the device counter (IterState::tile_next) and
// walks each tile's dims in chunks of `dims`; for every chunk it issues one
// bulk copy per state array and dim -- the tile's 2 kB segment of that row of
// X, V or P, contiguous in the SoA layout -- into a ring of `stages` shared
// memory stages, plus, with a tile's first chunk, the tile's personal-best
// costs and flags.  A "full" mbarrier per stage counts the stage's bytes; an
// "empty" mbarrier counts the consumer warps that are done with it.  The
// bytes in flight per SM are then stages x 3 x dims x 2 kB per resident block
// whatever the warps are computing, and the loads cost the consumers no
// instructions (no addresses, no load queue): they read their particles'
// float2 pairs from shared memory (conflict-free), run Philox and the update,
// and write X, V (and the deferred personal best) back with coalesced stores.
//
// Alignment.  A bulk copy wants 16-byte aligned addresses and a size that is a
// multiple of 16 bytes: the host takes this kernel only when every state array
// is 16-byte aligned and the particle stride (npad) is a multiple of 32, so a
// row segment starts at a multiple of 2 kB from its row and a tile's last
// segment holds a multiple of 32 particles (128 bytes; 32 flag bytes).
//
// Every mbarrier wait is bounded (2 s); a block whose wait gives up stops,
// lets the copies it issued land (bounded again), and sets bit 2 of
// IterState::status, which the host reports as PPS_ETIMEOUT.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pps_internal.h"
#include "pps_mbarrier.cuh"
#include "pps_publish.cuh"

namespace pps {

constexpr int kBulkWarps = 8;                        // consumer warps per block
constexpr int kBulkThreads = 32 * (kBulkWarps + 1);  // + the producer warp
constexpr int kBulkTile = 64 * kBulkWarps;           // particles per tile (two per consumer thread)
constexpr int kBulkMaxStages = 8;
constexpr uint32_t kBulkEnd = 0xFFFFFFFFu;           // stage tag: no tile left
constexpr uint64_t kBulkWaitNs = 2000000000ull;
constexpr unsigned int kStatusBulkTimeout = 4u;      // bit of IterState::status

struct BulkShape {
  int dims;    // dims per stage (even)
  int stages;  // stages in the ring
};

// one stage: X, V, P segments of `dims` rows (kBulkTile floats each), then the
// tile's personal-best costs (kBulkTile floats) and flags (kBulkTile bytes)
__host__ __device__ constexpr size_t bulk_stage_bytes(int dims) {
  return (3 * (size_t)dims + 1) * kBulkTile * 4 + kBulkTile;
}
static size_t bulk_smem_bytes(const BulkShape& sh, int dim) {
  return (size_t)sh.stages * bulk_stage_bytes(sh.dims) + 3 * sizeof(float) * (size_t)dim;
}

template <int OBJ, int SD>
__global__ void __launch_bounds__(kBulkThreads, 3)
    k_sync_step_bulk(SwarmDev s, ObjParams op, PhiloxKeys keys, float c1, float c2, int from_position,
                     int K) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bar[kBulkMaxStages];
  __shared__ __align__(8) uint64_t empty_bar[kBulkMaxStages];
  __shared__ uint32_t stage_tile[kBulkMaxStages];
  __shared__ uint32_t stage_chunk[kBulkMaxStages];
  __shared__ volatile int abort_flag;
  const int D = s.dim;
  const size_t stage_bytes = bulk_stage_bytes(SD);
  float* sg = reinterpret_cast<float*>(smem + (size_t)K * stage_bytes);
  float* slb = sg + D;
  float* sub = slb + D;
  IterState* st = s.st;
  const uint32_t t = st->t;
  const float w = st->w;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int d = tid; d < D; d += blockDim.x) {
    sg[d] = s.g[d];
    slb[d] = s.lb[d];
    sub[d] = s.ub[d];
  }
  if (tid == 0) {
    for (int k = 0; k < K; ++k) {
      mbar_init(smem_u32(&full_bar[k]), 1);
      mbar_init(smem_u32(&empty_bar[k]), kBulkWarps);
    }
    mbar_init_fence();
    abort_flag = 0;
  }
  __syncthreads();
  const int64_t npad = s.npad;
  const int64_t n = s.n;
  const uint32_t ntiles = (uint32_t)((npad + kBulkTile - 1) / kBulkTile);
  const int nchunks = (D + SD - 1) / SD;
  unsigned long long best = ~0ull;
  uint32_t issued = 0;  // producer: chunks whose copies were issued (ring positions 0 .. issued-1)

  if (warp == kBulkWarps) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      uint32_t c = 0;
      for (bool done = false; !done;) {
        const uint32_t tile = atomicAdd(&st->tile_next, 1u);
        const bool end = tile >= ntiles;
        const int64_t i0 = (int64_t)tile * kBulkTile;
        const uint32_t np = end ? 0u : (uint32_t)(npad - i0 < kBulkTile ? npad - i0 : kBulkTile);
        const uint32_t seg = np * 4u;
        const int nch = end ? 1 : nchunks;
        for (int ch = 0; ch < nch; ++ch) {
          const uint32_t k = c % (uint32_t)K, use = c / (uint32_t)K;
          if (use >= 1 && !mbar_wait_bounded(smem_u32(&empty_bar[k]), (use - 1u) & 1u, &abort_flag, kBulkWaitNs)) {
            done = true;
            break;
          }
          stage_tile[k] = end ? kBulkEnd : tile;
          stage_chunk[k] = (uint32_t)ch;
          const uint32_t fb = smem_u32(&full_bar[k]);
          ++c;
          if (end) {
            mbar_arrive(fb);
            done = true;
            break;
          }
          const int j0 = ch * SD, nd = D - j0 < SD ? D - j0 : SD;
          mbar_arrive_expect_tx(fb, 3u * (uint32_t)nd * seg + (ch == 0 ? seg + np : 0u));
          unsigned char* stg = smem + (size_t)k * stage_bytes;
          for (int jj = 0; jj < nd; ++jj) {
            const int64_t o = (int64_t)(j0 + jj) * npad + i0;
            bulk_g2s(smem_u32(stg + ((size_t)0 * SD + jj) * kBulkTile * 4), s.X + o, seg, fb);
            bulk_g2s(smem_u32(stg + ((size_t)1 * SD + jj) * kBulkTile * 4), s.V + o, seg, fb);
            bulk_g2s(smem_u32(stg + ((size_t)2 * SD + jj) * kBulkTile * 4), s.P + o, seg, fb);
          }
          if (ch == 0) {
            bulk_g2s(smem_u32(stg + (size_t)3 * SD * kBulkTile * 4), s.pcost + i0, seg, fb);
            bulk_g2s(smem_u32(stg + (size_t)(3 * SD + 1) * kBulkTile * 4), s.flag + i0, np, fb);
          }
        }
      }
      issued = c;
    }
  } else {
    // ------------------------------------------------------------ consumers
    int64_t i0 = 0;       // first of this thread's two particles in the current tile
    uint32_t gi0 = 0;     // its index in the whole swarm
    bool active = false;  // the tile holds this thread's particles
    bool anyfl = false;
    uint8_t fl[2] = {0, 0};
    float pc[2] = {0.0f, 0.0f};
    Acc<OBJ> acc[2];
    for (uint32_t c = 0;; ++c) {
      const uint32_t k = c % (uint32_t)K, use = c / (uint32_t)K;
      const bool ok = mbar_wait_bounded(smem_u32(&full_bar[k]), use & 1u, &abort_flag, kBulkWaitNs);
      if (__any_sync(0xffffffffu, !ok)) break;
      const uint32_t tile = stage_tile[k];
      if (tile == kBulkEnd) break;
      const int ch = (int)stage_chunk[k];
      const unsigned char* stg = smem + (size_t)k * stage_bytes;
      if (ch == 0) {
        i0 = (int64_t)tile * kBulkTile + 2 * tid;
        active = i0 < npad;
        gi0 = (uint32_t)(s.first + i0);
        if (active) {
          const uchar2 f = *reinterpret_cast<const uchar2*>(stg + (size_t)(3 * SD + 1) * kBulkTile * 4 + 2 * tid);
          const float2 p = *reinterpret_cast<const float2*>(stg + (size_t)3 * SD * kBulkTile * 4 + 8 * tid);
          fl[0] = f.x;
          fl[1] = f.y;
          pc[0] = p.x;
          pc[1] = p.y;
        }
        anyfl = (fl[0] | fl[1]) != 0;
        acc[0] = Acc<OBJ>();
        acc[1] = Acc<OBJ>();
      }
      if (active) {
        const int j0 = ch * SD, nd = D - j0 < SD ? D - j0 : SD;
        const float* sx = reinterpret_cast<const float*>(stg) + 2 * tid;
        const float* sv = sx + (size_t)SD * kBulkTile;
        const float* sp = sv + (size_t)SD * kBulkTile;
        // one dim of both particles: the deferred personal-best copy, the
        // update (src/kernels.jl:1-26), the objective's running sums
        auto move = [&](int jj, uint32_t ra0, uint32_t rb0, uint32_t ra1, uint32_t rb1) {
          const int j = j0 + jj;
          float2 x = *reinterpret_cast<const float2*>(sx + (size_t)jj * kBulkTile);
          float2 v = *reinterpret_cast<const float2*>(sv + (size_t)jj * kBulkTile);
          float2 p = *reinterpret_cast<const float2*>(sp + (size_t)jj * kBulkTile);
          const int64_t o = (int64_t)j * npad + i0;
          if (anyfl) {
            p.x = fl[0] ? x.x : p.x;
            p.y = fl[1] ? x.y : p.y;
            *reinterpret_cast<float2*>(s.P + o) = p;
          }
          const float gd = sg[j], lo = slb[j], hi = sub[j];
          v.x = velocity(x.x, v.x, p.x, gd, w, c1, c2, u01(ra0), u01(rb0));
          v.y = velocity(x.y, v.y, p.y, gd, w, c1, c2, u01(ra1), u01(rb1));
          x.x = clamp_lb_ub(__fadd_rn(x.x, v.x), lo, hi);
          x.y = clamp_lb_ub(__fadd_rn(x.y, v.y), lo, hi);
          acc[0].add(op, j, x.x);
          acc[1].add(op, j, x.y);
          *reinterpret_cast<float2*>(s.X + o) = x;
          *reinterpret_cast<float2*>(s.V + o) = v;
        };
        // groups of up to four dims: the group's draws first (four independent
        // chains for the scheduler to interleave; a short last chunk computes
        // a few it does not use), then its dims
        constexpr int G = SD < 4 ? SD : 4;
#pragma unroll
        for (int h = 0; h < SD; h += G) {
          Rand4 r0[G / 2], r1[G / 2];
#pragma unroll
          for (int q = 0; q < G / 2; ++q) {
            r0[q] = philox4x32_10(gi0, (uint32_t)((j0 + h) / 2 + q), t, kTagStep, keys);
            r1[q] = philox4x32_10(gi0 + 1u, (uint32_t)((j0 + h) / 2 + q), t, kTagStep, keys);
          }
#pragma unroll
          for (int q = 0; q < G / 2; ++q) {
            const int jj = h + 2 * q;
            if (jj < nd) move(jj, r0[q].a, r0[q].b, r1[q].a, r1[q].b);
            if (jj + 1 < nd) move(jj + 1, r0[q].c, r0[q].d, r1[q].c, r1[q].d);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&empty_bar[k]));  // the stage is free once every warp is done with it
      if (active && ch == nchunks - 1) {
        float cc[2];
        uint8_t nf[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          cc[q] = finalize<OBJ>(op, acc[q].s1, acc[q].s2);
          const bool valid = i0 + q < n;
          // if cost < best_cost: best = position (strict <, src/kernels.jl:21-24)
          nf[q] = (valid && cc[q] < pc[q]) ? 1 : 0;
          pc[q] = nf[q] ? cc[q] : pc[q];
          if (valid) {
            const unsigned long long key = argmin_key(pc[q], gi0 + (uint32_t)q);
            best = key < best ? key : best;
          }
        }
        *reinterpret_cast<float2*>(s.pcost + i0) = make_float2(pc[0], pc[1]);
        *reinterpret_cast<float2*>(s.cost + i0) = make_float2(cc[0], cc[1]);
        *reinterpret_cast<uchar2*>(s.flag + i0) = make_uchar2(nf[0], nf[1]);
      }
    }
  }
  __syncthreads();
  if (abort_flag) {
    if (warp == kBulkWarps && lane == 0) {
      // the copies of the last `stages` chunks may still be in flight: let
      // them land (bounded) before the block's shared memory is released
      const uint32_t first = issued > (uint32_t)K ? issued - (uint32_t)K : 0u;
      const uint64_t t0 = globaltimer();
      for (uint32_t c = first; c < issued; ++c)
        while (!mbar_try_wait(smem_u32(&full_bar[c % (uint32_t)K]), (c / (uint32_t)K) & 1u) &&
               globaltimer() - t0 < 1000000000ull) {
        }
      atomicOr(&st->status, kStatusBulkTimeout);
    }
    __syncthreads();
  }
  if (publish_block_min(best, st)) finish_iteration(s, from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
}

// ---------------------------------------------------------------- host side
// PPS_SYNC_KERNEL=bulk selects this kernel (the default is k_sync_step);
// PPS_SYNC_BULK=dims,stages pins its ring (dims 2, 4 or 8 per stage,
// 2 <= stages <= 8; default 4 dims, 3 stages).
static BulkShape bulk_shape() {
  static const BulkShape shape = [] {
    BulkShape sh{4, 3};
    if (const char* e = getenv("PPS_SYNC_BULK")) {
      int d = 0, k = 0;
      if (sscanf(e, "%d,%d", &d, &k) == 2 && (d == 2 || d == 4 || d == 8) && k >= 2 && k <= kBulkMaxStages)
        sh = BulkShape{d, k};
    }
    return sh;
  }();
  return shape;
}

static bool bulk_enabled() {
  static const bool on = [] {
    const char* e = getenv("PPS_SYNC_KERNEL");
    return e && strcmp(e, "bulk") == 0;
  }();
  return on;
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

using BulkKernel = void (*)(SwarmDev, ObjParams, PhiloxKeys, float, float, int, int);

template <int SD>
static BulkKernel bulk_kernel_sd(int objective) {
  switch (objective) {
    case kSphere: return k_sync_step_bulk<kSphere, SD>;
    case kRosenbrock: return k_sync_step_bulk<kRosenbrock, SD>;
    case kRastrigin: return k_sync_step_bulk<kRastrigin, SD>;
    case kShiftedSphere: return k_sync_step_bulk<kShiftedSphere, SD>;
    case kAckley: return k_sync_step_bulk<kAckley, SD>;
    case kBeale: return k_sync_step_bulk<kBeale, SD>;
    case kBooth: return k_sync_step_bulk<kBooth, SD>;
    case kHimmelblau: return k_sync_step_bulk<kHimmelblau, SD>;
    case kQuadratic: return k_sync_step_bulk<kQuadratic, SD>;
    case kBoundaryQuadratic: return k_sync_step_bulk<kBoundaryQuadratic, SD>;
    default: return nullptr;
  }
}

static BulkKernel bulk_kernel(int objective, int dims) {
  return dims == 2 ? bulk_kernel_sd<2>(objective) : dims == 8 ? bulk_kernel_sd<8>(objective)
                                                              : bulk_kernel_sd<4>(objective);
}

// The bulk kernel and its resident blocks per SM for this swarm, or
// *blocks = 0 where it does not apply: a constrained problem, an objective
// without a streaming kernel, an array that is not 16-byte aligned, npad not a
// multiple of 32, or a ring that does not fit in shared memory.  The
// occupancy query and the shared-memory attribute are cached per objective,
// device, dim and shape; the first call for a swarm happens outside any
// stream capture (sync_grid).
static int bulk_resolve(pps_swarm* s, BulkKernel* kern, size_t* smem, int* blocks) {
  *blocks = 0;
  if (!bulk_enabled() || s->dv.ncons > 0 || s->dv.npad % 32 != 0) return PPS_OK;
  const void* ptrs[] = {s->dv.X, s->dv.V, s->dv.P, s->dv.pcost, s->dv.cost, s->dv.flag};
  for (const void* p : ptrs)
    if (!aligned16(p)) return PPS_OK;
  const BulkShape sh = bulk_shape();
  *kern = bulk_kernel(s->objective, sh.dims);
  if (!*kern) return PPS_OK;
  *smem = bulk_smem_bytes(sh, s->dv.dim);
  if (*smem > 227 * 1024) return PPS_OK;
  struct Entry {
    int objective = -1, device = -1, dim = -1, blocks = 0;
  };
  static thread_local Entry cache[kBoundaryQuadratic + 1];
  Entry& e = cache[s->objective];
  if (e.objective != s->objective || e.device != s->device || e.dim != s->dv.dim) {
    PPS_CUDA(cudaFuncSetAttribute(*kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem));
    int per_sm = 0;
    PPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, *kern, kBulkThreads, *smem));
    e = Entry{s->objective, s->device, s->dv.dim, per_sm};
  }
  *blocks = e.blocks;
  return PPS_OK;
}

int sync_bulk_prepare(pps_swarm* s, int* blocks_per_sm) {
  BulkKernel kern = nullptr;
  size_t smem = 0;
  return bulk_resolve(s, &kern, &smem, blocks_per_sm);
}

// The bulk step where it applies (*taken true), else nothing (*taken false:
// the caller launches k_sync_step).
int launch_sync_step_bulk(pps_swarm* s, float c1, float c2, bool* taken) {
  *taken = false;
  BulkKernel kern = nullptr;
  size_t smem = 0;
  int per_sm = 0;
  int rc = bulk_resolve(s, &kern, &smem, &per_sm);
  if (rc || per_sm < 1) return rc;
  const int64_t ntiles = (s->dv.npad + kBulkTile - 1) / kBulkTile;
  const int64_t resident = (int64_t)per_sm * s->sm_count;
  const int grid = (int)(resident < ntiles ? resident : ntiles);
  const int from_pos = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  kern<<<grid, kBulkThreads, smem, s->stream>>>(s->dv, s->op, philox_round_keys(s->seed), c1, c2, from_pos,
                                                bulk_shape().stages);
  PPS_CUDA(cudaGetLastError());
  s->bounded_waits = 1;
  *taken = true;
  return PPS_OK;
}

}  // namespace pps
