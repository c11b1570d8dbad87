// pps_mlp.cu -- the MLP-regression objective on the 5th-generation tensor cores.
//
// Objective (the reference trains an MLP by PSO in examples/neural_network/nn.jl:20-62;
// the workload's variant): a 2-layer tanh network, 16 inputs -> 32 hidden ->
// 1 output, MSE over S samples of a synthetic teacher.  A particle is the
// flattened parameter vector (577 floats):
//   W1[i][j] at i*32 + j (input i, hidden j), b1 at 512 + j, w2 at 544 + j, b2 at 576.
//   loss = (1/S) sum_s (w2 . tanh(W1^T x_s + b1) + b2 - y_s)^2
//
// GB300 design.  For a tile of 8 particles the hidden pre-activations of all S
// samples are one GEMM, [S x 16] (samples, bf16) x [16 x 256] (8 particles x 32
// hidden units, bf16) -> [S x 256] fp32: per 128-sample block one
// tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = 256, K = 16) issued by one
// thread, operands in shared memory (canonical K-major layout, no swizzle:
// 8-row x 16-byte core matrices), the accumulator in tensor memory (256
// columns).  The epilogue warps read it back with tcgen05.ld (warp w owns TMEM
// lanes 32 (w % 4) .. +31 = samples, warps 0-3 particles 0-3 and warps 4-7
// particles 4-7), apply b1, tanh (tanh.approx.f32), the output layer and the
// squared error, and reduce per particle in a fixed order.  The samples (A
// operand) are converted to the core-matrix layout once per swarm and copied
// into shared memory once per CTA.
//
// Every wait on the MMA-completion mbarrier is bounded by %globaltimer; a
// timeout sets bit 1 of a status word (IterState::status for a swarm) and the
// host reports PPS_ETIMEOUT.
#include <cstring>
#include <mutex>

#include <cuda_bf16.h>

#include "pps_internal.h"
#include "pps_publish.cuh"

namespace pps {

constexpr int kMlpIn = 16;
constexpr int kMlpHidden = 32;
constexpr int kMlpDim = kMlpIn * kMlpHidden + 2 * kMlpHidden + 1;  // 577
constexpr int kMlpTileParticles = 8;
constexpr int kMlpN = kMlpTileParticles * kMlpHidden;  // 256 accumulator columns
constexpr int kMlpThreads = 256;
constexpr int kMlpMaxSamples = 4096;
constexpr uint32_t kMlpTmemCols = 256;
constexpr size_t kMlpATileBytes = 128 * kMlpIn * 2;  // 4 KB per 128 samples
constexpr size_t kMlpBBytes = (size_t)kMlpN * kMlpIn * 2;  // 8 KB

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// shared-memory matrix descriptor: canonical layout without swizzle; LBO is
// the byte distance between core matrices along K, SBO along M / N
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
  return d;                // base offset 0, absolute LBO mode, no swizzle
}
// instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t mlp_idesc(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ uint16_t bf16_bits(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

// byte offset of element (row r, k) of a K-major operand tile with K = 16:
// core matrix (r / 8, k / 8) at (r / 8) * 256 + (k / 8) * 128, 16 bytes per row
__host__ __device__ __forceinline__ uint32_t kmajor_offset(uint32_t r, uint32_t k) {
  return (r >> 3) * 256u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// ---------------------------------------------------------------- the kernel
// MODE 0: init (cost -> pcost, flag 0, argmin publication)
// MODE 1: step (cost, personal-best update, argmin publication)
// MODE 2: evaluate points (write f only; X = points, npad = stride)
struct MlpArgs {
  const uint8_t* A;      // S/128 tiles of the samples in the core-matrix layout (bf16)
  const float* y;        // S targets
  int S;
  int from_position;     // gbest gathered from positions (PPS_FLAG_GBEST_FROM_POSITION)
  float* f;              // MODE 2 output
  unsigned int* status;  // bit 1 set when a wait for the tensor core gave up
};

template <int MODE>
__global__ void __launch_bounds__(kMlpThreads, 1) k_mlp_eval(SwarmDev s, MlpArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int mtiles = a.S / 128;
  uint8_t* sA = smem;                                             // mtiles x 4 KB
  uint8_t* sB = sA + (size_t)mtiles * kMlpATileBytes;             // 8 KB
  float* sPrm = reinterpret_cast<float*>(sB + kMlpBBytes);        // 8 x (32 b1 + 32 w2 + 1 b2)
  float* sY = sPrm + kMlpTileParticles * 65;                      // S
  float* sRed = sY + a.S;                                         // 8 warps x 4
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  IterState* st = s.st;

  // samples and targets into shared memory (16-byte copies)
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.A);
    uint4* dst = reinterpret_cast<uint4*>(sA);
    const int n16 = (int)((size_t)mtiles * kMlpATileBytes / 16);
    for (int k = tid; k < n16; k += blockDim.x) dst[k] = src[k];
    for (int k = tid; k < a.S; k += blockDim.x) sY[k] = a.y[k];
  }
  if (warp == 0) tmem_alloc(smem_u32(&tmem_base), kMlpTmemCols);
  if (tid == 0) mbar_init(smem_u32(&mbar), 1);
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t mbar_a = smem_u32(&mbar);
  const uint32_t idesc = mlp_idesc(128, kMlpN);
  const uint64_t bdesc = smem_desc(smem_u32(sB), 128, 256);
  uint32_t phase = 0;
  bool timed_out = false;

  const int64_t n = s.n;
  const int64_t ntiles = (n + kMlpTileParticles - 1) / kMlpTileParticles;
  unsigned long long best = ~0ull;
  const int q = warp & 3;        // TMEM lane quarter: samples 32q .. 32q + 31 of each block
  const int pgroup = warp >> 2;  // particles 4 pgroup .. 4 pgroup + 3 of the tile

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t i0 = tile * kMlpTileParticles;
    // ---- B: the tile's W1 as bf16, K-major (row = particle*32 + hidden unit)
    for (int e = tid; e < kMlpTileParticles * kMlpIn * kMlpHidden; e += blockDim.x) {
      const int p = e & 7, d = e >> 3;  // 8 consecutive particles of one parameter
      const int i = d / kMlpHidden, j = d % kMlpHidden;
      const int64_t pi = i0 + p;
      const float w = (pi < n) ? s.X[(int64_t)d * s.npad + pi] : 0.0f;
      *reinterpret_cast<uint16_t*>(sB + kmajor_offset((uint32_t)(p * kMlpHidden + j), (uint32_t)i)) = bf16_bits(w);
    }
    for (int e = tid; e < kMlpTileParticles * 65; e += blockDim.x) {
      const int p = e & 7, r = e >> 3;  // r: b1 (0..31), w2 (32..63), b2 (64)
      const int64_t pi = i0 + p;
      sPrm[p * 65 + r] = (pi < n) ? s.X[(int64_t)(512 + r) * s.npad + pi] : 0.0f;
    }
    fence_async_smem();  // the generic-proxy writes of B become visible to the tensor core
    tc_before_sync();
    __syncthreads();
    tc_after_sync();

    float lacc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int m = 0; m < mtiles; ++m) {
      if (tid == 0) {
        tc_after_sync();
        const uint64_t adesc = smem_desc(smem_u32(sA + (size_t)m * kMlpATileBytes), 128, 256);
        mma_bf16_ss(tmem, adesc, bdesc, idesc, 0u);
        mma_commit(mbar_a);
      }
      // bounded wait for the MMA (2 s of %globaltimer); a timeout ends the
      // launch for the whole block at the barrier below
      bool ok = true;
      {
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(mbar_a, phase)) {
          if (globaltimer() - t0 > 2000000000ull) {
            ok = false;
            break;
          }
        }
      }
      phase ^= 1u;
      tc_after_sync();
      // ---- epilogue: this thread's sample row, 4 particles of its group
      const int srow = m * 128 + q * 32 + lane;
      const float ys = sY[srow];
#pragma unroll
      for (int pp = 0; pp < 4; ++pp) {
        const int p = pgroup * 4 + pp;
        const float* prm = sPrm + p * 65;
        float o = prm[64];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(p * kMlpHidden + half * 16), v);
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int jj = half * 16 + k;
            o = __fmaf_rn(prm[32 + jj], tanh_fast(__fadd_rn(v[k], prm[jj])), o);
          }
        }
        const float e = __fsub_rn(o, ys);
        lacc[pp] = __fmaf_rn(e, e, lacc[pp]);
      }
      tc_before_sync();
      // TMEM reads done before the next MMA overwrites the accumulator
      if (__syncthreads_or(!ok)) {
        timed_out = true;
        break;
      }
    }
    if (timed_out) break;  // block-uniform
    // ---- per-particle loss: warp tree over samples, then the 4 warps in order
#pragma unroll
    for (int pp = 0; pp < 4; ++pp) {
      float vsum = lacc[pp];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) vsum = __fadd_rn(vsum, __shfl_xor_sync(0xffffffffu, vsum, off));
      if (lane == 0) sRed[warp * 4 + pp] = vsum;
    }
    __syncthreads();
    if (tid < kMlpTileParticles) {
      const int p = tid, g = p >> 2, pp = p & 3;
      float tot = 0.0f;
      for (int w = 0; w < 4; ++w) tot = __fadd_rn(tot, sRed[(g * 4 + w) * 4 + pp]);
      const float c = __fdiv_rn(tot, (float)a.S);
      const int64_t pi = i0 + p;
      if (pi < n) {
        if (MODE == 2) {
          a.f[pi] = c;
        } else {
          float pc = c;
          uint8_t fl = 0;
          if (MODE == 1) {
            pc = s.pcost[pi];
            fl = (c < pc) ? 1 : 0;  // strict <, src/kernels.jl:21-24
            pc = fl ? c : pc;
          }
          s.cost[pi] = c;
          s.pcost[pi] = pc;
          s.flag[pi] = fl;
          const unsigned long long key = argmin_key(pc, (uint32_t)pi);
          best = key < best ? key : best;
        }
      }
    }
    __syncthreads();  // sB / sPrm / sRed reused by the next tile
  }
  if (timed_out && tid == 0) {
    atomicOr(a.status, 2u);
    // the MMA in flight still writes the accumulator: wait for it (bounded)
    // before the columns are released
    const uint64_t t0 = globaltimer();
    while (!mbar_try_wait(mbar_a, phase ^ 1u) && globaltimer() - t0 < 1000000000ull) {
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (warp == 0) tmem_dealloc(tmem, kMlpTmemCols);
  if (MODE != 2) {
    if (publish_block_min(best, st)) {
      if (MODE == 0)
        finish_iteration(s, a.from_position != 0, 0u, st->w);
      else
        finish_iteration(s, a.from_position != 0, st->t + 1u, __fmul_rn(st->w, st->wdamp));
    }
  }
}

// ---------------------------------------------------------------- host side
size_t mlp_a_bytes(int S) { return (size_t)(S / 128) * kMlpATileBytes; }

// the samples (S x 16 floats, row-major) as bf16 core-matrix tiles
void mlp_pack_a(const float* X, int S, uint8_t* out) {
  for (int s = 0; s < S; ++s) {
    const int m = s / 128, r = s % 128;
    for (int k = 0; k < kMlpIn; ++k) {
      float v = X[(size_t)s * kMlpIn + k];
      uint32_t b;
      memcpy(&b, &v, 4);
      uint16_t h;
      if ((b & 0x7f800000u) == 0x7f800000u) {
        h = (uint16_t)(b >> 16) | ((b & 0x7fffffu) ? 0x40u : 0u);
      } else {
        b += 0x7fffu + ((b >> 16) & 1u);  // round to nearest even
        h = (uint16_t)(b >> 16);
      }
      memcpy(out + (size_t)m * kMlpATileBytes + kmajor_offset((uint32_t)r, (uint32_t)k), &h, 2);
    }
  }
}

int mlp_check(const pps_problem* prob) {
  if (prob->dim != kMlpDim)
    return set_error(PPS_EINVAL, "the MLP objective has %d parameters (16 inputs, 32 hidden, 1 output), got dim %d",
                     kMlpDim, prob->dim);
  if (!prob->data || prob->ndata <= 0 || prob->ndata % 17 != 0)
    return set_error(PPS_EINVAL, "MLP data is S samples x 16 inputs followed by S targets (17 S floats)");
  const int64_t S = prob->ndata / 17;
  if (S % 128 != 0 || S < 128 || S > kMlpMaxSamples)
    return set_error(PPS_EINVAL, "MLP sample count must be a multiple of 128 in [128, %d] (got %lld)", kMlpMaxSamples,
                     (long long)S);
  return PPS_OK;
}

static size_t mlp_smem(int S) {
  const size_t need = mlp_a_bytes(S) + kMlpBBytes + sizeof(float) * (kMlpTileParticles * 65 + S + 32) + 1024;
  // at least 100 KB so that at most two CTAs share an SM: each holds 256 of
  // the SM's 512 tensor-memory columns, so an allocation never has to wait
  return need > 100 * 1024 ? need : 100 * 1024;
}

static int mlp_grid(pps_swarm* s, int64_t n) {
  const int64_t ntiles = (n + kMlpTileParticles - 1) / kMlpTileParticles;
  int64_t grid = 2 * (int64_t)s->sm_count;
  if (grid > ntiles) grid = ntiles;
  return (int)(grid < 1 ? 1 : grid);
}

// The kernels' dynamic shared-memory limit is raised once per device to what
// the largest sample set needs (launches inside a stream capture then need no
// attribute call).
static int mlp_set_smem_limit() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  PPS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(PPS_ENOTSUP, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return PPS_OK;
  const int smem = (int)mlp_smem(kMlpMaxSamples);
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  done[dev] = true;
  return PPS_OK;
}

template <int MODE>
static int launch_mlp(const SwarmDev& dv, const MlpArgs& a, int grid, cudaStream_t stream) {
  const size_t smem = mlp_smem(a.S);
  k_mlp_eval<MODE><<<grid, kMlpThreads, smem, stream>>>(dv, a);
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

static MlpArgs args_of(pps_swarm* s) {
  MlpArgs a;
  a.S = (int)(s->od.ndata / 17);
  a.A = reinterpret_cast<const uint8_t*>(s->mlp_a_dev);
  a.y = s->od.data + (size_t)a.S * kMlpIn;
  a.from_position = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  a.f = nullptr;
  a.status = &s->dv.st->status;
  return a;
}

int launch_mlp_init_eval(pps_swarm* s) {
  const int rc = mlp_set_smem_limit();  // init precedes every captured run of this swarm
  if (rc) return rc;
  return launch_mlp<0>(s->dv, args_of(s), mlp_grid(s, s->dv.n), s->stream);
}
int launch_mlp_step_eval(pps_swarm* s) { return launch_mlp<1>(s->dv, args_of(s), mlp_grid(s, s->dv.n), s->stream); }

// objective values at npts points x[d * stride + i]; a_dev holds the samples
// packed by mlp_pack_a, status one zeroed word
int launch_mlp_points(const float* data_dev, int64_t ndata, const uint8_t* a_dev, const float* x, int64_t npts,
                      int64_t stride, float* f, unsigned int* status, cudaStream_t stream) {
  SwarmDev dv{};
  dv.X = const_cast<float*>(x);
  dv.n = npts;
  dv.npad = stride;
  dv.dim = kMlpDim;
  MlpArgs a;
  a.S = (int)(ndata / 17);
  a.A = a_dev;
  a.y = data_dev + (size_t)a.S * kMlpIn;
  a.from_position = 0;
  a.f = f;
  a.status = status;
  const int rc = mlp_set_smem_limit();
  if (rc) return rc;
  int sm = 0, dev = 0;
  PPS_CUDA(cudaGetDevice(&dev));
  PPS_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t ntiles = (npts + kMlpTileParticles - 1) / kMlpTileParticles;
  int64_t grid = 2 * (int64_t)sm;
  if (grid > ntiles) grid = ntiles;
  return launch_mlp<2>(dv, a, (int)(grid < 1 ? 1 : grid), stream);
}

}  // namespace pps
