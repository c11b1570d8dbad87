// pps_mlp.cu -- the MLP-regression objective on the 5th-generation tensor cores.
//
// Objective (the reference trains an MLP by PSO in examples/neural_network/nn.jl:20-62;
// the workload's variant): a 2-layer tanh network, 16 inputs -> 32 hidden ->
// 1 output, MSE over S samples of a synthetic teacher.  A particle is the
// flattened parameter vector (577 floats):
//   W1[i][j] at i*32 + j (input i, hidden j), b1 at 512 + j, w2 at 544 + j, b2 at 576.
//   loss = (1/S) sum_s (w2 . tanh(W1^T x_s + b1) + b2 - y_s)^2
//
// GB300 design.  One launch per PSO iteration does everything: the position
// update (src/kernels.jl:1-26, the arithmetic and Philox counters of the
// other step kernels), the loss, the personal best and the argmin publication.
// For a tile of 8 particles the hidden pre-activations of all S samples are a
// GEMM, [S x 16] (samples, bf16) x [16 x 256] (8 particles x 32 hidden units,
// bf16) -> [S x 256] fp32, plus the bias: per 128-sample block one
// tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = 256, K = 16) of samples x
// W1 and a second one that adds b1 as the product of a constant operand (ones
// in K columns 0-2) with b1 split into three bf16 terms hi + mid + lo (exact
// for a float).  Thread 0 issues both from shared memory (canonical K-major
// layout, no swizzle: 8-row x 16-byte core matrices) into one of two
// tensor-memory accumulator buffers (2 x 256 of the SM's 512 columns), so the
// MMAs of block m + 1 run while the 16 warps drain block m: "full" mbarriers
// (tcgen05.commit) hand a buffer to the warps, "empty" mbarriers (one arrival
// per warp) hand it back to the issuing thread.  Warp w reads TMEM lanes
// 32 (w % 4) .. +31 (its samples) and the 64 columns of particles 2 (w / 4)
// and 2 (w / 4) + 1, computes b2 + sum_j w2_j tanh(h_j) (tanh.approx.f32) and
// the squared error, and keeps one running sum per particle.  The
// per-particle losses are reduced in a fixed order (lanes by a shuffle tree,
// then the four sample quarters in order), so a particle's loss does not
// depend on its tile or block.  While a tile computes, every thread moves (or
// in the other modes loads) one dim pair of the next tile per sample block
// and stores its parameters into the second operand buffer.  The samples (A
// operand) are converted to the core-matrix layout once per swarm and copied
// into shared memory once per CTA.
//
// The epilogue is bound by the special-function pipe (one tanh per sample,
// particle and hidden unit: 16 per clock per SM); the GEMM is 2 x 16 flops
// per tanh.
//
// Every mbarrier wait is bounded by %globaltimer; a timeout ends the launch
// for the block, sets bit 1 of a status word (IterState::status for a swarm)
// and the host reports PPS_ETIMEOUT.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cuda_bf16.h>

#include "pps_internal.h"
#include "pps_mbarrier.cuh"
#include "pps_publish.cuh"

namespace pps {

constexpr int kMlpIn = 16;
constexpr int kMlpHidden = 32;
constexpr int kMlpDim = kMlpIn * kMlpHidden + 2 * kMlpHidden + 1;  // 577
constexpr int kMlpTileParticles = 8;
constexpr int kMlpN = kMlpTileParticles * kMlpHidden;  // 256 accumulator columns
constexpr int kMlpWarps = 16;
constexpr int kMlpThreads = 32 * kMlpWarps;
constexpr int kMlpMaxSamples = 4096;
constexpr uint32_t kMlpTmemCols = 2 * kMlpN;  // two accumulator buffers
constexpr size_t kMlpATileBytes = 128 * kMlpIn * 2;  // 4 KB per 128 samples
constexpr size_t kMlpBBytes = (size_t)kMlpN * kMlpIn * 2;  // 8 KB
constexpr uint64_t kMlpWaitNs = 2000000000ull;
constexpr int kMlpFmaUnitsDefault = 4;  // hidden units (of 32) whose tanh runs on the FP32 pipe

// ---------------------------------------------------------------- PTX helpers
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
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive fp32 columns of this thread's TMEM lane; the load and the
// wait are one asm statement, so no use of a value precedes the wait
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// tanh on the FP32 pipe (no special-function instruction): x P(x^2) / Q(x^2)
// on |x| <= kTanhClamp, a rational fit of this project's own
// (tanh_coefficients.py: least maximum error, Loeb's linearisation with
// Lawson's reweighting), the argument clamped beyond; 1 / Q from a seed taken
// from the bits (kRcpMagic - bits(Q)) refined by one Newton and one
// third-order step.  Maximum absolute error 1.6e-5 over all finite x (the
// special-function tanh.approx.f32 has relative error up to about 2^-11).
// 16 FP32/ALU instructions.
constexpr float kTanhClamp = 0x1.900000p+2f;  // 6.25
constexpr float kTanhA0 = 0x1.fffb1ep-1f, kTanhA1 = 0x1.d2ccf0p-4f, kTanhA2 = 0x1.7fcdecp-10f;
constexpr float kTanhB1 = 0x1.c9ea3ep-2f, kTanhB2 = 0x1.1b6c34p-6f, kTanhB3 = 0x1.be8a44p-15f;
constexpr int kRcpMagic = 0x7EF311C2;
__device__ __forceinline__ float tanh_fma(float h) {
  const float x = fminf(fmaxf(h, -kTanhClamp), kTanhClamp);
  const float z = __fmul_rn(x, x);
  float p = __fmaf_rn(kTanhA2, z, kTanhA1);
  p = __fmaf_rn(p, z, kTanhA0);
  p = __fmul_rn(p, x);
  float q = __fmaf_rn(kTanhB3, z, kTanhB2);
  q = __fmaf_rn(q, z, kTanhB1);
  q = __fmaf_rn(q, z, 1.0f);
  float y = __int_as_float(kRcpMagic - __float_as_int(q));
  float e = __fmaf_rn(-q, y, 1.0f);
  y = __fmaf_rn(y, e, y);
  e = __fmaf_rn(-q, y, 1.0f);
  y = __fmaf_rn(y, __fmaf_rn(e, e, e), y);
  return __fmul_rn(p, y);
}
// tanh_fma of two arguments with Blackwell's packed f32x2 multiply and
// multiply-add: each lane runs tanh_fma's operations (bit-identical to it),
// one instruction issue for both -- 19 instructions for two tanh instead of
// 32.  (No packed add of a product appears, so the assembler's fusion of a
// packed multiply into a following packed add cannot change a rounding.)
__device__ __forceinline__ float2 tanh_fma2(float h0, float h1) {
  const float2 x = make_float2(fminf(fmaxf(h0, -kTanhClamp), kTanhClamp), fminf(fmaxf(h1, -kTanhClamp), kTanhClamp));
  const float2 z = __fmul2_rn(x, x);
  float2 p = __ffma2_rn(make_float2(kTanhA2, kTanhA2), z, make_float2(kTanhA1, kTanhA1));
  p = __ffma2_rn(p, z, make_float2(kTanhA0, kTanhA0));
  p = __fmul2_rn(p, x);
  float2 q = __ffma2_rn(make_float2(kTanhB3, kTanhB3), z, make_float2(kTanhB2, kTanhB2));
  q = __ffma2_rn(q, z, make_float2(kTanhB1, kTanhB1));
  q = __ffma2_rn(q, z, make_float2(1.0f, 1.0f));
  float2 y = make_float2(__int_as_float(kRcpMagic - __float_as_int(q.x)), __int_as_float(kRcpMagic - __float_as_int(q.y)));
  const float2 nq = make_float2(-q.x, -q.y), one = make_float2(1.0f, 1.0f);
  float2 e = __ffma2_rn(nq, y, one);
  y = __ffma2_rn(y, e, y);
  e = __ffma2_rn(nq, y, one);
  y = __ffma2_rn(y, __ffma2_rn(e, e, e), y);
  return __fmul2_rn(p, y);
}
// the k-th of the NF hidden units whose tanh runs on the FP32 pipe: units j
// with (j % 8) < NF / 4, in increasing order
template <int NF>
__host__ __device__ constexpr int fma_unit(int k) {
  return (k / (NF / 4)) * 8 + k % (NF / 4);
}
__device__ __forceinline__ uint16_t bf16_bits(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ float bf16_value(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

// byte offset of element (row r, k) of a K-major operand tile with K = 16:
// core matrix (r / 8, k / 8) at (r / 8) * 256 + (k / 8) * 128, 16 bytes per row
__host__ __device__ __forceinline__ uint32_t kmajor_offset(uint32_t r, uint32_t k) {
  return (r >> 3) * 256u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// ---------------------------------------------------------------- the kernel
// MODE 0: init (cost -> pcost, flag 0, argmin publication)
// MODE 1: step: position update (src/kernels.jl:1-26), loss, personal best,
//         argmin publication, (t, w) advanced
// MODE 2: evaluate points (write f only; X = points, npad = stride)
struct MlpArgs {
  const uint8_t* A;      // S/128 tiles of the samples in the core-matrix layout (bf16)
  const float* y;        // S targets
  int S;
  int from_position;     // gbest gathered from positions (PPS_FLAG_GBEST_FROM_POSITION)
  float* f;              // MODE 2 output
  unsigned int* status;  // bit 1 set when a wait for the tensor core gave up
  uint64_t seed;         // MODE 1: Philox key
  float c1, c2;
};

constexpr int kMlpPairs = (kMlpDim + 1) / 2;                    // 289 dim pairs per particle
constexpr int kMlpTilePairs = kMlpTileParticles * kMlpPairs;    // 2312 per tile
constexpr int kMlpChunks = (kMlpTilePairs + kMlpThreads - 1) / kMlpThreads;  // 5 per thread
constexpr int kMlpW2Stride = 36;  // per particle: w2[32], b2, pad (16-byte rows)

// A thread owns the pairs e = tid + 512 c (c < 5) of a tile: particle e % 8,
// dims 2 (e / 8) and 2 (e / 8) + 1; a warp's accesses are 32-byte sectors (8
// consecutive particles of one dim).
struct PairLoad {
  float x0, v0, p0, x1, v1, p1;
  uint8_t flag;
};

template <bool MOVE>
__device__ __forceinline__ void pair_issue(const SwarmDev& s, int64_t tile, int64_t ntiles, int e, PairLoad& L) {
  const int p = e & 7, pr = e >> 3;
  const int64_t pi = tile * kMlpTileParticles + p;
  const bool live = tile < ntiles && e < kMlpTilePairs && pi < s.n;
  const int d0 = 2 * pr, d1 = d0 + 1;
  const bool has1 = d1 < kMlpDim;
  const int64_t o0 = (int64_t)d0 * s.npad + pi, o1 = o0 + s.npad;
  L.x0 = live ? s.X[o0] : 0.0f;
  L.x1 = (live && has1) ? s.X[o1] : 0.0f;
  if constexpr (MOVE) {
    L.v0 = live ? s.V[o0] : 0.0f;
    L.p0 = live ? s.P[o0] : 0.0f;
    L.v1 = (live && has1) ? s.V[o1] : 0.0f;
    L.p1 = (live && has1) ? s.P[o1] : 0.0f;
    L.flag = live ? s.flag[pi] : 0;
  }
}

// the position update of one pair (k_sync_step's arithmetic and Philox
// counters); returns the new positions in L.x0, L.x1
__device__ __forceinline__ void pair_move(const SwarmDev& s, const MlpArgs& a, int64_t tile, int64_t ntiles, int e,
                                          uint32_t t, float w, const float* sG, const float* sLb, const float* sUb,
                                          PairLoad& L) {
  const int p = e & 7, pr = e >> 3;
  const int64_t pi = tile * kMlpTileParticles + p;
  if (!(tile < ntiles && e < kMlpTilePairs && pi < s.n)) return;
  const int d0 = 2 * pr, d1 = d0 + 1;
  const int64_t o0 = (int64_t)d0 * s.npad + pi, o1 = o0 + s.npad;
  const Rand4 r = philox4x32_10((uint32_t)pi, (uint32_t)pr, t, kTagStep, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
  if (L.flag) {  // deferred personal-best copy of the previous step
    L.p0 = L.x0;
    s.P[o0] = L.x0;
  }
  L.v0 = velocity(L.x0, L.v0, L.p0, sG[d0], w, a.c1, a.c2, u01(r.a), u01(r.b));
  L.x0 = clamp_lb_ub(__fadd_rn(L.x0, L.v0), sLb[d0], sUb[d0]);
  s.X[o0] = L.x0;
  s.V[o0] = L.v0;
  if (d1 < kMlpDim) {
    if (L.flag) {
      L.p1 = L.x1;
      s.P[o1] = L.x1;
    }
    L.v1 = velocity(L.x1, L.v1, L.p1, sG[d1], w, a.c1, a.c2, u01(r.c), u01(r.d));
    L.x1 = clamp_lb_ub(__fadd_rn(L.x1, L.v1), sLb[d1], sUb[d1]);
    s.X[o1] = L.x1;
    s.V[o1] = L.v1;
  }
}

// one parameter of particle p into the tile's operand buffers: W1 (bf16) into
// B, b1 as three bf16 terms hi + mid + lo (exact) into the bias operand, w2
// and b2 into the epilogue's table
__device__ __forceinline__ void put_param(int p, int d, float x, uint8_t* sB, uint8_t* sBb, float* sW2) {
  if (d < kMlpIn * kMlpHidden) {
    const int i = d / kMlpHidden, j = d % kMlpHidden;
    *reinterpret_cast<uint16_t*>(sB + kmajor_offset((uint32_t)(p * kMlpHidden + j), (uint32_t)i)) = bf16_bits(x);
  } else if (d < kMlpIn * kMlpHidden + kMlpHidden) {
    const int j = d - kMlpIn * kMlpHidden;
    const float hi = bf16_value(x);
    const float mid = bf16_value(__fsub_rn(x, hi));
    const float lo = bf16_value(__fsub_rn(__fsub_rn(x, hi), mid));
    const uint32_t row = (uint32_t)(p * kMlpHidden + j);
    *reinterpret_cast<uint16_t*>(sBb + kmajor_offset(row, 0)) = bf16_bits(hi);
    *reinterpret_cast<uint16_t*>(sBb + kmajor_offset(row, 1)) = bf16_bits(mid);
    *reinterpret_cast<uint16_t*>(sBb + kmajor_offset(row, 2)) = bf16_bits(lo);
  } else {
    sW2[p * kMlpW2Stride + (d - kMlpIn * kMlpHidden - kMlpHidden)] = x;  // w2[0..31], b2 at 32
  }
}

__device__ __forceinline__ void pair_put(int e, const PairLoad& L, uint8_t* sB, uint8_t* sBb, float* sW2) {
  if (e >= kMlpTilePairs) return;
  const int p = e & 7, d0 = 2 * (e >> 3);
  put_param(p, d0, L.x0, sB, sBb, sW2);
  if (d0 + 1 < kMlpDim) put_param(p, d0 + 1, L.x1, sB, sBb, sW2);
}

// NF: hidden units (of 32) whose tanh runs on the FP32 pipe (tanh_fma), the
// rest on the special-function pipe (tanh.approx.f32); every mode of a
// process uses the same split, so a point's loss is the same in init, step
// and evaluation.
template <int MODE, int NF>
__global__ void __launch_bounds__(kMlpThreads, 1) k_mlp_eval(SwarmDev s, MlpArgs a) {
  constexpr bool MOVE = MODE == 1;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int S = a.S;
  const int mtiles = S / 128;
  uint8_t* sA = smem;                                                  // mtiles x 4 KB
  uint8_t* sOnes = sA + (size_t)mtiles * kMlpATileBytes;               // 4 KB
  uint8_t* sB = sOnes + kMlpATileBytes;                                // 2 x 8 KB (W1)
  uint8_t* sBb = sB + 2 * kMlpBBytes;                                  // 2 x 8 KB (b1 terms)
  float* sW2 = reinterpret_cast<float*>(sBb + 2 * kMlpBBytes);         // 2 x 8 x 36
  float* sY = sW2 + 2 * kMlpTileParticles * kMlpW2Stride;              // S
  float* sRed = sY + S;                                                // 2 x 16 warps x 2
  float* sG = sRed + 2 * kMlpWarps * 2;                                // 3 x 580 (MODE 1)
  float* sLb = sG + 580;
  float* sUb = sLb + 580;
  __shared__ uint64_t full_bar[2], empty_bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ int64_t s_next[2];  // the tile after the next one, fetched a tile ahead
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3;    // TMEM lane quarter: samples 32 q .. 32 q + 31 of each block
  const int pg = warp >> 2;  // particles 2 pg, 2 pg + 1 of the tile
  const int64_t n = s.n;
  const int64_t ntiles = (n + kMlpTileParticles - 1) / kMlpTileParticles;
  int64_t tile = blockIdx.x;
  // Tiles after the first: in a swarm (MODE 0, 1) taken from the iteration
  // state's counter, so CTAs on slower SMs take fewer; for points in turn.
  int64_t static_next = blockIdx.x;
  auto grab = [&]() -> int64_t {
    if constexpr (MODE == 2) {
      static_next += gridDim.x;
      return static_next;
    } else {
      return (int64_t)gridDim.x + (int64_t)atomicAdd(&s.st->tile_next, 1u);
    }
  };
  uint32_t t = 0;
  float w = 0.0f;
  if constexpr (MOVE) {
    t = s.st->t;
    w = s.st->w;
  }

  // samples, targets, the constant operand of the bias MMA (ones in K columns
  // 0-2), zeroed bias operands, and (MODE 1) gbest and the bounds
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.A);
    uint4* dst = reinterpret_cast<uint4*>(sA);
    const int n16 = (int)((size_t)mtiles * kMlpATileBytes / 16);
    for (int k = tid; k < n16; k += kMlpThreads) dst[k] = src[k];
    for (int k = tid; k < S; k += kMlpThreads) sY[k] = a.y[k];
    uint4* zb = reinterpret_cast<uint4*>(sBb);
    for (int k = tid; k < (int)(2 * kMlpBBytes / 16); k += kMlpThreads) zb[k] = make_uint4(0u, 0u, 0u, 0u);
    for (int k = tid; k < 128 * kMlpIn; k += kMlpThreads) {
      const int r = k / kMlpIn, c = k % kMlpIn;
      *reinterpret_cast<uint16_t*>(sOnes + kmajor_offset((uint32_t)r, (uint32_t)c)) = (c < 3) ? 0x3F80u : 0u;
    }
    if constexpr (MOVE) {
      for (int d = tid; d < kMlpDim; d += kMlpThreads) {
        sG[d] = s.g[d];
        sLb[d] = s.lb[d];
        sUb[d] = s.ub[d];
      }
    }
  }
  __syncthreads();  // zeroed bias operands and gbest before the first tile's parameters
  // the first tile's parameters (moved in MODE 1)
#pragma unroll 1
  for (int c = 0; c < kMlpChunks; ++c) {
    const int e = tid + kMlpThreads * c;
    PairLoad L;
    pair_issue<MOVE>(s, tile, ntiles, e, L);
    if constexpr (MOVE) pair_move(s, a, tile, ntiles, e, t, w, sG, sLb, sUb, L);
    pair_put(e, L, sB, sBb, sW2);
  }
  if (warp == 0) tmem_alloc(smem_u32(&tmem_base), kMlpTmemCols);
  if (tid == 0) {
    mbar_init(smem_u32(&full_bar[0]), 1);
    mbar_init(smem_u32(&full_bar[1]), 1);
    mbar_init(smem_u32(&empty_bar[0]), kMlpWarps);
    mbar_init(smem_u32(&empty_bar[1]), kMlpWarps);
    mbar_init_fence();
    abort_flag = 0;
    s_next[0] = grab();
  }
  fence_async_smem();  // operands written by the generic proxy, read by the tensor core
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = mlp_idesc(128, kMlpN);
  uint32_t issued = 0;    // blocks issued by thread 0 (block g goes to buffer g & 1)
  uint32_t consumed = 0;  // blocks this thread has drained
  unsigned long long best = ~0ull;
  int tb = 0;  // operand buffer of the current tile

  // thread 0: D = X W1 + b1 of block g (sample block m of the current tile)
  auto issue = [&](int m) {
    const uint32_t g = issued;
    const uint32_t b = g & 1u, use = g >> 1;
    if (use >= 1 && !mbar_wait_bounded(smem_u32(&empty_bar[b]), (use - 1u) & 1u, &abort_flag, kMlpWaitNs)) return;
    tc_after_sync();
    const uint32_t d = tmem + b * (uint32_t)kMlpN;
    mma_bf16_ss(d, smem_desc(smem_u32(sA + (size_t)m * kMlpATileBytes), 128, 256),
                smem_desc(smem_u32(sB + (size_t)tb * kMlpBBytes), 128, 256), idesc, 0u);
    mma_bf16_ss(d, smem_desc(smem_u32(sOnes), 128, 256), smem_desc(smem_u32(sBb + (size_t)tb * kMlpBBytes), 128, 256),
                idesc, 1u);
    mma_commit(smem_u32(&full_bar[b]));
    issued = g + 1;
  };

  for (int k = 0; tile < ntiles; ++k, tb ^= 1) {
    const int64_t i0 = tile * kMlpTileParticles;
    const int64_t next = s_next[k & 1];  // read by every thread before the end-of-tile barrier
    if (tid == 0) s_next[(k + 1) & 1] = grab();  // read at the top of the tile after next
    if (tid == 0) issue(0);
    // MODE 1: the personal-best costs the tile compares against, loaded early
    float pc_old = 0.0f;
    if (MODE == 1 && tid < kMlpTileParticles && i0 + tid < n) pc_old = s.pcost[i0 + tid];
    const float* w2base = sW2 + (size_t)tb * kMlpTileParticles * kMlpW2Stride + (2 * pg) * kMlpW2Stride;
    uint8_t* nB = sB + (size_t)(tb ^ 1) * kMlpBBytes;
    uint8_t* nBb = sBb + (size_t)(tb ^ 1) * kMlpBBytes;
    float* nW2 = sW2 + (size_t)(tb ^ 1) * kMlpTileParticles * kMlpW2Stride;
    float acc[2] = {0.0f, 0.0f};
    for (int m = 0; m < mtiles; ++m) {
      if (tid == 0 && m + 1 < mtiles) issue(m + 1);
      // one chunk of the next tile's parameters per block: loads issued here,
      // used after the epilogue
      PairLoad L;
      const int e = tid + kMlpThreads * m;
      const bool chunk = m < kMlpChunks;
      if (chunk) pair_issue<MOVE>(s, next, ntiles, e, L);
      __syncwarp();
      const uint32_t g = consumed;
      const uint32_t b = g & 1u;
      // every lane waits; the warp goes on only if all of them saw the phase
      // (tcgen05.ld below is a warp-wide instruction)
      int okl = 1;
      if (lane == 0) okl = mbar_wait_bounded(smem_u32(&full_bar[b]), (g >> 1) & 1u, &abort_flag, kMlpWaitNs) ? 1 : 0;
      const bool ok = __shfl_sync(0xffffffffu, okl, 0) != 0;
      __syncwarp();
      if (!ok) {
        abort_flag = 1;
        break;
      }
      tc_after_sync();
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + b * (uint32_t)kMlpN + (uint32_t)(pg * 64);
      const float ys = sY[m * 128 + q * 32 + lane];
#pragma unroll
      for (int pp = 0; pp < 2; ++pp) {
        float v[32];
        tmem_ld32(taddr + (uint32_t)(pp * 32), v);
        if (pp == 1) {  // both halves read: hand the buffer back
          tc_before_sync();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&empty_bar[b]));
        }
        const float* w2 = w2base + pp * kMlpW2Stride;
        float o = w2[32];  // b2
        // units j with (j % 8) < NF / 4 use the FP32 pipe, spread over the sum (placing
        // them last in each group of 8 measured no faster: 0.2017 vs 0.1996 ms); their
        // tanh first, two per packed instruction, then the sum in unit order
        float tf[NF > 0 ? NF : 2];
#pragma unroll
        for (int k = 0; k < NF; k += 2) {
          const float2 t2 = tanh_fma2(v[fma_unit<NF>(k)], v[fma_unit<NF>(k + 1)]);
          tf[k] = t2.x;
          tf[k + 1] = t2.y;
        }
#pragma unroll
        for (int j = 0; j < kMlpHidden; j += 4) {
          const float4 ww = *reinterpret_cast<const float4*>(w2 + j);
          const float wj[4] = {ww.x, ww.y, ww.z, ww.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int jj = j + u;
            const bool on_fma = NF > 0 && (jj & 7) < NF / 4;
            const float th = on_fma ? tf[(jj >> 3) * (NF > 0 ? NF / 4 : 1) + (jj & 7)] : tanh_fast(v[jj]);
            o = __fmaf_rn(wj[u], th, o);
          }
        }
        const float err = __fsub_rn(o, ys);
        acc[pp] = __fmaf_rn(err, err, acc[pp]);
      }
      consumed = g + 1;
      if (chunk) {
        if constexpr (MOVE) pair_move(s, a, next, ntiles, e, t, w, sG, sLb, sUb, L);
        pair_put(e, L, nB, nBb, nW2);
      }
    }
    // chunks left when the tile has fewer sample blocks than chunks
#pragma unroll 1
    for (int c = mtiles; c < kMlpChunks; ++c) {
      const int e = tid + kMlpThreads * c;
      PairLoad L;
      pair_issue<MOVE>(s, next, ntiles, e, L);
      if constexpr (MOVE) pair_move(s, a, next, ntiles, e, t, w, sG, sLb, sUb, L);
      pair_put(e, L, nB, nBb, nW2);
    }
    // ---- per-particle loss: shuffle tree over the lanes, then the quarters in order
    float* red = sRed + (size_t)tb * kMlpWarps * 2;
#pragma unroll
    for (int pp = 0; pp < 2; ++pp) {
      float vsum = acc[pp];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) vsum = __fadd_rn(vsum, __shfl_xor_sync(0xffffffffu, vsum, off));
      if (lane == 0) red[warp * 2 + pp] = vsum;
    }
    fence_async_smem();  // the next tile's operands, written above, for the tensor core
    __syncthreads();
    if (abort_flag) break;  // block-uniform after the barrier
    if (tid < kMlpTileParticles) {
      const int p = tid, g4 = p >> 1, pp = p & 1;
      float tot = 0.0f;
      for (int qq = 0; qq < 4; ++qq) tot = __fadd_rn(tot, red[(g4 * 4 + qq) * 2 + pp]);
      const float c = __fdiv_rn(tot, (float)S);
      const int64_t pi = i0 + p;
      if (pi < n) {
        if (MODE == 2) {
          a.f[pi] = c;
        } else {
          float pc = c;
          uint8_t fl = 0;
          if (MODE == 1) {
            pc = pc_old;
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
    tile = next;
  }
  if (abort_flag && tid == 0) {
    atomicOr(a.status, 2u);
    // the last block issued may still write its buffer: wait for it (bounded)
    // before the columns are released
    if (issued > 0) {
      const uint32_t g = issued - 1;
      const uint64_t t0 = globaltimer();
      while (!mbar_try_wait(smem_u32(&full_bar[g & 1u]), (g >> 1) & 1u) && globaltimer() - t0 < 1000000000ull) {
      }
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (warp == 0) tmem_dealloc(tmem, kMlpTmemCols);
  if (MODE != 2) {
    if (publish_block_min(best, s.st)) {
      IterState* st = s.st;
      if (MODE == 0)
        finish_iteration(s, a.from_position != 0, 0u, st->w);
      else
        finish_iteration(s, a.from_position != 0, t + 1u, __fmul_rn(w, st->wdamp));
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
        h = (uint16_t)((b >> 16) | ((b & 0x7fffffu) ? 0x40u : 0u));
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
  const size_t need = mlp_a_bytes(S) + kMlpATileBytes + 4 * kMlpBBytes +
                      sizeof(float) * (2 * kMlpTileParticles * kMlpW2Stride + S + 2 * kMlpWarps * 2 + 3 * 580) + 1024;
  // at least 120 KB so that no two CTAs share an SM: each holds all 512
  // tensor-memory columns, so an allocation never has to wait
  return need > 120 * 1024 ? need : 120 * 1024;
}

// one CTA per SM (tensor memory), at most one per tile
static int mlp_grid_for(int sm_count, int64_t n) {
  const int64_t ntiles = (n + kMlpTileParticles - 1) / kMlpTileParticles;
  int64_t grid = sm_count;
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
#define PPS_MLP_SMEM(NF)                                                                               \
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<0, NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<1, NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
  PPS_CUDA(cudaFuncSetAttribute(k_mlp_eval<2, NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))
  PPS_MLP_SMEM(0);
  PPS_MLP_SMEM(4);
  PPS_MLP_SMEM(8);
  PPS_MLP_SMEM(12);
#undef PPS_MLP_SMEM
  done[dev] = true;
  return PPS_OK;
}

// hidden units per 32 on the FP32 pipe: PPS_MLP_FMA_TANH = 0, 4, 8 or 12
// overrides the default (every split computes the same network; the loss
// differs only by the two tanh approximations' errors)
static int mlp_fma_units() {
  static int nf = [] {
    const char* e = getenv("PPS_MLP_FMA_TANH");
    const int v = e ? atoi(e) : kMlpFmaUnitsDefault;
    return (v == 0 || v == 4 || v == 8 || v == 12) ? v : kMlpFmaUnitsDefault;
  }();
  return nf;
}

template <int MODE>
static int launch_mlp(const SwarmDev& dv, const MlpArgs& a, int grid, cudaStream_t stream) {
  const size_t smem = mlp_smem(a.S);
  switch (mlp_fma_units()) {
    case 4: k_mlp_eval<MODE, 4><<<grid, kMlpThreads, smem, stream>>>(dv, a); break;
    case 8: k_mlp_eval<MODE, 8><<<grid, kMlpThreads, smem, stream>>>(dv, a); break;
    case 12: k_mlp_eval<MODE, 12><<<grid, kMlpThreads, smem, stream>>>(dv, a); break;
    default: k_mlp_eval<MODE, 0><<<grid, kMlpThreads, smem, stream>>>(dv, a); break;
  }
  PPS_CUDA(cudaGetLastError());
  return PPS_OK;
}

static MlpArgs args_of(pps_swarm* s) {
  MlpArgs a{};
  a.S = (int)(s->od.ndata / 17);
  a.A = reinterpret_cast<const uint8_t*>(s->mlp_a_dev);
  a.y = s->od.data + (size_t)a.S * kMlpIn;
  a.from_position = (s->flags & PPS_FLAG_GBEST_FROM_POSITION) ? 1 : 0;
  a.f = nullptr;
  a.status = &s->dv.st->status;
  a.seed = s->seed;
  return a;
}

int launch_mlp_init_eval(pps_swarm* s) {
  const int rc = mlp_set_smem_limit();  // init precedes every captured run of this swarm
  if (rc) return rc;
  return launch_mlp<0>(s->dv, args_of(s), mlp_grid_for(s->sm_count, s->dv.n), s->stream);
}

// one synchronous iteration: move, evaluate, personal bests, argmin
int launch_mlp_step(pps_swarm* s, float c1, float c2) {
  MlpArgs a = args_of(s);
  a.c1 = c1;
  a.c2 = c2;
  return launch_mlp<1>(s->dv, a, mlp_grid_for(s->sm_count, s->dv.n), s->stream);
}

// objective values at npts points x[d * stride + i]; a_dev holds the samples
// packed by mlp_pack_a, status one zeroed word
int launch_mlp_points(const float* data_dev, int64_t ndata, const uint8_t* a_dev, const float* x, int64_t npts,
                      int64_t stride, float* f, unsigned int* status, cudaStream_t stream) {
  SwarmDev dv{};
  dv.X = const_cast<float*>(x);
  dv.n = npts;
  dv.npad = stride;
  dv.dim = kMlpDim;
  MlpArgs a{};
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
  return launch_mlp<2>(dv, a, mlp_grid_for(sm, npts), stream);
}

}  // namespace pps
