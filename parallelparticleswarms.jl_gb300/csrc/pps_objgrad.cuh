// pps_objgrad.cuh -- whole-vector objective value and analytic gradient of
// the registered objectives, for the per-particle local optimisers.
//
// The reference differentiates the user's closure with ForwardDiff
// (ForwardDiffGradient, src/utils.jl:379-384); the workload asks for analytic
// gradients, written out here for every registered objective.  Sums run over
// dims in order, one binary32 operation at a time (the library is compiled
// with -fmad=false), the same sequence the CPU restatement performs.
#pragma once
#include "pps_device.cuh"

namespace pps {

// Loops run to the compile-time bound MAXD with a d < D guard, so register
// arrays of the caller stay in registers.
#define PPS_FOR_D(d) _Pragma("unroll") for (int d = 0; d < MAXD; ++d) if (d < D)

// a user objective (compiled by NVRTC with its source): f and, when the source
// defines PPS_HAS_GRADIENT, pps_gradient(x, dim, p, data, ndata, g) returning f
constexpr int kUserObjective = 255;

template <int OBJ, int MAXD>
__device__ __forceinline__ float obj_value(const ObjParams& op, const float (&x)[MAXD], int D) {
#ifdef PPS_USER_SOURCE
  if constexpr (OBJ == kUserObjective) return pps_objective(pps_point{x, 1}, D, op.p, op.data, op.ndata);
#endif
  Acc<OBJ> acc;
  PPS_FOR_D(d) acc.add(op, d, x[d]);
  return finalize<OBJ>(op, acc.s1, acc.s2);
}

// f(x) and grad f(x) into g[0..D)
template <int OBJ, int MAXD>
__device__ __forceinline__ float obj_grad(const ObjParams& op, const float (&x)[MAXD], float (&g)[MAXD], int D) {
#if defined(PPS_USER_SOURCE) && defined(PPS_HAS_GRADIENT)
  if constexpr (OBJ == kUserObjective) return pps_gradient(pps_point{x, 1}, D, op.p, op.data, op.ndata, g);
#endif
  const float f = obj_value<OBJ, MAXD>(op, x, D);
  if constexpr (OBJ == kSphere) {
    PPS_FOR_D(d) g[d] = __fmul_rn(2.0f, x[d]);
  } else if constexpr (OBJ == kRosenbrock) {
    const float p1 = prm(op, 0, 1.0f), p2 = prm(op, 1, 100.0f);
    PPS_FOR_D(d) {
      float gd = 0.0f;
      if (d < D - 1 && d + 1 < MAXD) {
        const float t = __fsub_rn(x[d + 1], __fmul_rn(x[d], x[d]));
        gd = __fsub_rn(__fmul_rn(__fmul_rn(__fmul_rn(-4.0f, p2), x[d]), t), __fmul_rn(2.0f, __fsub_rn(p1, x[d])));
      }
      if (d > 0) {
        const float t = __fsub_rn(x[d], __fmul_rn(x[d - 1], x[d - 1]));
        gd = __fadd_rn(gd, __fmul_rn(__fmul_rn(2.0f, p2), t));
      }
      g[d] = gd;
    }
  } else if constexpr (OBJ == kRastrigin) {
    const float twopiA = __fmul_rn(prm(op, 0, 10.0f), 0x1.921fb6p+2f);
    PPS_FOR_D(d) g[d] = __fadd_rn(__fmul_rn(2.0f, x[d]), __fmul_rn(twopiA, sin2pi(x[d])));
  } else if constexpr (OBJ == kAckley) {
    const float a = prm(op, 0, 20.0f), b = prm(op, 1, 0.2f), k = prm(op, 2, 1.0f);
    const float Df = (float)D;
    float s1 = 0.0f, s2 = 0.0f;
    PPS_FOR_D(d) {
      s1 = __fadd_rn(s1, __fmul_rn(x[d], x[d]));
      s2 = __fadd_rn(s2, cos2pi(__fmul_rn(k, x[d])));
    }
    const float rms = __fsqrt_rn(__fdiv_rn(s1, Df));
    const float e1 = exp_f(__fmul_rn(-b, rms));
    const float e2 = exp_f(__fdiv_rn(s2, Df));
    const float c1 = (rms > 0.0f) ? __fdiv_rn(__fmul_rn(__fmul_rn(a, b), e1), __fmul_rn(Df, rms)) : 0.0f;
    const float c2 = __fdiv_rn(__fmul_rn(e2, __fmul_rn(0x1.921fb6p+2f, k)), Df);
    PPS_FOR_D(d) g[d] = __fadd_rn(__fmul_rn(c1, x[d]), __fmul_rn(c2, sin2pi(__fmul_rn(k, x[d]))));
  } else if constexpr (OBJ == kBeale && MAXD >= 2) {
    const float x1 = x[0], x2 = x[1], x22 = sq(x2), x23 = __fmul_rn(x22, x2);
    const float a = __fadd_rn(__fsub_rn(1.5f, x1), __fmul_rn(x1, x2));
    const float b = __fadd_rn(__fsub_rn(2.25f, x1), __fmul_rn(x1, x22));
    const float c = __fadd_rn(__fsub_rn(2.625f, x1), __fmul_rn(x1, x23));
    // (2a(x2-1) + 2b(x2^2-1)) + 2c(x2^3-1)
    g[0] = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(2.0f, a), __fsub_rn(x2, 1.0f)),
                               __fmul_rn(__fmul_rn(2.0f, b), __fsub_rn(x22, 1.0f))),
                     __fmul_rn(__fmul_rn(2.0f, c), __fsub_rn(x23, 1.0f)));
    // (2a x1 + 2b (2 x1 x2)) + 2c (3 x1 x2^2)
    g[1] = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(2.0f, a), x1),
                               __fmul_rn(__fmul_rn(2.0f, b), __fmul_rn(__fmul_rn(2.0f, x1), x2))),
                     __fmul_rn(__fmul_rn(2.0f, c), __fmul_rn(__fmul_rn(3.0f, x1), x22)));
  } else if constexpr (OBJ == kBooth && MAXD >= 2) {
    const float a = __fsub_rn(__fadd_rn(x[0], __fmul_rn(2.0f, x[1])), 7.0f);
    const float b = __fsub_rn(__fadd_rn(__fmul_rn(2.0f, x[0]), x[1]), 5.0f);
    g[0] = __fadd_rn(__fmul_rn(2.0f, a), __fmul_rn(4.0f, b));
    g[1] = __fadd_rn(__fmul_rn(4.0f, a), __fmul_rn(2.0f, b));
  } else if constexpr (OBJ == kHimmelblau && MAXD >= 2) {
    const float a = __fsub_rn(__fadd_rn(sq(x[0]), x[1]), 11.0f);
    const float b = __fsub_rn(__fadd_rn(x[0], sq(x[1])), 7.0f);
    g[0] = __fadd_rn(__fmul_rn(__fmul_rn(4.0f, a), x[0]), __fmul_rn(2.0f, b));
    g[1] = __fadd_rn(__fmul_rn(2.0f, a), __fmul_rn(__fmul_rn(4.0f, b), x[1]));
  } else if constexpr (OBJ == kQuadratic) {
    g[0] = __fmul_rn(__fmul_rn(2.0f, prm(op, 0, 1.0f)), __fsub_rn(x[0], 1.0f));
    if constexpr (MAXD >= 2) {
      if (D > 1) g[1] = __fmul_rn(2.0f, __fadd_rn(x[1], 2.0f));
    }
  } else if constexpr (OBJ == kBoundaryQuadratic) {
    g[0] = __fmul_rn(2.0f, __fadd_rn(x[0], 1.0f));
    PPS_FOR_D(d) if (d > 0) g[d] = 0.0f;
  }
  return f;
}

}  // namespace pps
