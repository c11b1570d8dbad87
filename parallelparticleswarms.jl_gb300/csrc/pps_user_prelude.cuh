// pps_user_prelude.cuh -- what the source of a user objective sees.  NVRTC
// compiles this header, then the user's source, then pps_user_kernels.cuh
// into one program per registered objective (pps_user.cu).
//
// The user's source defines
//
//   PPS_DEVICE float pps_objective(pps_point x, int dim, const float* p,
//                                  const float* data, long long ndata)
//
// x[d] is coordinate d of the point (d < dim), p the problem's parameters
// (8 floats, zero past nparams) and data / ndata the problem's data buffer
// in device memory (NULL / 0 when it has none).  The same text compiles as
// plain C with `typedef const float* pps_point;` and an empty PPS_DEVICE,
// which is how a CPU check evaluates it.  Arithmetic is compiled with
// --fmad=false: every + and * is one binary32 operation in source order.
// pps_exp, pps_cos2pi and pps_sin2pi are the library's own exp(x),
// cos(2 pi x) and sin(2 pi x) (the functions of the registered objectives);
// CUDA's math functions (expf, cosf, ...) are available as well.
//
// HybridPSO's local stage needs a gradient: a source that defines
// PPS_HAS_GRADIENT also defines
//
//   PPS_DEVICE float pps_gradient(pps_point x, int dim, const float* p,
//                                 const float* data, long long ndata, float* g)
//
// writing grad f(x) to g[0..dim) and returning f(x).
//
// The synchronous step can evaluate f without reading the new position back
// from memory when f is a fold over the coordinates in increasing order.  A
// source that defines PPS_HAS_STREAM also defines a state type pps_stream and
//
//   PPS_DEVICE void  pps_stream_start(pps_stream* s, int dim, const float* p,
//                                     const float* data, long long ndata)
//   PPS_DEVICE void  pps_stream_add(pps_stream* s, int d, float xd, int dim,
//                                   const float* p, const float* data,
//                                   long long ndata)
//   PPS_DEVICE float pps_stream_finish(const pps_stream* s, int dim,
//                                      const float* p, const float* data,
//                                      long long ndata)
//
// The step kernel calls start, add for d = 0, 1, ..., dim - 1, then finish,
// whose value must equal pps_objective at the same point bit for bit (the
// same operations in the same order); the other kernels keep calling
// pps_objective.
#pragma once
#include "pps_device.cuh"

#define PPS_USER_SOURCE 1

// coordinate accessor over a strided column of the SoA state: one particle
// per thread, so a warp's x[d] is one coalesced 128-byte line
struct pps_point {
  const float* base;
  long long ld;
  __device__ __forceinline__ float operator[](int d) const { return base[(long long)d * ld]; }
};

#define PPS_DEVICE __device__ __forceinline__

__device__ __forceinline__ float pps_exp(float x) { return pps::exp_f(x); }
__device__ __forceinline__ float pps_cos2pi(float x) { return pps::cos2pi(x); }
__device__ __forceinline__ float pps_sin2pi(float x) { return pps::sin2pi(x); }
