// pps_vec.cuh -- vector loads and stores of PPT consecutive particles
// (float / float2 / float4 along the particle axis of the SoA state).
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>

#include <cuda_runtime.h>
#endif

namespace pps {

template <int P>
struct VecOf;
template <>
struct VecOf<1> { using T = float; };
template <>
struct VecOf<2> { using T = float2; };
template <>
struct VecOf<4> { using T = float4; };

template <int P>
__device__ __forceinline__ void ldv(float (&r)[P], const float* __restrict__ p) {
  if constexpr (P == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
  } else if constexpr (P == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    r[0] = t.x; r[1] = t.y;
  } else {
    r[0] = *p;
  }
}
template <int P>
__device__ __forceinline__ void stv(float* __restrict__ p, const float (&r)[P]) {
  if constexpr (P == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
  } else if constexpr (P == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
  } else {
    *p = r[0];
  }
}
template <int P>
__device__ __forceinline__ void ldflags(uint8_t (&f)[P], const uint8_t* __restrict__ p) {
  if constexpr (P == 4) {
    const uchar4 t = *reinterpret_cast<const uchar4*>(p);
    f[0] = t.x; f[1] = t.y; f[2] = t.z; f[3] = t.w;
  } else if constexpr (P == 2) {
    const uchar2 t = *reinterpret_cast<const uchar2*>(p);
    f[0] = t.x; f[1] = t.y;
  } else {
    f[0] = *p;
  }
}
template <int P>
__device__ __forceinline__ void stflags(uint8_t* __restrict__ p, const uint8_t (&f)[P]) {
  if constexpr (P == 4) {
    *reinterpret_cast<uchar4*>(p) = make_uchar4(f[0], f[1], f[2], f[3]);
  } else if constexpr (P == 2) {
    *reinterpret_cast<uchar2*>(p) = make_uchar2(f[0], f[1]);
  } else {
    *p = f[0];
  }
}

}  // namespace pps
