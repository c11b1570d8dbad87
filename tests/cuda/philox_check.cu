// Test-only kernels: this project's device Philox4x32-10 and math functions
// next to cuRAND's Philox4_32_10 generator, for tests/test_gpu_philox.py.
#include <cstdint>

#include <curand_kernel.h>

#include "pps_device.cuh"

// ours[i] = philox(ctr[i], key[i]); theirs[i] = first curand4() of a
// Philox4_32_10 state initialised with seed = key, subsequence = ctr.z|ctr.w<<32
// and offset = 4*ctr.x (ctr.y = 0).
__global__ void k_philox(int n, const uint32_t* ck, uint32_t* ours, uint32_t* theirs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t* c = ck + 6 * i;
  const pps::Rand4 r = pps::philox4x32_10(c[0], c[1], c[2], c[3], c[4], c[5]);
  ours[4 * i + 0] = r.a;
  ours[4 * i + 1] = r.b;
  ours[4 * i + 2] = r.c;
  ours[4 * i + 3] = r.d;
  curandStatePhilox4_32_10_t st;
  const unsigned long long seed = (unsigned long long)c[4] | ((unsigned long long)c[5] << 32);
  const unsigned long long sub = (unsigned long long)c[2] | ((unsigned long long)c[3] << 32);
  curand_init(seed, sub, 4ull * c[0], &st);
  const uint4 o = curand4(&st);
  theirs[4 * i + 0] = o.x;
  theirs[4 * i + 1] = o.y;
  theirs[4 * i + 2] = o.z;
  theirs[4 * i + 3] = o.w;
}

__global__ void k_math(int n, const float* x, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[4 * i + 0] = pps::cos2pi(x[i]);
  out[4 * i + 1] = pps::sin2pi(x[i]);
  out[4 * i + 2] = pps::exp_f(x[i]);
  out[4 * i + 3] = pps::u01(__float_as_uint(x[i]));
}

extern "C" int philox_check(int n, const uint32_t* ck_h, uint32_t* ours_h, uint32_t* theirs_h) {
  uint32_t *ck, *ours, *theirs;
  if (cudaMalloc(&ck, 6 * sizeof(uint32_t) * n) != cudaSuccess) return 1;
  cudaMalloc(&ours, 4 * sizeof(uint32_t) * n);
  cudaMalloc(&theirs, 4 * sizeof(uint32_t) * n);
  cudaMemcpy(ck, ck_h, 6 * sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
  k_philox<<<(n + 127) / 128, 128>>>(n, ck, ours, theirs);
  cudaMemcpy(ours_h, ours, 4 * sizeof(uint32_t) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(theirs_h, theirs, 4 * sizeof(uint32_t) * n, cudaMemcpyDeviceToHost);
  cudaFree(ck);
  cudaFree(ours);
  cudaFree(theirs);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int math_check(int n, const float* x_h, float* out_h) {
  float *x, *out;
  if (cudaMalloc(&x, sizeof(float) * n) != cudaSuccess) return 1;
  cudaMalloc(&out, 4 * sizeof(float) * n);
  cudaMemcpy(x, x_h, sizeof(float) * n, cudaMemcpyHostToDevice);
  k_math<<<(n + 127) / 128, 128>>>(n, x, out);
  cudaMemcpy(out_h, out, 4 * sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaFree(x);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
