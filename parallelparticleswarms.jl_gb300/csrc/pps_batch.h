// pps_batch.h -- internals shared by the batched launch (pps_batch.cu) and
// the request server (pps_serve.cu).  Not part of the public C ABI.
#pragma once
#include <vector>

#include "pps_internal.h"

namespace pps {

constexpr int kBatchMaxDim = 1024;
constexpr int64_t kBatchMaxParticles = 1 << 16;

// one swarm of a batched launch (device pointers into an arena)
struct BatchSwarm {
  int objective, dim, maxiters, sampler;
  int64_t n, ld;
  float w, wdamp, c1, c2;
  uint64_t seed;
  ObjParams op;
  int64_t ndata;
  const float* data;
  float *X, *V, *P, *pcost, *cost;
  const float *lb, *ub, *u0;
  float* g;       // dim floats: global best position (out)
  float* result;  // [gcost, gidx as bits, iterations]
  float* mail;    // optional mapped host memory: dim floats of g, then gcost, gidx bits
  int* done;      // optional mapped host flag, set to 1 once the result is in mail
};

// swarms launched together: same kernel (separable or ODE), block size and
// cluster size
struct LaunchGroup {
  int kind;        // 0: separable objectives (k_batch), 1: ODE fits (k_batch_ode)
  int T;           // threads per CTA
  int C;           // CTAs per swarm (a thread-block cluster when C > 1)
  int offset;      // first entry of this group in the order array
  int count;       // swarms in the group
  int maxdim;      // largest dim of the group
  int data_floats; // largest ODE data of the group
  int64_t maxn;      // largest swarm of the group
};

// bytes of arena one swarm needs (X, V, P, pcost, cost, lb, ub, u0, g,
// result, data), each region 256-byte aligned
size_t batch_swarm_bytes(int dim, int64_t ld, int64_t ndata);
// carve a swarm's regions from `base` (256-byte aligned)
void batch_carve(BatchSwarm& d, char* base);
double batch_work_estimate(const BatchSwarm& d);
// validate a problem for batching and fill a descriptor (no device pointers);
// host_inputs receives lb | ub | u0 | data
int batch_describe(const pps_problem* prob, int64_t n, uint64_t seed, int32_t maxiters, float w, float wdamp,
                   float c1, float c2, BatchSwarm* d, std::vector<float>* host_inputs);
size_t batch_smem_bytes(int maxdim, int data_floats, int64_t maxchunk);
// the (kind, T, C) a swarm is launched with: separable swarms use the
// batch's block size and about `spread` particles per thread per iteration
// (8 by default; fewer split a swarm over more CTAs), ODE fits two particles
// per thread (their RK4 losses packed; up to 1024 threads per CTA), both
// split over up to 16 CTAs
LaunchGroup batch_group_of(const BatchSwarm& d, int threads, int ppt, int spread = 8);
// group swarms by (kind, T, C); order lists descriptor indices group by
// group, longest estimated work first inside each group
void batch_plan(const std::vector<BatchSwarm>& descs, int threads, int ppt, std::vector<int>* order,
                std::vector<LaunchGroup>* groups, int spread = 8);
// launch one group: descs[dorder[g.offset + k]], k < g.count, on `stream`
int batch_launch_group(cudaStream_t stream, const BatchSwarm* ddescs, const int* dorder, const LaunchGroup& g,
                       int ppt);

}  // namespace pps
