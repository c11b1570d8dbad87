// pps_state.cuh -- the device-visible swarm state shared by every step kernel
// (compiled both by nvcc into the library and by NVRTC into the kernels of a
// user objective, so it includes nothing beyond pps_device.cuh).
#pragma once
#include "pps_device.cuh"

namespace pps {

// Device-resident iteration state of one swarm.  The last block of every
// step launch publishes the new global best here and advances t and w, so
// consecutive launches need no host round trip and capture into a CUDA graph
// with identical parameters.
struct IterState {
  unsigned long long key;  // running argmin key of the current launch
  unsigned int count;      // blocks finished in the current launch
  unsigned int t;          // iteration counter of the next launch
  float w;                 // inertia weight of the next launch
  float wdamp;
  float gcost;             // global best cost
  unsigned int gidx;       // global best particle
  unsigned int status;     // nonzero: a kernel detected a bad launch
  unsigned int tile_next;  // step kernel: next tile to hand out (0 at launch start)
  unsigned int pad[6];
};

// Swarm state in HBM (structure of arrays, particle index fastest):
//   X, V, P   [dim][npad] float   position, velocity, personal best
//   pcost     [npad] float        personal best cost
//   cost      [npad] float        current cost
//   flag      [npad] uint8        1: personal best improved in the last step
//                                  and not yet copied (P lags X by one step)
//   g         [dim] float         global best position
//   lb, ub    [dim] float
struct SwarmDev {
  float* X;
  float* V;
  float* P;
  float* pcost;
  float* cost;
  uint8_t* flag;
  float* g;
  float* lb;
  float* ub;
  IterState* st;
  int64_t n;
  int64_t npad;
  int dim;
  int ncons;          // constraints of the penalty path (0: none)
  const float* cons;  // ncons rows of (c_k, a_k[dim], b_k[dim])
  // Particle-range shard of a larger swarm: local particle i is particle
  // first + i of nglobal.  Random-stream counters, argmin keys and the
  // penalty's particle index are global, so a shard's particles move exactly
  // as they do in the whole swarm.  A whole swarm has first = 0, nglobal = n.
  int64_t first;
  int64_t nglobal;
  // Shard: the last block of an init or step launch writes the shard's best
  // particle to this exchange record instead of publishing it as the global
  // best (nullptr: publish into g / gcost / gidx).
  unsigned char* xrec;
};

// Exchange record of a shard (16-byte aligned, shard_record_bytes(dim) bytes):
//   [0, 8)    argmin key of the shard's best particle: orderable cost << 32 | global index
//   [8, 12)   its personal-best cost
//   [12, 16)  zero
//   [16, ...) its vector (dim floats): the position if it improved in the
//             step that produced the record (or with the CPU-backend rule), else its personal best
__host__ __device__ inline int64_t shard_record_bytes(int dim) { return (16 + 4 * (int64_t)dim + 15) / 16 * 16; }

}  // namespace pps
