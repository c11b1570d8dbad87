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
};

}  // namespace pps
