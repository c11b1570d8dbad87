// pps_local.cuh -- HybridPSO's local optimisers, one per particle: the
// device code of the L-BFGS and Broyden stages, shared by the registered
// objectives' kernels (pps_hybrid.cu) and the NVRTC-compiled kernels of a user
// objective with a gradient (pps_user_kernels.cuh), so it includes nothing
// beyond the device headers.  The algorithms and the reference behaviour
// they restate are described in pps_hybrid.cu.
#pragma once
#include "pps_objgrad.cuh"

namespace pps {

constexpr int kMaxHistory = 16;

struct LocalOpts {
  int history;
  int maxiters;
  float c1;
  float gtol;
  int max_backtracks;
};

template <int MAXD>
__device__ __forceinline__ float dotv(const float (&a)[MAXD], const float (&b)[MAXD], int D) {
  float s = 0.0f;
  PPS_FOR_D(d) s = __fadd_rn(s, __fmul_rn(a[d], b[d]));
  return s;
}

// the history of one thread: in shared memory (SMEM) or thread-local arrays
template <int MAXD, bool SMEM>
struct LbfgsHistory;
// blocks of the shared-memory variant: element e of a thread's history at
// e * kLbfgsThreads + t, vectors of stride MAXD, so within a slot every access
// is one load or store at a compile-time offset from the slot's row
constexpr int kLbfgsThreads = 64;
template <int MAXD>
struct LbfgsHistory<MAXD, true> {
  float *s_, *y_, *rho_, *alpha_;
  __device__ __forceinline__ LbfgsHistory(float* sm, int, int m) {
    s_ = sm + threadIdx.x;
    y_ = s_ + m * MAXD * kLbfgsThreads;
    rho_ = y_ + m * MAXD * kLbfgsThreads;
    alpha_ = rho_ + m * kLbfgsThreads;
  }
  __device__ __forceinline__ float& S(int slot, int d) { return s_[(slot * MAXD + d) * kLbfgsThreads]; }
  __device__ __forceinline__ float& Y(int slot, int d) { return y_[(slot * MAXD + d) * kLbfgsThreads]; }
  __device__ __forceinline__ float& rho(int slot) { return rho_[slot * kLbfgsThreads]; }
  __device__ __forceinline__ float& alpha(int slot) { return alpha_[slot * kLbfgsThreads]; }
};
template <int MAXD>
struct LbfgsHistory<MAXD, false> {
  float s_[kMaxHistory][MAXD], y_[kMaxHistory][MAXD], rho_[kMaxHistory], alpha_[kMaxHistory];
  __device__ __forceinline__ LbfgsHistory(float*, int, int) {}
  __device__ __forceinline__ float& S(int slot, int d) { return s_[slot][d]; }
  __device__ __forceinline__ float& Y(int slot, int d) { return y_[slot][d]; }
  __device__ __forceinline__ float& rho(int slot) { return rho_[slot]; }
  __device__ __forceinline__ float& alpha(int slot) { return alpha_[slot]; }
};

// floats of shared memory one thread's L-BFGS history takes
__host__ __device__ constexpr size_t lbfgs_hist_floats(int m, int maxd) { return (size_t)2 * m * maxd + 2 * (size_t)m; }

// One L-BFGS per particle.  With `next` NULL each thread runs particle
// blockIdx.x * blockDim.x + threadIdx.x.  With a work counter `next` (zero at
// launch) the grid is the resident threads, and a thread whose particle has
// stopped takes the next one, particle gridDim.x * blockDim.x + atomicAdd(next, 1):
// particles stop after very different numbers of iterations, and a warp
// would otherwise run until its slowest particle stops while the other lanes
// idle.  Either way a particle's operations are the same, so its result does
// not depend on the thread that computes it.
template <int OBJ, int MAXD, bool SMEM>
__device__ __forceinline__ void lbfgs_run(const float* __restrict__ X0, int64_t ld, int64_t n, const ObjParams& op,
                                          const float* __restrict__ lbp, const float* __restrict__ ubp,
                                          const LocalOpts& o, float* __restrict__ xout, float* __restrict__ fout,
                                          float* __restrict__ itout, unsigned int* next = nullptr) {
  extern __shared__ float hist_sm[];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int D = op.dim;
  const int m = o.history;
  float lb[MAXD], ub[MAXD], x[MAXD], g[MAXD], pg[MAXD], q[MAXD], dir[MAXD], xn[MAXD], gn[MAXD];
  LbfgsHistory<MAXD, SMEM> H(hist_sm, D, m);
  PPS_FOR_D(d) {
    lb[d] = lbp[d];
    ub[d] = ubp[d];
  }
  int hist, head, it;
  float f;
  auto start = [&]() {
    PPS_FOR_D(d) x[d] = clamp_lb_ub(X0[(int64_t)d * ld + i], lb[d], ub[d]);
    hist = 0;
    head = 0;
    it = 0;
    f = obj_grad<OBJ, MAXD>(op, x, g, D);
  };
  start();
  while (true) {
    // one iteration of particle i, or its end (the stopping tests in the
    // order of the loop they restate: maxiters, a non-finite value, the
    // projected gradient, no descent direction, a failed line search)
    bool stop = it >= o.maxiters || !isfinite(f);
    if (!stop) {
      PPS_FOR_D(d) {
        const bool hold = (x[d] <= lb[d] && g[d] > 0.0f) || (x[d] >= ub[d] && g[d] < 0.0f);
        pg[d] = hold ? 0.0f : g[d];
      }
      const float gn2 = dotv<MAXD>(pg, pg, D);
      stop = __fsqrt_rn(gn2) <= o.gtol;
    }
    if (!stop) {
      PPS_FOR_D(d) q[d] = pg[d];
      for (int j = 0; j < hist; ++j) {  // newest pair first
        int slot = head - 1 - j;  // (head - 1 - j) mod m, head < m, j < m
        if (slot < 0) slot += m;
        float sq_ = 0.0f;
        PPS_FOR_D(d) sq_ = __fadd_rn(sq_, __fmul_rn(H.S(slot, d), q[d]));
        const float a = __fmul_rn(H.rho(slot), sq_);
        H.alpha(slot) = a;
        PPS_FOR_D(d) q[d] = __fsub_rn(q[d], __fmul_rn(a, H.Y(slot, d)));
      }
      float gamma = 1.0f;
      if (hist > 0) {
        const int nw = head > 0 ? head - 1 : m - 1;
        float sy = 0.0f, yy = 0.0f;
        PPS_FOR_D(d) sy = __fadd_rn(sy, __fmul_rn(H.S(nw, d), H.Y(nw, d)));
        PPS_FOR_D(d) yy = __fadd_rn(yy, __fmul_rn(H.Y(nw, d), H.Y(nw, d)));
        gamma = __fdiv_rn(sy, yy);
      }
      PPS_FOR_D(d) q[d] = __fmul_rn(gamma, q[d]);
      for (int j = hist - 1; j >= 0; --j) {  // oldest pair first
        int slot = head - 1 - j;
        if (slot < 0) slot += m;
        float yq = 0.0f;
        PPS_FOR_D(d) yq = __fadd_rn(yq, __fmul_rn(H.Y(slot, d), q[d]));
        const float b = __fmul_rn(H.rho(slot), yq);
        PPS_FOR_D(d) q[d] = __fadd_rn(q[d], __fmul_rn(H.S(slot, d), __fsub_rn(H.alpha(slot), b)));
      }
      PPS_FOR_D(d) {
        const float dd = -q[d];
        const bool hold = (x[d] <= lb[d] && dd < 0.0f) || (x[d] >= ub[d] && dd > 0.0f);
        dir[d] = hold ? 0.0f : dd;
      }
      float gd = dotv<MAXD>(g, dir, D);
      if (!(gd < 0.0f)) {  // not a descent direction: restart from steepest descent
        hist = 0;
        head = 0;
        PPS_FOR_D(d) dir[d] = -pg[d];
        gd = dotv<MAXD>(g, dir, D);
        stop = !(gd < 0.0f);
      }
    }
    if (!stop) {
      float step = 1.0f;
      bool ok = false;
      float fn = f;
      for (int bt = 0; bt < o.max_backtracks; ++bt) {
        PPS_FOR_D(d) xn[d] = clamp_lb_ub(__fadd_rn(x[d], __fmul_rn(step, dir[d])), lb[d], ub[d]);
        fn = obj_value<OBJ, MAXD>(op, xn, D);
        float dec = 0.0f;
        PPS_FOR_D(d) dec = __fadd_rn(dec, __fmul_rn(g[d], __fsub_rn(xn[d], x[d])));
        if (fn <= __fadd_rn(f, __fmul_rn(o.c1, dec))) {
          ok = true;
          break;
        }
        step = __fmul_rn(step, 0.5f);
      }
      stop = !ok;
      if (ok) {
        fn = obj_grad<OBJ, MAXD>(op, xn, gn, D);
        float sy = 0.0f;
        float sv[MAXD], yv[MAXD];
        PPS_FOR_D(d) {
          sv[d] = __fsub_rn(xn[d], x[d]);
          yv[d] = __fsub_rn(gn[d], g[d]);
          sy = __fadd_rn(sy, __fmul_rn(sv[d], yv[d]));
        }
        if (sy > 1e-12f) {
          PPS_FOR_D(d) {
            H.S(head, d) = sv[d];
            H.Y(head, d) = yv[d];
          }
          H.rho(head) = __fdiv_rn(1.0f, sy);
          head = head + 1 == m ? 0 : head + 1;
          if (hist < m) ++hist;
        }
        PPS_FOR_D(d) {
          x[d] = xn[d];
          g[d] = gn[d];
        }
        f = fn;
        ++it;
      }
    }
    if (stop) {
      PPS_FOR_D(d) xout[(int64_t)d * ld + i] = x[d];
      fout[i] = isfinite(f) ? f : __int_as_float(0x7f800000);  // non-finite -> Inf (src/lbfgs.jl:20)
      itout[i] = (float)it;
      if (!next) return;
      i = (int64_t)gridDim.x * blockDim.x + (int64_t)atomicAdd(next, 1u);
      if (i >= n) return;
      start();
    }
  }
}

// BoundedGrad (src/hybrid.jl:23-31): the gradient inside the box grown by
// twice its width, 1e15 in every component outside it
template <int OBJ, int MAXD>
__device__ __forceinline__ void bounded_grad(const ObjParams& op, const float (&x)[MAXD], const float (&lb)[MAXD],
                                             const float (&ub)[MAXD], float (&F)[MAXD], int D) {
  bool in_box = true;
  PPS_FOR_D(d) {
    const float w = __fsub_rn(ub[d], lb[d]);
    if (!isfinite(x[d]) || x[d] < __fsub_rn(lb[d], __fmul_rn(2.0f, w)) || x[d] > __fadd_rn(ub[d], __fmul_rn(2.0f, w)))
      in_box = false;
  }
  if (in_box) {
    obj_grad<OBJ, MAXD>(op, x, F, D);
  } else {
    PPS_FOR_D(d) F[d] = 1.0e15f;
  }
}

// Broyden's inverse Jacobian of one thread: in shared memory (SMEM; blocks of
// kBroydenThreads, element (a, b) of thread t at (a MAXD + b) kBroydenThreads
// + t, so every access is one load or store at a compile-time offset and a
// warp's accesses hit 32 banks) or a register array (small MAXD)
constexpr int kBroydenThreads = 64;
template <int MAXD, bool SMEM>
struct BroydenJ;
template <int MAXD>
struct BroydenJ<MAXD, true> {
  float* base;
  __device__ __forceinline__ explicit BroydenJ(float* sm) : base(sm + threadIdx.x) {}
  __device__ __forceinline__ float& at(int a, int b) { return base[(a * MAXD + b) * kBroydenThreads]; }
};
template <int MAXD>
struct BroydenJ<MAXD, false> {
  float m[MAXD][MAXD];
  __device__ __forceinline__ explicit BroydenJ(float*) {}
  __device__ __forceinline__ float& at(int a, int b) { return m[a][b]; }
};

// One Broyden solve per particle; `next` as for lbfgs_run (a thread whose
// particle has stopped takes the next one).
template <int OBJ, int MAXD, bool SMEM>
__device__ __forceinline__ void broyden_run(const float* __restrict__ X0, int64_t ld, int64_t n, const ObjParams& op,
                                            const float* __restrict__ lbp, const float* __restrict__ ubp,
                                            const LocalOpts& o, float* __restrict__ xout, float* __restrict__ fout,
                                            float* __restrict__ itout, unsigned int* next = nullptr) {
  extern __shared__ float jsm[];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int D = op.dim;
  float lb[MAXD], ub[MAXD], x[MAXD], F[MAXD], xn[MAXD], Fn[MAXD], dx[MAXD], dF[MAXD], JdF[MAXD], dxJ[MAXD], step[MAXD];
  BroydenJ<MAXD, SMEM> J(jsm);
  PPS_FOR_D(d) {
    lb[d] = lbp[d];
    ub[d] = ubp[d];
  }
  float phi;
  int it;
  auto start = [&]() {
    PPS_FOR_D(d) x[d] = X0[(int64_t)d * ld + i];
    PPS_FOR_D(a) {
      PPS_FOR_D(b) J.at(a, b) = (a == b) ? 1.0f : 0.0f;
    }
    bounded_grad<OBJ, MAXD>(op, x, lb, ub, F, D);
    phi = dotv<MAXD>(F, F, D);
    it = 0;
  };
  start();
  while (true) {
    bool stop = it >= o.maxiters || !(__fsqrt_rn(phi) > o.gtol);
    if (!stop) {
      PPS_FOR_D(a) {
        float s = 0.0f;
        PPS_FOR_D(b) s = __fadd_rn(s, __fmul_rn(J.at(a, b), F[b]));
        step[a] = -s;
      }
      float sc = 1.0f, phin = phi;
      bool ok = false;
      for (int bt = 0; bt < o.max_backtracks; ++bt) {
        PPS_FOR_D(d) xn[d] = __fadd_rn(x[d], __fmul_rn(sc, step[d]));
        bounded_grad<OBJ, MAXD>(op, xn, lb, ub, Fn, D);
        phin = dotv<MAXD>(Fn, Fn, D);
        if (phin < phi) {
          ok = true;
          break;
        }
        sc = __fmul_rn(sc, 0.5f);
      }
      stop = !ok;
      if (ok) {
        PPS_FOR_D(d) {
          dx[d] = __fsub_rn(xn[d], x[d]);
          dF[d] = __fsub_rn(Fn[d], F[d]);
        }
        PPS_FOR_D(a) {
          float s = 0.0f;
          PPS_FOR_D(b) s = __fadd_rn(s, __fmul_rn(J.at(a, b), dF[b]));
          JdF[a] = s;
        }
        PPS_FOR_D(b) {
          float s = 0.0f;
          PPS_FOR_D(a) s = __fadd_rn(s, __fmul_rn(dx[a], J.at(a, b)));
          dxJ[b] = s;
        }
        const float den = dotv<MAXD>(dx, JdF, D);
        if (den != 0.0f && isfinite(den)) {
          PPS_FOR_D(a) {
            const float c = __fdiv_rn(__fsub_rn(dx[a], JdF[a]), den);
            PPS_FOR_D(b) J.at(a, b) = __fadd_rn(J.at(a, b), __fmul_rn(c, dxJ[b]));
          }
        }
        PPS_FOR_D(d) {
          x[d] = xn[d];
          F[d] = Fn[d];
        }
        phi = phin;
        ++it;
      }
    }
    if (stop) {
      PPS_FOR_D(d) xout[(int64_t)d * ld + i] = x[d];
      const float v = obj_value<OBJ, MAXD>(op, x, D);
      fout[i] = isfinite(v) ? v : __int_as_float(0x7f800000);  // NaN / Inf -> Inf (src/hybrid.jl:44)
      itout[i] = (float)it;
      if (!next) return;
      i = (int64_t)gridDim.x * blockDim.x + (int64_t)atomicAdd(next, 1u);
      if (i >= n) return;
      start();
    }
  }
}

}  // namespace pps
