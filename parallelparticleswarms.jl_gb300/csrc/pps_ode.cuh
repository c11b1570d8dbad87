// pps_ode.cuh -- the ode_pso objective: integrate the model with the
// particle's position as its parameters, SSE against observations.
//
// Reference: parameter_estim_ode! (src/ode_pso.jl:113-170) builds one ODE
// problem per particle (default_prob_func, :43-45), integrates them with
// DiffEqGPU's GPUTsit5 and reduces the loss with _reduce_losses! (:47-52):
//   loss = sum over save points of sum over states (data - u)^2.
// The workload integrates with the classical fixed-step RK4 instead; the
// stage arithmetic below is exactly the CPU restatement's (fused multiply-adds
// where it writes fmaf).
// Integrators: the workload's classical fixed-step RK4 with saves every
// save_every steps, or the reference's own method, Tsitouras' 5(4) pair
// (GPUTsit5) at a fixed step, adaptive = false as the reference's benchmarks
// run it (benchmarks/Lotka_Volterra/lotka_volterra.jl:122-127), with saves
// at t_m = m save_dt taken from the method's 4th-order continuous extension.
// Right-hand sides (the reference's benchmark models):
//   Lotka-Volterra  benchmarks/Lotka_Volterra/lotka_volterra.jl:9-13
//     du1 = p1 u1 - p2 u1 u2,  du2 = -p3 u2 + p4 u1 u2
//   FitzHugh-Nagumo benchmarks/Fitzhugh_Nagumo/ode_estimation.jl:6-12
//     dv = v - v^3/3 - w + l,  dw = tinv (v + a - b w),  p = (a, b, tinv) with l
//     fixed, or p = (a, b, tinv, l) as the reference's benchmark fits it
// evaluated in factored form -- u1 fma(-p2, u2, p1), u2 fma(p4, u1, -p3),
// (fma(v^3, -1/3, v) - w) + l, tinv fma(-b, w, v + a) -- two roundings per
// term and no division, which halves the instructions of an RK4 step.
#pragma once
#include "pps_device.cuh"

namespace pps {

constexpr int kOdeLV = 0;
constexpr int kOdeFHN = 1;
constexpr int kOdeMaxSaves = 4096;
constexpr int kOdeRk4 = 0;
constexpr int kOdeTsit5 = 1;
constexpr int kOdeTsit5Adaptive = 2;
constexpr int kOdeMaxSteps = 100000;  // accepted + rejected steps per adaptive solve (then the loss is +inf)

// Fit configuration, packed by the host from pps_problem.params:
// params = [u0_1, u0_2, dt, nsteps, save_every, l (FHN), method, save_dt],
// data = nsaves x 2 (t = 0 included).  method 0 (default): RK4, a save every
// save_every steps; 1: Tsit5 at a fixed step, saves at m * save_dt; 2: Tsit5
// with adaptive steps from dt, saves at m * save_dt up to (nsaves - 1)
// save_dt, params[3] = reltol and params[4] = abstol in place of nsteps and
// save_every.
struct OdeCfg {
  float u0a, u0b, dt, l;
  int nsteps, save_every, nsaves;
  int method;
  float save_dt;
  int dim;  // FHN: 3 fits (a, b, tinv) with l fixed, 4 fits l as well
  float rtol, atol;  // method 2
};

__host__ __device__ inline OdeCfg ode_cfg(const ObjParams& op, int64_t ndata) {
  OdeCfg c;
  c.u0a = op.p[0];
  c.u0b = op.p[1];
  c.dt = op.p[2];
  c.nsteps = (int)op.p[3];
  c.save_every = (int)op.p[4];
  c.l = op.p[5];
  c.nsaves = (int)(ndata / 2);
  c.method = op.np > 6 ? (int)op.p[6] : kOdeRk4;
  c.save_dt = op.np > 7 ? op.p[7] : 0.0f;
  c.dim = op.dim;
  c.rtol = op.p[3];
  c.atol = op.p[4];
  if (c.method == kOdeTsit5Adaptive) c.nsteps = c.save_every = 0;
  return c;
}

// FHN's l: fixed by the fit, or the particle's 4th parameter
__device__ __forceinline__ float ode_l(const float* p, const OdeCfg& c) { return c.dim > 3 ? p[3] : c.l; }

template <int MODEL>
__device__ __forceinline__ void ode_rhs(const float* p, float l, float u0, float u1, float& d0, float& d1) {
  if constexpr (MODEL == kOdeLV) {
    d0 = __fmul_rn(u0, __fmaf_rn(-p[1], u1, p[0]));
    d1 = __fmul_rn(u1, __fmaf_rn(p[3], u0, -p[2]));
  } else {
    const float v3 = __fmul_rn(__fmul_rn(u0, u0), u0);
    d0 = __fadd_rn(__fsub_rn(__fmaf_rn(v3, -0x1.555556p-2f, u0), u1), l);
    d1 = __fmul_rn(p[2], __fmaf_rn(-p[1], u1, __fadd_rn(u0, p[0])));
  }
}

template <int MODEL>
__device__ __forceinline__ void rk4_step(const float* p, float l, float dt, float h2, float h6, float& u0, float& u1) {
  float k1a, k1b, k2a, k2b, k3a, k3b, k4a, k4b;
  ode_rhs<MODEL>(p, l, u0, u1, k1a, k1b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(h2, k1a, u0), __fmaf_rn(h2, k1b, u1), k2a, k2b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(h2, k2a, u0), __fmaf_rn(h2, k2b, u1), k3a, k3b);
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, k3a, u0), __fmaf_rn(dt, k3b, u1), k4a, k4b);
  float sa = __fmaf_rn(2.0f, k2a, k1a);
  sa = __fmaf_rn(2.0f, k3a, sa);
  sa = __fadd_rn(sa, k4a);
  float sb = __fmaf_rn(2.0f, k2b, k1b);
  sb = __fmaf_rn(2.0f, k3b, sb);
  sb = __fadd_rn(sb, k4b);
  u0 = __fmaf_rn(h6, sa, u0);
  u1 = __fmaf_rn(h6, sb, u1);
}

// SSE of the RK4 trajectory against data[nsaves][2] (t = 0 included)
template <int MODEL>
__device__ __forceinline__ float ode_loss(const float* p, const OdeCfg& c, const float* data) {
  const float dt = c.dt;
  const float h2 = __fmul_rn(dt, 0.5f);
  const float h6 = __fdiv_rn(dt, 6.0f);
  const float l = ode_l(p, c);
  float u0 = c.u0a, u1 = c.u0b;
  float e0 = __fsub_rn(data[0], u0), e1 = __fsub_rn(data[1], u1);
  float acc = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
  // save m after m * save_every steps ((nsaves - 1) save_every <= nsteps is
  // checked on the host); the steps between two saves run without a per-step
  // test, two per loop trip
  for (int m = 1; m < c.nsaves; ++m) {
#pragma unroll 2
    for (int k = 0; k < c.save_every; ++k) rk4_step<MODEL>(p, l, dt, h2, h6, u0, u1);
    e0 = __fsub_rn(data[2 * m], u0);
    e1 = __fsub_rn(data[2 * m + 1], u1);
    acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
  }
  return acc;
}

// ---------------------------------------------------------------- RK4, two particles at once
// ode_loss of two particles (lane x: xa, lane y: xb) with Blackwell's packed
// f32x2 instructions: each lane runs exactly ode_loss's operations, one
// instruction issue for both, bit-identical to two ode_loss calls.
// The assembler contracts a packed multiply whose only use is a packed add
// into one fused f32x2 multiply-add, even under -fmad=false and with .rn on
// both, which changes the rounding (scalar multiplies and adds are left
// alone).  So every add of a product is written here as fma(product, one,
// other) with `one` a run-time 1.0f (a kernel argument the compiler cannot
// see through): product * 1 is exact, so it rounds once, as the add does.
namespace rk4x2 {
__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a + b, a or b possibly a product
__device__ __forceinline__ float2 add(float2 a, float2 b, float2 one) { return __ffma2_rn(a, one, b); }

template <int MODEL>
__device__ __forceinline__ void rhs(const float2 (&p)[4], float2 l, float2 one, float2 u0, float2 u1, float2& d0,
                                    float2& d1) {
  if constexpr (MODEL == kOdeLV) {
    d0 = mul(u0, fma(neg(p[1]), u1, p[0]));
    d1 = mul(u1, fma(p[3], u0, neg(p[2])));
  } else {
    const float2 v3 = mul(mul(u0, u0), u0);
    d0 = add(add(fma(v3, dup(-0x1.555556p-2f), u0), neg(u1), one), l, one);
    d1 = mul(p[2], fma(neg(p[1]), u1, add(u0, p[0], one)));
  }
}
}  // namespace rk4x2

template <int MODEL>
__device__ __forceinline__ float2 ode_loss2(const float* pa, const float* pb, const OdeCfg& c, const float* data,
                                            float one_) {
  using namespace rk4x2;
  const float2 one = dup(one_);
  float2 p[4];
#pragma unroll
  for (int d = 0; d < 4; ++d) p[d] = make_float2(pa[d], pb[d]);
  const float2 l = make_float2(ode_l(pa, c), ode_l(pb, c));
  const float dt = c.dt;
  const float2 h2 = dup(__fmul_rn(dt, 0.5f)), h6 = dup(__fdiv_rn(dt, 6.0f)), dt2 = dup(dt), two = dup(2.0f);
  float2 u0 = dup(c.u0a), u1 = dup(c.u0b);
  float2 e0 = add(dup(data[0]), neg(u0), one), e1 = add(dup(data[1]), neg(u1), one);
  float2 acc = add(mul(e0, e0), mul(e1, e1), one);
  for (int m = 1; m < c.nsaves; ++m) {
#pragma unroll 2
    for (int k = 0; k < c.save_every; ++k) {
      float2 k1a, k1b, k2a, k2b, k3a, k3b, k4a, k4b;
      rhs<MODEL>(p, l, one, u0, u1, k1a, k1b);
      rhs<MODEL>(p, l, one, fma(h2, k1a, u0), fma(h2, k1b, u1), k2a, k2b);
      rhs<MODEL>(p, l, one, fma(h2, k2a, u0), fma(h2, k2b, u1), k3a, k3b);
      rhs<MODEL>(p, l, one, fma(dt2, k3a, u0), fma(dt2, k3b, u1), k4a, k4b);
      float2 sa = fma(two, k2a, k1a);
      sa = fma(two, k3a, sa);
      sa = add(k4a, sa, one);
      float2 sb = fma(two, k2b, k1b);
      sb = fma(two, k3b, sb);
      sb = add(k4b, sb, one);
      u0 = fma(h6, sa, u0);
      u1 = fma(h6, sb, u1);
    }
    e0 = add(dup(data[2 * m]), neg(u0), one);
    e1 = add(dup(data[2 * m + 1]), neg(u1), one);
    acc = add(acc, add(mul(e0, e0), mul(e1, e1), one), one);
  }
  return acc;
}

// ---------------------------------------------------------------- Tsit5
// Tsitouras, "Runge-Kutta pairs of order 5(4) satisfying only the first
// column simplifying assumption", Comput. Math. Appl. 62 (2011) 770-775: the
// 7-stage first-same-as-last pair (b = the 7th stage's row) and its
// continuous extension b_i(theta) = delta_i1 theta + r_i2 theta^2 +
// r_i3 theta^3 + r_i4 theta^4.  Decimal constants rounded to binary32 by the
// compiler; the models are autonomous, so the nodes c_i are not needed.
namespace ts5 {
constexpr float a21 = 0.161f;
constexpr float a31 = -0.008480655492356989f, a32 = 0.335480655492357f;
constexpr float a41 = 2.897153057105493f, a42 = -6.359448489975075f, a43 = 4.3622954328695815f;
constexpr float a51 = 5.325864828439257f, a52 = -11.748883564062828f, a53 = 7.4955393428898365f,
                a54 = -0.09249506636175525f;
constexpr float a61 = 5.86145544294642f, a62 = -12.92096931784711f, a63 = 8.159367898576159f,
                a64 = -0.071584973281401f, a65 = -0.028269050394068383f;
constexpr float b1 = 0.09646076681806523f, b2 = 0.01f, b3 = 0.4798896504144996f, b4 = 1.379008574103742f,
                b5 = -3.290069515436081f, b6 = 2.324710524099774f;
// continuous extension (r_i2, r_i3, r_i4); r_11 = 1
constexpr float r12 = -2.763706197274826f, r13 = 2.9132554618219126f, r14 = -1.0530884977290216f;
constexpr float r22 = 0.1317f, r23 = -0.2234f, r24 = 0.1017f;
constexpr float r32 = 3.9302962368947516f, r33 = -5.941033872131505f, r34 = 2.490627285651253f;
constexpr float r42 = -12.411077166933676f, r43 = 30.33818863028232f, r44 = -16.548102889244902f;
constexpr float r52 = 37.50931341651104f, r53 = -88.1789048947664f, r54 = 47.37952196281928f;
constexpr float r62 = -27.896526289197286f, r63 = 65.09189467479366f, r64 = -34.87065786149661f;
constexpr float r72 = 1.5f, r73 = -4.0f, r74 = 2.5f;
// error weights d_i = b_i - bhat_i of the embedded 4th-order solution: the
// minimum-norm weights satisfying the order-4 conditions, derived by
// oracle/tsit5_coefficients.py (the conditions leave one free parameter)
constexpr float d1 = 0x1.44f608p-7f, d2 = 0x1.2a1940p-8f, d3 = -0x1.67af8ep-5f, d4 = 0x1.9cca80p-1f,
                d5 = -0x1.9f4bdcp+1f, d6 = 0x1.46ac0cp+1f, d7 = -0x1.59c28ep-4f;
}  // namespace ts5

// One step from u with k[0] = f(u) on entry; on exit k[0..6] are the seven
// stages, (n0, n1) = u + dt sum_i b_i k_i and k[6] = f(n) (the next step's k[0]).
// Stage sums are formed left to right with fused multiply-adds.
template <int MODEL>
__device__ __forceinline__ void tsit5_step(const float* p, float l, float dt, float u0, float u1, float (&ka)[7],
                                           float (&kb)[7], float& n0, float& n1) {
  using namespace ts5;
  float sa, sb;
  sa = __fmul_rn(a21, ka[0]);
  sb = __fmul_rn(a21, kb[0]);
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, sa, u0), __fmaf_rn(dt, sb, u1), ka[1], kb[1]);
  sa = __fmaf_rn(a32, ka[1], __fmul_rn(a31, ka[0]));
  sb = __fmaf_rn(a32, kb[1], __fmul_rn(a31, kb[0]));
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, sa, u0), __fmaf_rn(dt, sb, u1), ka[2], kb[2]);
  sa = __fmaf_rn(a43, ka[2], __fmaf_rn(a42, ka[1], __fmul_rn(a41, ka[0])));
  sb = __fmaf_rn(a43, kb[2], __fmaf_rn(a42, kb[1], __fmul_rn(a41, kb[0])));
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, sa, u0), __fmaf_rn(dt, sb, u1), ka[3], kb[3]);
  sa = __fmaf_rn(a54, ka[3], __fmaf_rn(a53, ka[2], __fmaf_rn(a52, ka[1], __fmul_rn(a51, ka[0]))));
  sb = __fmaf_rn(a54, kb[3], __fmaf_rn(a53, kb[2], __fmaf_rn(a52, kb[1], __fmul_rn(a51, kb[0]))));
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, sa, u0), __fmaf_rn(dt, sb, u1), ka[4], kb[4]);
  sa = __fmaf_rn(a65, ka[4],
                 __fmaf_rn(a64, ka[3], __fmaf_rn(a63, ka[2], __fmaf_rn(a62, ka[1], __fmul_rn(a61, ka[0])))));
  sb = __fmaf_rn(a65, kb[4],
                 __fmaf_rn(a64, kb[3], __fmaf_rn(a63, kb[2], __fmaf_rn(a62, kb[1], __fmul_rn(a61, kb[0])))));
  ode_rhs<MODEL>(p, l, __fmaf_rn(dt, sa, u0), __fmaf_rn(dt, sb, u1), ka[5], kb[5]);
  sa = __fmaf_rn(b6, ka[5], __fmaf_rn(b5, ka[4], __fmaf_rn(b4, ka[3],
                 __fmaf_rn(b3, ka[2], __fmaf_rn(b2, ka[1], __fmul_rn(b1, ka[0]))))));
  sb = __fmaf_rn(b6, kb[5], __fmaf_rn(b5, kb[4], __fmaf_rn(b4, kb[3],
                 __fmaf_rn(b3, kb[2], __fmaf_rn(b2, kb[1], __fmul_rn(b1, kb[0]))))));
  n0 = __fmaf_rn(dt, sa, u0);
  n1 = __fmaf_rn(dt, sb, u1);
  ode_rhs<MODEL>(p, l, n0, n1, ka[6], kb[6]);
}

// b_i(theta) = theta^2 (r_i2 + theta (r_i3 + theta r_i4)), i >= 2, by Horner's rule
__device__ __forceinline__ float tsit5_weight(float th, float th2, float r2, float r3, float r4) {
  return __fmul_rn(th2, __fmaf_rn(th, __fmaf_rn(th, r4, r3), r2));
}

// u + dt sum_i b_i(theta) k_i
__device__ __forceinline__ float tsit5_dense(float u, float dt, float th, const float (&k)[7]) {
  using namespace ts5;
  const float th2 = __fmul_rn(th, th);
  const float w1 = __fmul_rn(th, __fmaf_rn(th, __fmaf_rn(th, __fmaf_rn(th, r14, r13), r12), 1.0f));
  float s = __fmul_rn(w1, k[0]);
  s = __fmaf_rn(tsit5_weight(th, th2, r22, r23, r24), k[1], s);
  s = __fmaf_rn(tsit5_weight(th, th2, r32, r33, r34), k[2], s);
  s = __fmaf_rn(tsit5_weight(th, th2, r42, r43, r44), k[3], s);
  s = __fmaf_rn(tsit5_weight(th, th2, r52, r53, r54), k[4], s);
  s = __fmaf_rn(tsit5_weight(th, th2, r62, r63, r64), k[5], s);
  s = __fmaf_rn(tsit5_weight(th, th2, r72, r73, r74), k[6], s);
  return __fmaf_rn(dt, s, u);
}

// The fixed-step saves of a Tsit5 fit, shared by all its particles: save m
// falls in step n(m), the first step whose end t_n+1 = (n+1) dt reaches
// t_m = m save_dt, at theta = (t_m - t_n) / dt, so its continuous-extension
// weights b_i(theta) are the same for every particle.  Row m (m >= 1) of the
// table: n(m) (as int bits), then b_1..b_7(theta); saves past the last step
// get n(m) = nsteps (never reached, as in the step loop).  Built by all threads
// of a block before the particles' integrations (8 nsaves floats of shared
// memory); each weight is the operation sequence tsit5_dense performs.
__device__ __forceinline__ void tsit5_table_build(const OdeCfg& c, float* tab) {
  using namespace ts5;
  const float dt = c.dt;
  for (int m = 1 + (int)threadIdx.x; m < c.nsaves; m += (int)blockDim.x) {
    const float tm = __fmul_rn(__int2float_rn(m), c.save_dt);
    // the smallest n with tm <= (n + 1) dt: an estimate, then corrected
    int n = (int)__fdiv_rn(tm, dt) - 1;
    if (n < 0) n = 0;
    while (n > 0 && tm <= __fmul_rn(__int2float_rn(n), dt)) --n;
    while (n < c.nsteps && tm > __fmul_rn(__int2float_rn(n + 1), dt)) ++n;
    const float tn = __fmul_rn(__int2float_rn(n), dt);
    const float th = __fdiv_rn(__fsub_rn(tm, tn), dt);
    const float th2 = __fmul_rn(th, th);
    float* row = tab + 8 * m;
    row[0] = __int_as_float(n);
    row[1] = __fmul_rn(th, __fmaf_rn(th, __fmaf_rn(th, __fmaf_rn(th, r14, r13), r12), 1.0f));
    row[2] = tsit5_weight(th, th2, r22, r23, r24);
    row[3] = tsit5_weight(th, th2, r32, r33, r34);
    row[4] = tsit5_weight(th, th2, r42, r43, r44);
    row[5] = tsit5_weight(th, th2, r52, r53, r54);
    row[6] = tsit5_weight(th, th2, r62, r63, r64);
    row[7] = tsit5_weight(th, th2, r72, r73, r74);
  }
}

// u + dt sum_i w_i k_i with the weights of a table row (tsit5_dense's sums)
__device__ __forceinline__ float tsit5_dense_w(float u, float dt, const float* w, const float (&k)[7]) {
  float s = __fmul_rn(w[0], k[0]);
#pragma unroll
  for (int i = 1; i < 7; ++i) s = __fmaf_rn(w[i], k[i], s);
  return __fmaf_rn(dt, s, u);
}

// tsit5_loss with the saves' weights from the table: the same operations
template <int MODEL>
__device__ __forceinline__ float tsit5_loss_tab(const float* p, const OdeCfg& c, const float* data, const float* tab) {
  const float dt = c.dt;
  float u0 = c.u0a, u1 = c.u0b;
  float e0 = __fsub_rn(data[0], u0), e1 = __fsub_rn(data[1], u1);
  float acc = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
  const float l = ode_l(p, c);
  float ka[7], kb[7];
  ode_rhs<MODEL>(p, l, u0, u1, ka[0], kb[0]);
  int m = 1;
  for (int n = 0; n < c.nsteps && m < c.nsaves; ++n) {
    float n0, n1;
    tsit5_step<MODEL>(p, l, dt, u0, u1, ka, kb, n0, n1);
    while (m < c.nsaves && __float_as_int(tab[8 * m]) == n) {  // the saves inside (t_n, t_n+1]
      const float* w = tab + 8 * m + 1;
      e0 = __fsub_rn(data[2 * m], tsit5_dense_w(u0, dt, w, ka));
      e1 = __fsub_rn(data[2 * m + 1], tsit5_dense_w(u1, dt, w, kb));
      acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
      ++m;
    }
    u0 = n0;
    u1 = n1;
    ka[0] = ka[6];
    kb[0] = kb[6];
  }
  return acc;
}

// SSE of the Tsit5 solution at t_m = m save_dt (m < nsaves) against data
template <int MODEL>
__device__ __forceinline__ float tsit5_loss(const float* p, const OdeCfg& c, const float* data) {
  const float dt = c.dt;
  float u0 = c.u0a, u1 = c.u0b;
  float e0 = __fsub_rn(data[0], u0), e1 = __fsub_rn(data[1], u1);
  float acc = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
  const float l = ode_l(p, c);
  float ka[7], kb[7];
  ode_rhs<MODEL>(p, l, u0, u1, ka[0], kb[0]);
  int m = 1;
  float tm = c.save_dt;
  for (int n = 0; n < c.nsteps && m < c.nsaves; ++n) {
    const float tn = __fmul_rn(__int2float_rn(n), dt);
    const float tn1 = __fmul_rn(__int2float_rn(n + 1), dt);
    float n0, n1;
    tsit5_step<MODEL>(p, l, dt, u0, u1, ka, kb, n0, n1);
    while (m < c.nsaves && tm <= tn1) {  // the saves inside (t_n, t_n+1]
      const float th = __fdiv_rn(__fsub_rn(tm, tn), dt);
      e0 = __fsub_rn(data[2 * m], tsit5_dense(u0, dt, th, ka));
      e1 = __fsub_rn(data[2 * m + 1], tsit5_dense(u1, dt, th, kb));
      acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
      ++m;
      tm = __fmul_rn(__int2float_rn(m), c.save_dt);
    }
    u0 = n0;
    u1 = n1;
    ka[0] = ka[6];
    kb[0] = kb[6];
  }
  return acc;
}

// ---------------------------------------------------------------- adaptive Tsit5
// The reference's parameter_estim_ode!(..., Val(true)) integrates with
// DiffEqGPU's vectorized_asolve (src/ode_pso.jl:54-111): adaptive steps,
// saves interpolated.  Restated from the published methods:
//   - local error estimate E = h sum_i d_i k_i of the embedded 4th-order
//     solution (d above), measured as err = sqrt(((E_1/sc_1)^2 + (E_2/sc_2)^2) / 2)
//     with sc = abstol + reltol max(|u_n|, |u_n+1|) (Hairer, Norsett & Wanner,
//     Solving ODEs I, sec. II.4, eq. 4.11);
//   - step accepted when err <= 1; the next step h fac with the stabilised
//     (PI) controller of the same section (Gustafsson's): fac = 0.9 err^-alpha
//     err_old^beta, beta = 0.04, alpha = 1/5 - 0.75 beta, clamped to [0.2, 10]
//     (at most 1 right after a rejection), err_old = max(err, 1e-4) of the last
//     accepted step (1e-4 at the start); a rejected step retries with
//     h max(0.2, 0.9 err^-1/5);
//   - the last step ends exactly at t_end = (nsaves - 1) save_dt; saves inside
//     an accepted step come from the continuous extension, as at a fixed step;
//   - at most kOdeMaxSteps steps, and a step that no longer advances t, give
//     a loss of +inf (a solve that did not finish).
// err^-alpha is exp_f(-alpha log_f(err)) (both this project's own), so the
// oracle reproduces every step size bit for bit.
constexpr float kCtlBeta = 0.04f, kCtlAlpha = 0.17f, kCtlSafe = 0.9f;
constexpr float kCtlFacMin = 0.2f, kCtlFacMax = 10.0f, kCtlErrMin = 1e-4f;

__device__ __forceinline__ float tsit5_err_sum(const float (&k)[7]) {
  using namespace ts5;
  float s = __fmul_rn(d1, k[0]);
  s = __fmaf_rn(d2, k[1], s);
  s = __fmaf_rn(d3, k[2], s);
  s = __fmaf_rn(d4, k[3], s);
  s = __fmaf_rn(d5, k[4], s);
  s = __fmaf_rn(d6, k[5], s);
  return __fmaf_rn(d7, k[6], s);
}

// SSE of the adaptive Tsit5 solution at t_m = m save_dt against data; steps
// (accepted and rejected) in *steps when given
template <int MODEL>
__device__ __forceinline__ float tsit5a_loss(const float* p, const OdeCfg& c, const float* data, int* steps = nullptr) {
  const float inf = __int_as_float(0x7f800000);
  float u0 = c.u0a, u1 = c.u0b;
  float e0 = __fsub_rn(data[0], u0), e1 = __fsub_rn(data[1], u1);
  float acc = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
  const float l = ode_l(p, c);
  const float tend = __fmul_rn(__int2float_rn(c.nsaves - 1), c.save_dt);
  float ka[7], kb[7];
  ode_rhs<MODEL>(p, l, u0, u1, ka[0], kb[0]);
  float t = 0.0f, h = c.dt, errold = kCtlErrMin;
  bool rejected = false;
  int m = 1, n = 0;
  float tm = c.save_dt;
  for (; m < c.nsaves; ++n) {
    if (n >= kOdeMaxSteps) {
      acc = inf;
      break;
    }
    const float rem = __fsub_rn(tend, t);
    const bool last = h >= rem;
    const float hh = last ? rem : h;
    const float tn1 = last ? tend : __fadd_rn(t, hh);
    if (!(tn1 > t)) {  // the step no longer advances t
      acc = inf;
      break;
    }
    float n0, n1;
    tsit5_step<MODEL>(p, l, hh, u0, u1, ka, kb, n0, n1);
    const float ea = __fmul_rn(hh, tsit5_err_sum(ka)), eb = __fmul_rn(hh, tsit5_err_sum(kb));
    const float sa = __fmaf_rn(c.rtol, fmaxf(fabsf(u0), fabsf(n0)), c.atol);
    const float sb = __fmaf_rn(c.rtol, fmaxf(fabsf(u1), fabsf(n1)), c.atol);
    const float ra = __fdiv_rn(ea, sa), rb = __fdiv_rn(eb, sb);
    const float err = __fsqrt_rn(__fmul_rn(__fmaf_rn(ra, ra, __fmul_rn(rb, rb)), 0.5f));
    if (err <= 1.0f) {
      while (m < c.nsaves && tm <= tn1) {  // the saves inside (t, t + hh]
        const float th = __fdiv_rn(__fsub_rn(tm, t), hh);
        e0 = __fsub_rn(data[2 * m], tsit5_dense(u0, hh, th, ka));
        e1 = __fsub_rn(data[2 * m + 1], tsit5_dense(u1, hh, th, kb));
        acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
        ++m;
        tm = __fmul_rn(__int2float_rn(m), c.save_dt);
      }
      t = tn1;
      u0 = n0;
      u1 = n1;
      ka[0] = ka[6];
      kb[0] = kb[6];
      float fac = kCtlFacMax;
      if (err > 0.0f)
        fac = __fmul_rn(kCtlSafe, exp_f(__fmaf_rn(kCtlBeta, log_f(errold), __fmul_rn(-kCtlAlpha, log_f(err)))));
      fac = fminf(rejected ? 1.0f : kCtlFacMax, fmaxf(kCtlFacMin, fac));
      errold = fmaxf(err, kCtlErrMin);
      h = __fmul_rn(hh, fac);
      rejected = false;
    } else {
      const float fac = fmaxf(kCtlFacMin, __fmul_rn(kCtlSafe, exp_f(__fmul_rn(-0.2f, log_f(err)))));
      h = __fmul_rn(hh, fac);
      rejected = true;
    }
  }
  if (steps) *steps = n;
  return acc;
}

}  // namespace pps
