"""Sources of user objectives shared by the CPU and GPU tests.

Each is the CUDA C of pps_objective_register and, with the oracle's prefix,
plain C for the CPU restatement.  ROSENBROCK and RASTRIGIN spell the
registered objectives' operations in the same order (src/kernels.jl:33 with
f from test/regression.jl:12-18 and the Rastrigin formula), so a swarm over
them reproduces the registered swarm bit for bit."""

HEAD = "PPS_DEVICE float pps_objective(pps_point x, int dim, const float* p, const float* data, long long ndata)"

ROSENBROCK = HEAD + """ {
  float s = 0.0f;
  for (int i = 0; i + 1 < dim; ++i) {
    const float t = x[i + 1] - x[i] * x[i];
    const float u = p[0] - x[i];
    s = s + (p[1] * (t * t) + u * u);
  }
  return s;
}
"""

RASTRIGIN = HEAD + """ {
  float s = 0.0f;
  for (int i = 0; i < dim; ++i) s = s + (x[i] * x[i] - p[0] * pps_cos2pi(x[i]));
  return p[0] * (float)dim + s;
}
"""

SHIFTED_SPHERE = HEAD + """ {
  float s = 0.0f;
  for (int i = 0; i < dim; ++i) {
    const float t = x[i] - (i < 8 ? p[i] : 0.0f);
    s = s + t * t;
  }
  return s;
}
"""

# mean squared residual of a quadratic model y = x0 + x1 t + x2 t^2 over the
# samples data = (t_0..t_{m-1}, y_0..y_{m-1})
POLYFIT = HEAD + """ {
  const long long m = ndata / 2;
  float s = 0.0f;
  for (long long k = 0; k < m; ++k) {
    const float t = data[k];
    const float r = (x[0] + x[1] * t + x[2] * (t * t)) - data[m + k];
    s = s + r * r;
  }
  return s / (float)m;
}
"""

# Styblinski-Tang plus a square-root term: IEEE sqrt on both sides
STYBLINSKI_SQRT = HEAD + """ {
  float s = 0.0f;
  for (int i = 0; i < dim; ++i) {
    const float v = x[i];
    const float v2 = v * v;
    s = s + ((v2 * v2 - 16.0f * v2) + 5.0f * v);
  }
  return 0.5f * s + sqrtf(fabsf(x[0]));
}
"""

# Griewank with the library's cos and a branch on the data
GRIEWANK = HEAD + """ {
  float s = 0.0f, q = 1.0f;
  for (int i = 0; i < dim; ++i) {
    s = s + x[i] * x[i];
    q = q * pps_cos2pi(x[i] / (6.2831855f * sqrtf((float)(i + 1))));
  }
  return (s / 4000.0f - q) + 1.0f;
}
"""

# Rosenbrock with its gradient, both spelled as the registered objective's
# (pps_objgrad.cuh): the HybridPSO local stage on it is the registered one
ROSENBROCK_GRAD = "#define PPS_HAS_GRADIENT 1\n" + ROSENBROCK + """
PPS_DEVICE float pps_gradient(pps_point x, int dim, const float* p, const float* data, long long ndata, float* g) {
  for (int d = 0; d < dim; ++d) {
    float gd = 0.0f;
    if (d < dim - 1) {
      const float t = x[d + 1] - x[d] * x[d];
      gd = ((-4.0f * p[1]) * x[d]) * t - 2.0f * (p[0] - x[d]);
    }
    if (d > 0) {
      const float t = x[d] - x[d - 1] * x[d - 1];
      gd = gd + (2.0f * p[1]) * t;
    }
    g[d] = gd;
  }
  return pps_objective(x, dim, p, data, ndata);
}
"""

# The same objectives with the fold the synchronous step uses instead of
# reading the new position back (PPS_HAS_STREAM): each add performs the
# objective loop's operations for one coordinate, in the same order, so the
# fold equals pps_objective bit for bit.
STREAM_ARGS = "const float* p, const float* data, long long ndata"

RASTRIGIN_STREAM = "#define PPS_HAS_STREAM 1\n" + RASTRIGIN + f"""
typedef struct {{ float s; }} pps_stream;
PPS_DEVICE void pps_stream_start(pps_stream* st, int dim, {STREAM_ARGS}) {{ st->s = 0.0f; }}
PPS_DEVICE void pps_stream_add(pps_stream* st, int d, float v, int dim, {STREAM_ARGS}) {{
  st->s = st->s + (v * v - p[0] * pps_cos2pi(v));
}}
PPS_DEVICE float pps_stream_finish(const pps_stream* st, int dim, {STREAM_ARGS}) {{
  return p[0] * (float)dim + st->s;
}}
"""

ROSENBROCK_STREAM = "#define PPS_HAS_STREAM 1\n" + ROSENBROCK + f"""
typedef struct {{ float s, prev; }} pps_stream;
PPS_DEVICE void pps_stream_start(pps_stream* st, int dim, {STREAM_ARGS}) {{
  st->s = 0.0f;
  st->prev = 0.0f;
}}
PPS_DEVICE void pps_stream_add(pps_stream* st, int d, float v, int dim, {STREAM_ARGS}) {{
  if (d > 0) {{
    const float t = v - st->prev * st->prev;
    const float u = p[0] - st->prev;
    st->s = st->s + (p[1] * (t * t) + u * u);
  }}
  st->prev = v;
}}
PPS_DEVICE float pps_stream_finish(const pps_stream* st, int dim, {STREAM_ARGS}) {{ return st->s; }}
"""

SHIFTED_SPHERE_STREAM = "#define PPS_HAS_STREAM 1\n" + SHIFTED_SPHERE + f"""
typedef struct {{ float s; }} pps_stream;
PPS_DEVICE void pps_stream_start(pps_stream* st, int dim, {STREAM_ARGS}) {{ st->s = 0.0f; }}
PPS_DEVICE void pps_stream_add(pps_stream* st, int d, float v, int dim, {STREAM_ARGS}) {{
  const float t = v - (d < 8 ? p[d] : 0.0f);
  st->s = st->s + t * t;
}}
PPS_DEVICE float pps_stream_finish(const pps_stream* st, int dim, {STREAM_ARGS}) {{ return st->s; }}
"""

# sum_d w_d x_d^2 with the weights w in the problem's data (one per coordinate)
WEIGHTED_SPHERE_STREAM = "#define PPS_HAS_STREAM 1\n" + HEAD + """ {
  float s = 0.0f;
  for (int i = 0; i < dim; ++i) s = s + data[i] * (x[i] * x[i]);
  return s;
}
""" + f"""
typedef struct {{ float s; }} pps_stream;
PPS_DEVICE void pps_stream_start(pps_stream* st, int dim, {STREAM_ARGS}) {{ st->s = 0.0f; }}
PPS_DEVICE void pps_stream_add(pps_stream* st, int d, float v, int dim, {STREAM_ARGS}) {{
  st->s = st->s + data[d] * (v * v);
}}
PPS_DEVICE float pps_stream_finish(const pps_stream* st, int dim, {STREAM_ARGS}) {{ return st->s; }}
"""
