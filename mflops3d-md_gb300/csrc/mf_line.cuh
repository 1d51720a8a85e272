// Device routine shared by the derivative kernels and the residuals of the
// solver's iterative refinement: one quasi-pentadiagonal compact-scheme line
// solve,
//   y = L^-1 (R x + boundary terms),
// with L given by its pentalu factors and R by a 7-wide explicit stencil
// (rows 1,2 on x(1..7), rows n-1,n on x(n-6..n), 5 points in between).
// Restates derx_rhs + pentares (class_derivatives.f90:262-295,425-466).
//
// T is the arithmetic type (double for the FP64 paths, float for the
// correction residual); In is the storage type of the line being
// differentiated (a float input is widened exactly to double).
#pragma once
#include <cstdint>

namespace mf {

// Packed per-row coefficients: p, f, 1/c, d, e, r[0..6].
constexpr int kRow = 12;

template <class T>
struct LineSetT {
  const T* __restrict__ c;  // n rows of kRow values
  int n;
};
using LineSet = LineSetT<double>;

// Boundary contributions folded into rows 1, 2, n-1, n of the right-hand side.
template <class T>
struct LineBCT {
  T lo = 0, hi = 0;  // boundary values at both ends
  T c0 = 0, c1 = 0;  // coefficients of `lo` in rows 1, 2
  T c2 = 0, c3 = 0;  // coefficients of `hi` in rows n-1, n
};
using LineBC = LineBCT<double>;

// Exact float -> double widening built from the bit fields (integer pipe;
// GB300's conversion unit shares the narrow FP64 rate).  Subnormal floats
// flush to signed zero, infinities and NaN keep their class.
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint64_t sgn = (uint64_t)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sgn);
  const uint64_t exp = (e == 0xFFu) ? 0x7FFull : (uint64_t)(e + 896u);
  return __longlong_as_double((long long)(sgn | (exp << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29)));
}

// FP64 -> FP32 rounded to nearest even from the bit fields (integer pipe).
// Results below the normal FP32 range flush to signed zero, overflow gives
// infinity, NaN stays NaN.
__device__ __forceinline__ float narrow(double d) {
  const uint64_t u = (uint64_t)__double_as_longlong(d);
  const uint32_t sgn = (uint32_t)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7FF);
  const uint64_t m = u & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sgn | 0x7F800000u | (m ? 0x400000u : 0u));
  const int ef = e - 1023 + 127;
  if (ef <= 0) return __uint_as_float(sgn);
  if (ef >= 255) return __uint_as_float(sgn | 0x7F800000u);
  uint32_t r = ((uint32_t)ef << 23) | (uint32_t)(m >> 29);
  const uint32_t rest = (uint32_t)(m & 0x1FFFFFFFu);
  if (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ++r;  // may carry into the exponent
  return __uint_as_float(sgn | r);
}

template <class T, class In>
__device__ __forceinline__ T load_as(const In* p, long long i);
template <>
__device__ __forceinline__ double load_as<double, double>(const double* p, long long i) { return p[i]; }
template <>
__device__ __forceinline__ double load_as<double, float>(const float* p, long long i) { return widen(p[i]); }
template <>
__device__ __forceinline__ float load_as<float, float>(const float* p, long long i) { return p[i]; }

// Default final store: out(i) = y.  Final-store functors receive the row
// index i, the element offset idx = i*s of the row in the line, and y.
struct StorePlain {
  template <class T>
  __device__ __forceinline__ void operator()(T* out, int, long long idx, T y) const {
    out[idx] = y;
  }
};

// Right-hand-side evaluators of one row: plain products, or the compensated
// form (see CompSum below) for the FP32 correction residual.
template <class T>
struct PlainStencil {
  __device__ __forceinline__ T row5(const T* c, T w0, T w1, T w2, T w3, T w4) const {
    return c[5] * w0 + c[6] * w1 + c[7] * w2 + c[8] * w3 + c[9] * w4;
  }
  __device__ __forceinline__ T row7(const T* c, T a0, T a1, T a2, T a3, T a4, T a5, T a6) const {
    return c[5] * a0 + c[6] * a1 + c[7] * a2 + c[8] * a3 + c[9] * a4 + c[10] * a5 + c[11] * a6;
  }
};

// ---------------------------------------------------------------------------
// Compensated FP32 stencil.
//
// On smooth data a second-difference stencil with coefficients ~1/h^2
// cancels by 1e4-1e5 on a stretched 257-node line, so plain FP32 (and the
// FP32 rounding of the coefficients) loses most digits.  Here each product
// c*x is formed exactly (hi part by the FMA two-product, plus the lo part of
// the coefficient) and summed with TwoSum compensation; only the result of
// the cancellation is rounded to FP32.  The triangular sweeps that follow are
// well conditioned and run in plain FP32.
// Row layout: p, f, 1/c, d, e, r_hi[0..6], r_lo[0..6].
constexpr int kRowF = 19;

struct CompSum {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add(float chi, float clo, float x) {
    const float p = chi * x;
    const float pe = fmaf(chi, x, -p);
    const float t = s + p;
    const float bb = t - s;
    const float te = (s - (t - bb)) + (p - bb);
    s = t;
    e += te + pe + clo * x;
  }
  __device__ __forceinline__ float value() const { return s + e; }
};

struct CompStencil {
  __device__ __forceinline__ float row5(const float* c, float w0, float w1, float w2, float w3,
                                        float w4) const {
    CompSum cs;
    cs.add(c[5], c[12], w0);
    cs.add(c[6], c[13], w1);
    cs.add(c[7], c[14], w2);
    cs.add(c[8], c[15], w3);
    cs.add(c[9], c[16], w4);
    return cs.value();
  }
  __device__ __forceinline__ float row7(const float* c, float a0, float a1, float a2, float a3,
                                        float a4, float a5, float a6) const {
    CompSum cs;
    cs.add(c[5], c[12], a0);
    cs.add(c[6], c[13], a1);
    cs.add(c[7], c[14], a2);
    cs.add(c[8], c[15], a3);
    cs.add(c[9], c[16], a4);
    cs.add(c[10], c[17], a5);
    cs.add(c[11], c[18], a6);
    return cs.value();
  }
};

// Loads issued this many steps ahead of their use in both sweeps (register
// ring), so that one thread's walk along its line is not serialised on the
// memory latency of every step.
constexpr int kAhead = 8;

// Solves one pencil.  `in` and `out` may alias (same type): every input
// value is read before the store that could overwrite it.  The
// forward-elimination values are parked in `out` and read back by the back
// substitution, whose result goes through `fin(out, i, index, y)`.
// R is the row stride of the packed coefficients C.
template <int R, class T, class In, class Fin, class St>
__device__ __forceinline__ void solve_line_impl(const T* __restrict__ C, int n, const In* in, T* out,
                                                long long s, const LineBCT<T>& bc, const Fin& fin,
                                                const St& st) {
  const T f0 = load_as<T, In>(in, 0), f1 = load_as<T, In>(in, s), f2 = load_as<T, In>(in, 2 * s),
          f3 = load_as<T, In>(in, 3 * s), f4 = load_as<T, In>(in, 4 * s),
          f5 = load_as<T, In>(in, 5 * s), f6 = load_as<T, In>(in, 6 * s);
  const T g0 = load_as<T, In>(in, (long long)(n - 7) * s), g1 = load_as<T, In>(in, (long long)(n - 6) * s),
          g2 = load_as<T, In>(in, (long long)(n - 5) * s), g3 = load_as<T, In>(in, (long long)(n - 4) * s),
          g4 = load_as<T, In>(in, (long long)(n - 3) * s), g5 = load_as<T, In>(in, (long long)(n - 2) * s),
          g6 = load_as<T, In>(in, (long long)(n - 1) * s);
  const T* c0 = C;
  const T* c1 = C + R;
  const T x0 = st.row7(c0, f0, f1, f2, f3, f4, f5, f6) + bc.c0 * bc.lo;
  const T x1 = st.row7(c1, f0, f1, f2, f3, f4, f5, f6) + bc.c1 * bc.lo - x0 * c1[1];
  out[0] = x0;
  out[s] = x1;
  T xm2 = x0, xm1 = x1;
  T w0 = f0, w1 = f1, w2 = f2, w3 = f3, w4 = f4;
  // forward sweep, rows 2 .. n-3; pf[u] = in(i + 3 + u)
  T pf[kAhead];
#pragma unroll
  for (int u = 0; u < kAhead; ++u) pf[u] = (5 + u < n) ? load_as<T, In>(in, (long long)(5 + u) * s) : T(0);
  int i = 2;
  for (; i + kAhead <= n - 2; i += kAhead) {
    T nb[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const int j = i + 3 + kAhead + u;
      nb[u] = (j < n) ? load_as<T, In>(in, (long long)j * s) : T(0);
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const T* c = C + R * (i + u);
      const T x = st.row5(c, w0, w1, w2, w3, w4) - c[0] * xm2 - c[1] * xm1;
      w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = pf[u];
      out[(long long)(i + u) * s] = x;
      xm2 = xm1;
      xm1 = x;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) pf[u] = nb[u];
  }
  for (; i < n - 2; ++i) {
    const T* c = C + R * i;
    const T x = st.row5(c, w0, w1, w2, w3, w4) - c[0] * xm2 - c[1] * xm1;
    w0 = w1; w1 = w2; w2 = w3; w3 = w4;
    if (i + 3 < n) w4 = load_as<T, In>(in, (long long)(i + 3) * s);
    out[(long long)i * s] = x;
    xm2 = xm1;
    xm1 = x;
  }
  const T* cA = C + R * (n - 2);
  const T* cB = C + R * (n - 1);
  const T xA = st.row7(cA, g0, g1, g2, g3, g4, g5, g6) + bc.c2 * bc.hi - cA[0] * xm2 - cA[1] * xm1;
  const T xB = st.row7(cB, g0, g1, g2, g3, g4, g5, g6) + bc.c3 * bc.hi - cB[0] * xm1 - cB[1] * xA -
               cB[4] * xm2;  // e(n) holds beta
  // back substitution; rb[u] = forward value of row i - u
  const T yB = xB * cB[2];
  const T yA = (xA - cA[3] * yB) * cA[2];
  fin(out, n - 1, (long long)(n - 1) * s, yB);
  fin(out, n - 2, (long long)(n - 2) * s, yA);
  T y2 = yB, y1 = yA, y3 = 0;
  i = n - 3;
  T rb[kAhead];
#pragma unroll
  for (int u = 0; u < kAhead; ++u) rb[u] = (i - u >= 1) ? out[(long long)(i - u) * s] : T(0);
  for (; i - (kAhead - 1) >= 1; i -= kAhead) {
    T nb[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const int j = i - kAhead - u;
      nb[u] = (j >= 1) ? out[(long long)j * s] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const T* c = C + R * (i - u);
      const T y = (rb[u] - c[4] * y2 - c[3] * y1) * c[2];
      fin(out, i - u, (long long)(i - u) * s, y);
      y3 = y2;
      y2 = y1;
      y1 = y;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) rb[u] = nb[u];
  }
  for (; i >= 1; --i) {
    const T* c = C + R * i;
    const T y = (out[(long long)i * s] - c[4] * y2 - c[3] * y1) * c[2];
    fin(out, i, (long long)i * s, y);
    y3 = y2;
    y2 = y1;
    y1 = y;
  }
  const T y0 = (out[0] - c0[4] * y2 - c0[3] * y1 - c0[0] * y3) * c0[2];
  fin(out, 0, 0, y0);
}

// ---------------------------------------------------------------------------
// Tridiagonal lines with 1/c folded into the rows.
//
// When the factored implicit part is tridiagonal (p = e = alpha = beta = 0,
// the compact schemes of order <= 6), x~_i = x_i / c_i turns the sweeps into
//   x~_i = sum_m w_m f_{j_m} - ft_i x~_{i-1},   y_i = x~_i - dt_i y_{i+1},
// with w_m = r_m / c_i, ft_i = f_i c_{i-1} / c_i, dt_i = d_i / c_i: one FMA
// per sweep instead of two plus a multiply.
struct DerTriRow {
  double w[7];   // explicit stencil / c_i, order of the packed rows
  double ft, dt;
};

// Same contract as solve_line (in and out may alias: every input value is
// read before the store that could overwrite it), plain final store.
__device__ __forceinline__ void solve_line_tri_d(const DerTriRow* __restrict__ R, int n,
                                                 const double* in, double* out, long long s) {
  double f[7], g[7];
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    f[m] = in[(long long)m * s];
    g[m] = in[(long long)(n - 7 + m) * s];
  }
  auto row7 = [](const DerTriRow& r, const double (&v)[7]) {
    double a = r.w[0] * v[0];
#pragma unroll
    for (int m = 1; m < 7; ++m) a = fma(r.w[m], v[m], a);
    return a;
  };
  const double x0 = row7(R[0], f);
  const double x1 = fma(-R[1].ft, x0, row7(R[1], f));
  out[0] = x0;
  out[s] = x1;
  double xm = x1;
  double w0 = f[0], w1 = f[1], w2 = f[2], w3 = f[3], w4 = f[4];
  double pf[kAhead];
#pragma unroll
  for (int u = 0; u < kAhead; ++u) pf[u] = (5 + u < n) ? in[(long long)(5 + u) * s] : 0.0;
  int i = 2;
  for (; i + kAhead <= n - 2; i += kAhead) {
    double nb[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const int j = i + 3 + kAhead + u;
      nb[u] = (j < n) ? in[(long long)j * s] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const DerTriRow& r = R[i + u];
      double a = r.w[0] * w0;
      a = fma(r.w[1], w1, a);
      a = fma(r.w[2], w2, a);
      a = fma(r.w[3], w3, a);
      a = fma(r.w[4], w4, a);
      const double x = fma(-r.ft, xm, a);
      w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = pf[u];
      out[(long long)(i + u) * s] = x;
      xm = x;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) pf[u] = nb[u];
  }
  for (; i < n - 2; ++i) {
    const DerTriRow& r = R[i];
    double a = r.w[0] * w0;
    a = fma(r.w[1], w1, a);
    a = fma(r.w[2], w2, a);
    a = fma(r.w[3], w3, a);
    a = fma(r.w[4], w4, a);
    const double x = fma(-r.ft, xm, a);
    w0 = w1; w1 = w2; w2 = w3; w3 = w4;
    if (i + 3 < n) w4 = in[(long long)(i + 3) * s];
    out[(long long)i * s] = x;
    xm = x;
  }
  const DerTriRow& rA = R[n - 2];
  const DerTriRow& rB = R[n - 1];
  const double xA = fma(-rA.ft, xm, row7(rA, g));
  const double xB = fma(-rB.ft, xA, row7(rB, g));
  // back substitution; rb[u] = forward value of row i - u
  out[(long long)(n - 1) * s] = xB;
  double y1 = fma(-rA.dt, xB, xA);
  out[(long long)(n - 2) * s] = y1;
  i = n - 3;
  double rb[kAhead];
#pragma unroll
  for (int u = 0; u < kAhead; ++u) rb[u] = (i - u >= 0) ? out[(long long)(i - u) * s] : 0.0;
  for (; i - (kAhead - 1) >= 0; i -= kAhead) {
    double nb[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const int j = i - kAhead - u;
      nb[u] = (j >= 0) ? out[(long long)j * s] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const double y = fma(-R[i - u].dt, y1, rb[u]);
      out[(long long)(i - u) * s] = y;
      y1 = y;
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) rb[u] = nb[u];
  }
  for (; i >= 0; --i) {
    const double y = fma(-R[i].dt, y1, out[(long long)i * s]);
    out[(long long)i * s] = y;
    y1 = y;
  }
}

template <class T, class In, class Fin>
__device__ __forceinline__ void solve_line(const T* __restrict__ C, int n, const In* in, T* out,
                                           long long s, const LineBCT<T>& bc, const Fin& fin) {
  solve_line_impl<kRow>(C, n, in, out, s, bc, fin, PlainStencil<T>());
}

template <class Fin>
__device__ __forceinline__ void solve_line_comp(const float* __restrict__ C, int n, const float* in,
                                                float* out, long long s, const Fin& fin) {
  solve_line_impl<kRowF>(C, n, in, out, s, LineBCT<float>(), fin, CompStencil());
}

}  // namespace mf
