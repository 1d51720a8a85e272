// Device routine shared by the derivative kernels and the FP64 residual of
// the solver: one quasi-pentadiagonal compact-scheme line solve,
//   y = L^-1 (R x + boundary terms),
// with L given by its pentalu factors and R by a 7-wide explicit stencil
// (rows 1,2 on x(1..7), rows n-1,n on x(n-6..n), 5 points in between).
// Restates derx_rhs + pentares (class_derivatives.f90:262-295,425-466).
#pragma once

namespace mf {

// Packed per-row coefficients: p, f, 1/c, d, e, r[0..6].
constexpr int kRow = 12;

struct LineSet {
  const double* __restrict__ c;  // n rows of kRow doubles
  int n;
};

// Boundary contributions folded into rows 1, 2, n-1, n of the right-hand side.
struct LineBC {
  double lo = 0.0, hi = 0.0;      // boundary values at both ends
  double c0 = 0.0, c1 = 0.0;      // coefficients of `lo` in rows 1, 2
  double c2 = 0.0, c3 = 0.0;      // coefficients of `hi` in rows n-1, n
};

// Default final store: out(i) = y.
struct StorePlain {
  __device__ __forceinline__ void operator()(double* out, long long idx, double y) const {
    out[idx] = y;
  }
};

// Solves one pencil.  `in` and `out` may alias: every input value is read
// before the store that could overwrite it.  The forward-elimination values
// are parked in `out` and read back by the back substitution, whose result
// goes through `fin(out, index, y)`.
template <class Fin>
__device__ __forceinline__ void solve_line(const double* __restrict__ C, int n, const double* in,
                                           double* out, long long s, const LineBC& bc,
                                           const Fin& fin) {
  const double f0 = in[0], f1 = in[s], f2 = in[2 * s], f3 = in[3 * s], f4 = in[4 * s],
               f5 = in[5 * s], f6 = in[6 * s];
  const double g0 = in[(long long)(n - 7) * s], g1 = in[(long long)(n - 6) * s],
               g2 = in[(long long)(n - 5) * s], g3 = in[(long long)(n - 4) * s],
               g4 = in[(long long)(n - 3) * s], g5 = in[(long long)(n - 2) * s],
               g6 = in[(long long)(n - 1) * s];
  const double* c0 = C;
  const double* c1 = C + kRow;
  const double x0 = c0[5] * f0 + c0[6] * f1 + c0[7] * f2 + c0[8] * f3 + c0[9] * f4 +
                    c0[10] * f5 + c0[11] * f6 + bc.c0 * bc.lo;
  const double b1 = c1[5] * f0 + c1[6] * f1 + c1[7] * f2 + c1[8] * f3 + c1[9] * f4 +
                    c1[10] * f5 + c1[11] * f6 + bc.c1 * bc.lo;
  const double x1 = b1 - x0 * c1[1];
  out[0] = x0;
  out[s] = x1;
  double xm2 = x0, xm1 = x1;
  double w0 = f0, w1 = f1, w2 = f2, w3 = f3, w4 = f4;
  for (int i = 2; i < n - 2; ++i) {
    const double* c = C + kRow * i;
    const double b = c[5] * w0 + c[6] * w1 + c[7] * w2 + c[8] * w3 + c[9] * w4;
    const double x = b - c[0] * xm2 - c[1] * xm1;
    w0 = w1; w1 = w2; w2 = w3; w3 = w4;
    if (i + 3 < n) w4 = in[(long long)(i + 3) * s];
    out[(long long)i * s] = x;
    xm2 = xm1;
    xm1 = x;
  }
  const double* cA = C + kRow * (n - 2);
  const double* cB = C + kRow * (n - 1);
  const double bA = cA[5] * g0 + cA[6] * g1 + cA[7] * g2 + cA[8] * g3 + cA[9] * g4 +
                    cA[10] * g5 + cA[11] * g6 + bc.c2 * bc.hi;
  const double xA = bA - cA[0] * xm2 - cA[1] * xm1;
  const double bB = cB[5] * g0 + cB[6] * g1 + cB[7] * g2 + cB[8] * g3 + cB[9] * g4 +
                    cB[10] * g5 + cB[11] * g6 + bc.c3 * bc.hi;
  const double xB = bB - cB[0] * xm1 - cB[1] * xA - cB[4] * xm2;  // e(n) holds beta
  const double yB = xB * cB[2];
  const double yA = (xA - cA[3] * yB) * cA[2];
  fin(out, (long long)(n - 1) * s, yB);
  fin(out, (long long)(n - 2) * s, yA);
  double y2 = yB, y1 = yA, y3 = 0.0;
  for (int i = n - 3; i >= 1; --i) {
    const double* c = C + kRow * i;
    const double y = (out[(long long)i * s] - c[4] * y2 - c[3] * y1) * c[2];
    fin(out, (long long)i * s, y);
    y3 = y2;
    y2 = y1;
    y1 = y;
  }
  const double y0 = (out[0] - c0[4] * y2 - c0[3] * y1 - c0[0] * y3) * c0[2];
  fin(out, 0, y0);
}

}  // namespace mf
