// Host set-up: compact-scheme coefficients, quasi-penta LU, dense inverse and
// a real nonsymmetric eigen-solver.  See mf_setup.h for the reference map.
#include "mf_setup.h"
#include "mflops_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace mf {

bool small_solve(int n, double* a, double* b) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = std::fabs(a[k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      double v = std::fabs(a[i * n + k]);
      if (v > best) { best = v; piv = i; }
    }
    if (best == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[piv * n + j]);
      std::swap(b[k], b[piv]);
    }
    const double inv = 1.0 / a[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double l = a[i * n + k] * inv;
      if (l == 0.0) continue;
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
      b[i] -= l * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
  return true;
}

// Taylor-matching matrix, row-major nt x nt.  Implicit columns hold the
// expansion of the unknown derivative values, explicit columns the function
// values (class_derivatives_coefficient.f90:150-168).
static void taylor_matrix(const double* h, int n1, int nt, int der, double* a) {
  std::fill(a, a + nt * nt, 0.0);
  for (int j = 0; j < n1; ++j) a[der * nt + j] = -1.0;
  for (int i = der + 1; i < nt; ++i)
    for (int j = 0; j < n1; ++j) a[i * nt + j] = a[(i - 1) * nt + j] * h[j] / double(i - der);
  for (int j = n1; j < nt; ++j) a[j] = 1.0;
  for (int i = 1; i < nt; ++i)
    for (int j = n1; j < nt; ++j) a[i * nt + j] = a[(i - 1) * nt + j] * h[j] / double(i);
}

// Distributes the solved unknowns r into the implicit/explicit coefficient
// arrays (class_derivatives_coefficient.f90:197-207).
static void export_coeffs(const double* r, int cl, int n1, int n2, int exp_shift,
                          double* coef_imp, double* coef_exp, int nexp) {
  std::fill(coef_imp, coef_imp + 5, 0.0);
  std::fill(coef_exp, coef_exp + nexp, 0.0);
  const int k = (cl == 3) ? (4 - n1) / 2 : 0;
  const int l = (n1 + k >= cl) ? n1 + 1 : n1;
  int j = 0;
  for (int i = 1; i <= l; ++i)
    if (i != cl - k) coef_imp[i + k - 1] = r[j++];
  if (cl <= 5) coef_imp[cl - 1] = 1.0;
  for (int m = 0; m < n2; ++m) coef_exp[exp_shift + m] = r[n1 + m];
}

bool der_coeffs_generic(const double h0[7], int cl, int der, int so,
                        double coef_imp[5], double coef_exp[7]) {
  int n1, n2;
  switch (cl) {
    case 1: n1 = so == 8 ? 3 : so == 2 ? 0 : 1; n2 = so == 8 || so == 6 ? 6 : so == 4 ? 4 : 3; break;
    case 2: n1 = so == 6 ? 2 : so == 2 ? 0 : 1; n2 = so == 6 ? 6 : so == 2 ? 3 : 5; break;
    default: n1 = so == 8 ? 4 : so == 2 ? 0 : 2; n2 = so == 4 || so == 2 ? 3 : 5; break;
  }
  const int nt = n1 + n2;
  double h[10] = {0};
  if (cl == 1) {
    for (int m = 0; m < n1; ++m) h[m] = h0[1 + m];
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[m];
  } else if (cl == 2) {
    h[0] = h0[0];
    for (int m = 1; m < n1; ++m) h[m] = h0[m + 1];
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[m];
  } else {
    const int s = (4 - n1) / 2;
    h[0] = h0[s];
    h[1] = h0[1 + s];
    for (int m = 2 - s; m < n1; ++m) h[m] = h0[m + 1 + s];
    const int s2 = (5 - n2) / 2;
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[s2 + m];
  }
  double a[100], r[10] = {0};
  taylor_matrix(h, n1, nt, der, a);
  r[der] = 1.0;
  if (!small_solve(nt, a, r)) return false;
  export_coeffs(r, cl, n1, n2, cl == 3 ? (5 - n2) / 2 : 0, coef_imp, coef_exp, 7);
  return true;
}

bool solver_coeffs_generic(const double h0[7], int cl, int der, int bct, int so,
                           double coef_imp[5], double coef_exp[8]) {
  int n1 = 0, n2 = 3;
  double h[10] = {0};
  if (cl == 1) {
    n1 = so == 8 ? 3 : so == 2 ? 0 : 1;
    n2 = so == 8 || so == 6 ? 6 : so == 4 ? 4 : 3;
    for (int m = 0; m < n1; ++m) h[m] = h0[2 + m];
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[m];
  } else if (cl == 4) {
    n1 = 0;
    n2 = so == 8 || so == 6 ? 7 : so == 4 ? 5 : 3;
    for (int m = 0; m < n2; ++m) h[m] = h0[m];
  } else if (cl == 2) {
    if (so == 2) { n1 = 0; n2 = 3; }
    else if (bct == 3) { n1 = so == 8 ? 2 : 1; n2 = so == 8 ? 7 : 3; }
    else { n1 = 1; n2 = 5; }
    h[0] = h0[1];
    for (int m = 1; m < n1; ++m) h[m] = h0[m + 2];
    const int s = std::max(0, (5 - n2) / 2);  // C++ division truncates like Fortran
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[s + m];
  } else {
    n1 = so == 8 ? 4 : so == 2 ? 0 : 2;
    n2 = so == 4 || so == 2 ? 3 : 5;
    const int s = (4 - n1) / 2;
    h[0] = h0[s];
    h[1] = h0[1 + s];
    for (int m = 2 - s; m < n1; ++m) h[m] = h0[m + 1 + s];
    const int s2 = (5 - n2) / 2;
    for (int m = 0; m < n2; ++m) h[n1 + m] = h0[s2 + m];
  }
  const int nt = n1 + n2;
  double a[100], r[10] = {0};
  taylor_matrix(h, n1, nt, der, a);
  // boundary column: derivative-of-order-(bct-1) value at the boundary node
  // (class_solver_coefficient_3d.f90:195-203)
  if ((cl == 2 && n2 > 4) || cl == 1) {
    for (int i = 0; i < bct - 1; ++i) a[i * nt + n1] = 0.0;
    a[(bct - 1) * nt + n1] = (bct == 3) ? -1.0 : 1.0;
    for (int i = bct; i < nt; ++i)
      a[i * nt + n1] = a[(i - 1) * nt + n1] * h[n1] / double(i + 1 - bct);
  }
  r[der] = 1.0;
  if (!small_solve(nt, a, r)) return false;
  int s = 0;
  if (cl == 3) s = (5 - n2) / 2;
  if (cl == 2) s = std::max(0, (5 - n2) / 2);
  export_coeffs(r, cl, n1, n2, s, coef_imp, coef_exp, 8);
  return true;
}

// Fortran CSHIFT(a, shift) of a length-m array: out[i] = a[(i + shift) mod m].
static void cshift(const double* a, int m, int shift, double* out) {
  for (int i = 0; i < m; ++i) out[i] = a[((i + shift) % m + m) % m];
}

bool der_line_coeffs(const double* grid, int n, int der, int so, double* dl, double* dr) {
  if (n < 7) return false;
  std::fill(dl, dl + 5 * n, 0.0);
  std::fill(dr, dr + 7 * n, 0.0);
  double h[7], ci[5], ce[7], tmp[7];
  for (int m = 0; m < 7; ++m) h[m] = grid[0] - grid[m];
  if (!der_coeffs_generic(h, 1, der, so, ci, ce)) return false;
  cshift(ci, 5, -2, dl);
  for (int m = 0; m < 7; ++m) dr[m] = -ce[m];
  for (int m = 0; m < 7; ++m) h[m] = grid[1] - grid[m];
  if (!der_coeffs_generic(h, 2, der, so, ci, ce)) return false;
  cshift(ci, 5, -1, dl + 5);
  for (int m = 0; m < 7; ++m) dr[7 + m] = -ce[m];
  for (int i = 2; i < n - 2; ++i) {
    for (int m = 0; m < 7; ++m) h[m] = m < 5 ? grid[i] - grid[i - 2 + m] : 0.0;
    if (!der_coeffs_generic(h, 3, der, so, ci, ce)) return false;
    for (int m = 0; m < 5; ++m) dl[5 * i + m] = ci[m];
    for (int m = 0; m < 7; ++m) dr[7 * i + m] = -ce[m];
  }
  for (int m = 0; m < 7; ++m) h[m] = grid[n - 2] - grid[n - 1 - m];
  if (!der_coeffs_generic(h, 2, der, so, ci, ce)) return false;
  for (int m = 0; m < 5; ++m) tmp[m] = ci[4 - m];
  cshift(tmp, 5, 1, dl + 5 * (n - 2));
  for (int m = 0; m < 7; ++m) dr[7 * (n - 2) + m] = -ce[6 - m];
  for (int m = 0; m < 7; ++m) h[m] = grid[n - 1] - grid[n - 1 - m];
  if (!der_coeffs_generic(h, 1, der, so, ci, ce)) return false;
  for (int m = 0; m < 5; ++m) tmp[m] = ci[4 - m];
  cshift(tmp, 5, 2, dl + 5 * (n - 1));
  for (int m = 0; m < 7; ++m) dr[7 * (n - 1) + m] = -ce[6 - m];
  if (der == 2)
    for (int m = 0; m < 7 * n; ++m) dr[m] = -dr[m];
  return true;
}

void pentalu(int n, double* dl) {
  auto P = [&](int i) -> double& { return dl[5 * i + 0]; };
  auto F = [&](int i) -> double& { return dl[5 * i + 1]; };
  auto C = [&](int i) -> double& { return dl[5 * i + 2]; };
  auto D = [&](int i) -> double& { return dl[5 * i + 3]; };
  auto E = [&](int i) -> double& { return dl[5 * i + 4]; };
  const double alpha = P(0);
  F(1) = F(1) / C(0);
  C(1) = C(1) - D(0) * F(1);
  D(1) = D(1) - E(0) * F(1);
  E(1) = E(1) - alpha * F(1);
  int i = 2;
  P(i) = P(i) / C(i - 2);
  F(i) = (F(i) - P(i) * D(i - 2)) / C(i - 1);
  C(i) = C(i) - D(i - 1) * F(i) - E(i - 2) * P(i);
  D(i) = D(i) - E(i - 1) * F(i) - alpha * P(i);
  for (i = 3; i < n - 1; ++i) {
    P(i) = P(i) / C(i - 2);
    F(i) = (F(i) - P(i) * D(i - 2)) / C(i - 1);
    C(i) = C(i) - E(i - 2) * P(i) - D(i - 1) * F(i);
    D(i) = D(i) - E(i - 1) * F(i);
  }
  const double beta = E(n - 1) / C(n - 4);
  E(n - 1) = beta;  // the (n, n-3) multiplier is kept in e(n)
  P(n - 1) = P(n - 1) - beta * D(n - 4);
  F(n - 1) = F(n - 1) - beta * E(n - 4);
  P(n - 1) = P(n - 1) / C(n - 3);
  F(n - 1) = (F(n - 1) - P(n - 1) * D(n - 3)) / C(n - 2);
  C(n - 1) = C(n - 1) - E(n - 3) * P(n - 1) - D(n - 2) * F(n - 1);
}

bool solver_dder_coeffs(const double* g, int nall, const int bct[2], int so,
                        double* ddl, double* ddr) {
  const int n = nall - 2;
  if (n < 7) return false;
  std::fill(ddl, ddl + 5 * n, 0.0);
  std::fill(ddr, ddr + 8 * n, 0.0);
  double h[7], ci[5], ce[8], tmp[8];
  for (int m = 0; m < 7; ++m) h[m] = g[1] - g[m];
  if (!solver_coeffs_generic(h, 1, 2, bct[0], so, ci, ce)) return false;
  cshift(ci, 5, -2, ddl);
  for (int m = 0; m < 8; ++m) ddr[m] = -ce[m];
  if (bct[0] == 2) ddr[0] = -ddr[0];
  for (int m = 0; m < 7; ++m) h[m] = g[2] - g[m];
  if (!solver_coeffs_generic(h, 2, 2, bct[0], so, ci, ce)) return false;
  cshift(ci, 5, -1, ddl + 5);
  for (int m = 0; m < 8; ++m) ddr[8 + m] = -ce[m];
  if (bct[0] == 2) ddr[8] = -ddr[8];
  for (int i = 3; i <= n - 2; ++i) {  // grid index i, row i-1
    for (int m = 0; m < 7; ++m) h[m] = m < 5 ? g[i] - g[i - 2 + m] : 0.0;
    if (!solver_coeffs_generic(h, 3, 2, 0, so, ci, ce)) return false;
    for (int m = 0; m < 5; ++m) ddl[5 * (i - 1) + m] = ci[m];
    for (int m = 0; m < 8; ++m) ddr[8 * (i - 1) + m] = -ce[m];
  }
  for (int m = 0; m < 7; ++m) h[m] = g[n - 1] - g[n + 1 - m];
  if (!solver_coeffs_generic(h, 2, 2, bct[1], so, ci, ce)) return false;
  for (int m = 0; m < 5; ++m) tmp[m] = ci[4 - m];
  cshift(tmp, 5, 1, ddl + 5 * (n - 2));
  for (int m = 0; m < 8; ++m) ddr[8 * (n - 2) + m] = -ce[7 - m];
  if (bct[1] == 2) ddr[8 * (n - 2) + 7] = -ddr[8 * (n - 2) + 7];
  for (int m = 0; m < 7; ++m) h[m] = g[n] - g[n + 1 - m];
  if (!solver_coeffs_generic(h, 1, 2, bct[1], so, ci, ce)) return false;
  for (int m = 0; m < 5; ++m) tmp[m] = ci[4 - m];
  cshift(tmp, 5, 2, ddl + 5 * (n - 1));
  double rev[8];
  for (int m = 0; m < 8; ++m) rev[m] = ce[7 - m];
  cshift(rev, 8, 1, tmp);
  for (int m = 0; m < 8; ++m) ddr[8 * (n - 1) + m] = -tmp[m];
  if (bct[1] == 2) ddr[8 * (n - 1) + 6] = -ddr[8 * (n - 1) + 6];
  for (int m = 0; m < 8 * n; ++m) ddr[m] = -ddr[m];
  return true;
}

bool solver_extrapolation_coeffs(const double* g, int nall, const int bct[2], int so,
                                 double* neum) {
  const int n = nall - 2;
  double h[7], ci[5], ce[8];
  for (int m = 0; m < 7; ++m) h[m] = g[0] - g[m];
  if (!solver_coeffs_generic(h, 4, 1, bct[0], so, ci, ce)) return false;
  for (int m = 0; m < 7; ++m) neum[m] = -ce[m];
  for (int m = 0; m < 7; ++m) h[m] = g[n + 1] - g[n + 1 - m];
  if (!solver_coeffs_generic(h, 4, 1, bct[1], so, ci, ce)) return false;
  for (int m = 0; m < 7; ++m) neum[7 + m] = -ce[6 - m];
  return true;
}

void solver_lhs_rhs(int n, const double* ddl, const double* ddr, double* lhs, double* rhs) {
  std::fill(lhs, lhs + (size_t)n * n, 0.0);
  std::fill(rhs, rhs + (size_t)n * n, 0.0);
  auto L = [&](int i, int j) -> double& { return lhs[(size_t)i * n + j]; };
  auto R = [&](int i, int j) -> double& { return rhs[(size_t)i * n + j]; };
  const double* dl = ddl;
  const double* dr = ddr;
  L(0, 0) = dl[2]; L(0, 1) = dl[3]; L(0, 2) = dl[4]; L(0, 3) = dl[0];
  for (int m = 0; m < 4; ++m) L(1, m) = dl[5 + 1 + m];
  for (int i = 2; i < n - 2; ++i)
    for (int m = 0; m < 5; ++m) L(i, i - 2 + m) = dl[5 * i + m];
  for (int m = 0; m < 4; ++m) L(n - 2, n - 4 + m) = dl[5 * (n - 2) + m];
  L(n - 1, n - 4) = dl[5 * (n - 1) + 4];
  for (int m = 0; m < 3; ++m) L(n - 1, n - 3 + m) = dl[5 * (n - 1) + m];
  for (int m = 0; m < 6; ++m) R(0, m) = dr[1 + m];
  for (int m = 0; m < 7; ++m) R(1, m) = dr[8 + 1 + m];
  for (int i = 2; i < n - 2; ++i)
    for (int m = 0; m < 5; ++m) R(i, i - 2 + m) = dr[8 * i + m];
  for (int m = 0; m < 7; ++m) R(n - 2, n - 7 + m) = dr[8 * (n - 2) + m];
  for (int m = 0; m < 6; ++m) R(n - 1, n - 6 + m) = dr[8 * (n - 1) + m];
}

bool invert(int n, double* a) {
  std::vector<double> lu(a, a + (size_t)n * n);
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(lu[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      double v = std::fabs(lu[(size_t)i * n + k]);
      if (v > best) { best = v; p = i; }
    }
    if (best == 0.0) return false;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(lu[(size_t)k * n + j], lu[(size_t)p * n + j]);
    const double inv = 1.0 / lu[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double& l = lu[(size_t)i * n + k];
      l *= inv;
      if (l == 0.0) continue;
      const double* rk = &lu[(size_t)k * n];
      double* ri = &lu[(size_t)i * n];
      for (int j = k + 1; j < n; ++j) ri[j] -= l * rk[j];
    }
  }
  // solve LU X = P I column by column (X stored row-major in a)
  std::vector<double> col(n);
  for (int c = 0; c < n; ++c) {
    std::fill(col.begin(), col.end(), 0.0);
    col[c] = 1.0;
    // apply the row interchanges in order
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(col[k], col[piv[k]]);
    for (int i = 0; i < n; ++i) {
      double s = col[i];
      const double* ri = &lu[(size_t)i * n];
      for (int j = 0; j < i; ++j) s -= ri[j] * col[j];
      col[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = col[i];
      const double* ri = &lu[(size_t)i * n];
      for (int j = i + 1; j < n; ++j) s -= ri[j] * col[j];
      col[i] = s / ri[i];
    }
    for (int i = 0; i < n; ++i) a[(size_t)i * n + c] = col[i];
  }
  return true;
}

// ---------------------------------------------------------------------------
// Real nonsymmetric eigen-solver.  Textbook pipeline (Golub & Van Loan,
// "Matrix Computations", ch. 7): Parlett-Reinsch balancing, Householder
// reduction to Hessenberg form, Francis double-shift QR to real Schur form
// with accumulated transformations, then back substitution on the
// triangular factor for the eigenvectors.  Matrices are row-major.
// ---------------------------------------------------------------------------
namespace {

struct Mat {
  int n;
  std::vector<double> a;
  explicit Mat(int n_) : n(n_), a((size_t)n_ * n_, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i * n + j]; }
  double operator()(int i, int j) const { return a[(size_t)i * n + j]; }
};

// v (length m) and beta with (I - beta v v^T) x = -+|x| e1; v[0] = 1.
static double householder(const double* x, int m, double* v) {
  double sigma = 0.0;
  for (int i = 1; i < m; ++i) sigma += x[i] * x[i];
  v[0] = 1.0;
  for (int i = 1; i < m; ++i) v[i] = x[i];
  if (sigma == 0.0) return 0.0;
  const double mu = std::sqrt(x[0] * x[0] + sigma);
  const double v0 = (x[0] <= 0.0) ? x[0] - mu : -sigma / (x[0] + mu);
  const double beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
  for (int i = 1; i < m; ++i) v[i] /= v0;
  return beta;
}

// rows r0..r0+m-1, columns c0..c1 of H  <-  (I - beta v v^T) H
static void apply_left(Mat& H, int r0, int m, int c0, int c1, const double* v, double beta) {
  if (beta == 0.0) return;
  for (int j = c0; j <= c1; ++j) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += v[i] * H(r0 + i, j);
    s *= beta;
    for (int i = 0; i < m; ++i) H(r0 + i, j) -= s * v[i];
  }
}

// rows r0..r1, columns c0..c0+m-1 of H  <-  H (I - beta v v^T)
static void apply_right(Mat& H, int r0, int r1, int c0, int m, const double* v, double beta) {
  if (beta == 0.0) return;
  for (int i = r0; i <= r1; ++i) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += H(i, c0 + j) * v[j];
    s *= beta;
    for (int j = 0; j < m; ++j) H(i, c0 + j) -= s * v[j];
  }
}

static void balance(Mat& A, std::vector<double>& d) {
  const int n = A.n;
  d.assign(n, 1.0);
  const double radix = 2.0, sqrdx = 4.0;
  bool done = false;
  int sweeps = 0;
  while (!done && sweeps++ < 100) {
    done = true;
    for (int i = 0; i < n; ++i) {
      double r = 0.0, c = 0.0;
      for (int j = 0; j < n; ++j)
        if (j != i) { c += std::fabs(A(j, i)); r += std::fabs(A(i, j)); }
      if (c == 0.0 || r == 0.0) continue;
      double g = r / radix, f = 1.0;
      const double s = c + r;
      while (c < g) { f *= radix; c *= sqrdx; }
      g = r * radix;
      while (c > g) { f /= radix; c /= sqrdx; }
      if ((c + r) / f < 0.95 * s) {
        done = false;
        const double gi = 1.0 / f;
        d[i] *= f;
        for (int j = 0; j < n; ++j) A(i, j) *= gi;
        for (int j = 0; j < n; ++j) A(j, i) *= f;
      }
    }
  }
}

}  // namespace

int eig_real(int n, const double* a_in, double* w, double* v_out, double* max_imag) {
  Mat H(n), Z(n);
  std::copy(a_in, a_in + (size_t)n * n, H.a.begin());
  std::vector<double> d;
  balance(H, d);
  for (int i = 0; i < n; ++i) Z(i, i) = 1.0;
  std::vector<double> x(n), v(n);
  // Hessenberg reduction: H = Q^T A Q, Z = Q
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;
    for (int i = 0; i < m; ++i) x[i] = H(k + 1 + i, k);
    const double beta = householder(x.data(), m, v.data());
    apply_left(H, k + 1, m, k, n - 1, v.data(), beta);
    apply_right(H, 0, n - 1, k + 1, m, v.data(), beta);
    apply_right(Z, 0, n - 1, k + 1, m, v.data(), beta);
    for (int i = k + 2; i < n; ++i) H(i, k) = 0.0;
  }
  double norm = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = std::max(0, i - 1); j < n; ++j) norm = std::max(norm, std::fabs(H(i, j)));
  const double eps = 2.220446049250313e-16;
  *max_imag = 0.0;
  int hi = n - 1, iter = 0, total_iter = 0;
  while (hi >= 0) {
    if (total_iter > 60 * n) return 2;
    // find the start l of the unreduced block ending at hi
    int l = hi;
    for (; l > 0; --l) {
      double s = std::fabs(H(l - 1, l - 1)) + std::fabs(H(l, l));
      if (s == 0.0) s = norm;
      if (std::fabs(H(l, l - 1)) <= eps * s) { H(l, l - 1) = 0.0; break; }
    }
    if (l == hi) {  // 1x1 block converged
      w[hi] = H(hi, hi);
      --hi;
      iter = 0;
      continue;
    }
    if (l == hi - 1) {  // 2x2 block: split into two real eigenvalues or fail
      const double p = H(hi - 1, hi - 1), q = H(hi - 1, hi), r = H(hi, hi - 1), s = H(hi, hi);
      const double tr = 0.5 * (p + s);
      const double disc = 0.25 * (p - s) * (p - s) + q * r;
      if (disc < 0.0) {
        *max_imag = std::max(*max_imag, std::sqrt(-disc));
        return 1;
      }
      const double sq = std::sqrt(disc);
      // eigenvalue farther from s first, then the rotation that triangularises
      const double lam = (tr >= 0.0) ? tr + sq : tr - sq;
      double e0 = q, e1 = lam - p;  // eigenvector from the first row
      double f0 = lam - s, f1 = r;  // eigenvector from the second row
      if (e0 * e0 + e1 * e1 < f0 * f0 + f1 * f1) { e0 = f0; e1 = f1; }
      const double nr = std::sqrt(e0 * e0 + e1 * e1);
      double cs = 1.0, sn = 0.0;
      if (nr > 0.0) { cs = e0 / nr; sn = e1 / nr; }
      // G = [[cs, -sn], [sn, cs]]; H <- G^T H G, Z <- Z G
      for (int j = hi - 1; j < n; ++j) {
        const double t0 = H(hi - 1, j), t1 = H(hi, j);
        H(hi - 1, j) = cs * t0 + sn * t1;
        H(hi, j) = -sn * t0 + cs * t1;
      }
      for (int i = 0; i <= hi; ++i) {
        const double t0 = H(i, hi - 1), t1 = H(i, hi);
        H(i, hi - 1) = cs * t0 + sn * t1;
        H(i, hi) = -sn * t0 + cs * t1;
      }
      for (int i = 0; i < n; ++i) {
        const double t0 = Z(i, hi - 1), t1 = Z(i, hi);
        Z(i, hi - 1) = cs * t0 + sn * t1;
        Z(i, hi) = -sn * t0 + cs * t1;
      }
      H(hi, hi - 1) = 0.0;
      w[hi - 1] = H(hi - 1, hi - 1);
      w[hi] = H(hi, hi);
      hi -= 2;
      iter = 0;
      continue;
    }
    // Francis double-shift step on the block l..hi
    ++iter;
    ++total_iter;
    double s, t;
    if (iter % 11 == 10) {  // exceptional shift
      const double e = std::fabs(H(hi, hi - 1)) + std::fabs(H(hi - 1, hi - 2));
      const double h11 = 0.75 * e + H(hi, hi);
      s = 2.0 * h11;
      t = h11 * h11 + 0.4375 * e * e;
    } else {
      s = H(hi - 1, hi - 1) + H(hi, hi);
      t = H(hi - 1, hi - 1) * H(hi, hi) - H(hi - 1, hi) * H(hi, hi - 1);
    }
    double xx = H(l, l) * H(l, l) + H(l, l + 1) * H(l + 1, l) - s * H(l, l) + t;
    double yy = H(l + 1, l) * (H(l, l) + H(l + 1, l + 1) - s);
    double zz = H(l + 1, l) * H(l + 2, l + 1);
    for (int k = l; k <= hi - 2; ++k) {
      double xv[3] = {xx, yy, zz}, vv[3];
      const double beta = householder(xv, 3, vv);
      const int q = std::max(l, k - 1);
      apply_left(H, k, 3, q, n - 1, vv, beta);
      const int r = std::min(k + 3, hi);
      apply_right(H, 0, r, k, 3, vv, beta);
      apply_right(Z, 0, n - 1, k, 3, vv, beta);
      if (k > l) { H(k + 1, k - 1) = 0.0; H(k + 2, k - 1) = 0.0; }
      xx = H(k + 1, k);
      yy = H(k + 2, k);
      if (k < hi - 2) zz = H(k + 3, k);
    }
    double xv[2] = {xx, yy}, vv[2];
    const double beta = householder(xv, 2, vv);
    apply_left(H, hi - 1, 2, hi - 2, n - 1, vv, beta);
    apply_right(H, 0, hi, hi - 1, 2, vv, beta);
    apply_right(Z, 0, n - 1, hi - 1, 2, vv, beta);
    H(hi, hi - 2) = 0.0;
  }
  // eigenvectors of the upper-triangular H: (H - w_k I) y = 0, y_k = 1
  Mat Y(n);
  const double small = eps * std::max(norm, 1e-300);
  for (int k = n - 1; k >= 0; --k) {
    const double lam = H(k, k);
    Y(k, k) = 1.0;
    for (int i = k - 1; i >= 0; --i) {
      double s = 0.0;
      for (int j = i + 1; j <= k; ++j) s += H(i, j) * Y(j, k);
      double den = H(i, i) - lam;
      if (std::fabs(den) < small) den = (den >= 0.0) ? small : -small;
      Y(i, k) = -s / den;
      if (std::fabs(Y(i, k)) > 1e100) {  // rescale to avoid overflow
        for (int j = i; j <= k; ++j) Y(j, k) *= 1e-100;
      }
    }
  }
  // V = D Z Y, columns normalised to unit 2-norm
  for (int k = 0; k < n; ++k) {
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = 0; j <= k; ++j) s += Z(i, j) * Y(j, k);
      s *= d[i];
      x[i] = s;
      nrm += s * s;
    }
    nrm = std::sqrt(nrm);
    for (int i = 0; i < n; ++i) v_out[(size_t)i * n + k] = x[i] / nrm;
  }
  return 0;
}

namespace {

// Double-double numbers (unevaluated sums hi + lo) for the few products of
// the eigen refinement below whose sums cancel: Knuth's TwoSum and an
// fma-based TwoProduct, both exact in IEEE-754 arithmetic (the host code is
// built without floating-point contraction, so nothing else is fused).
struct DD { double hi, lo; };
inline DD dd_quick(double a, double b) { const double s = a + b; return {s, b - (s - a)}; }
inline DD dd_add(DD a, DD b) {
  const double s = a.hi + b.hi, bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b.hi - bb);
  const double t = a.lo + b.lo, tb = t - a.lo;
  const double f = (a.lo - (t - tb)) + (b.lo - tb);
  DD r = dd_quick(s, e + t);
  return dd_quick(r.hi, r.lo + f);
}
inline DD dd_prod(double a, double b) { const double p = a * b; return {p, std::fma(a, b, -p)}; }
inline DD dd_mul(DD a, DD b) {
  DD p = dd_prod(a.hi, b.hi);
  return dd_quick(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
inline DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
inline DD dd_div(DD a, DD b) {
  const double q1 = a.hi / b.hi;
  DD r = dd_add(a, dd_neg(dd_mul(b, {q1, 0.0})));
  const double q2 = r.hi / b.hi;
  r = dd_add(r, dd_neg(dd_mul(b, {q2, 0.0})));
  const double q3 = r.hi / b.hi;
  return dd_add(dd_quick(q1, q2), {q3, 0.0});
}

}  // namespace

// One first-order refinement of T = V diag(w) V^-1 for T = lhs^-1 rhs.
//
// The QR eigen-solver (like LAPACK's dgeev, which the reference calls at
// class_solver_3d.f90:535) returns eigenvalues with an absolute error of
// order eps*|T|; the small ones, which a Poisson solution weights most, then
// carry a relative error of eps*lambda_max/lambda_min (~1e-11 on a stretched
// 257-node axis), and near a null eigenvalue the eigenvectors are off by
// as much.  Here A = V^-1 T V is formed with T V = lhs^-1 (rhs V) and the
// product by V^-1 in double-double (lhs by a band LU without pivoting in
// double-double; its bandwidths are read off the matrix), so its diagonal
// gives eigenvalues with a relative error of order eps*cond(V) and its off-
// diagonal the first-order correction of the basis:
//   w'_i = A_ii,  V' = V (I + G),  G_ij = A_ij / (w'_j - w'_i)  (i != j),
// then V'^-1 by the FP64 inverse.  The refinement is skipped (the tables
// stay as they are) when some |G_ij| > 1e-6, i.e. when the first-order step
// would not be small.  Row-major n x n arrays; returns whether it applied.
static bool refine_eigen(int n, const double* lhs, const double* rhs, std::vector<double>& v,
                         std::vector<double>& vinv, std::vector<double>& w) {
  int kl = 0, ku = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (lhs[(size_t)i * n + j] != 0.0) { kl = std::max(kl, i - j); ku = std::max(ku, j - i); }
  std::vector<DD> lu((size_t)n * n);
  for (size_t p = 0; p < (size_t)n * n; ++p) lu[p] = {lhs[p], 0.0};
  auto LU = [&](int i, int j) -> DD& { return lu[(size_t)i * n + j]; };
  for (int k = 0; k < n; ++k) {
    if (LU(k, k).hi == 0.0) return false;
    for (int i = k + 1; i <= std::min(n - 1, k + kl); ++i) {
      const DD m = dd_div(LU(i, k), LU(k, k));
      LU(i, k) = m;
      for (int j = k + 1; j <= std::min(n - 1, k + ku); ++j)
        LU(i, j) = dd_add(LU(i, j), dd_neg(dd_mul(m, LU(k, j))));
    }
  }
  // TV, column j = lhs^-1 (rhs v_j), stored column by column
  std::vector<DD> tv((size_t)n * n), b(n);
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) {
      DD s = {0.0, 0.0};
      const double* ri = &rhs[(size_t)i * n];
      for (int k = 0; k < n; ++k)
        if (ri[k] != 0.0) s = dd_add(s, dd_prod(ri[k], v[(size_t)k * n + j]));
      b[i] = s;
    }
    for (int i = 1; i < n; ++i)
      for (int k = std::max(0, i - kl); k < i; ++k) b[i] = dd_add(b[i], dd_neg(dd_mul(LU(i, k), b[k])));
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k <= std::min(n - 1, i + ku); ++k)
        b[i] = dd_add(b[i], dd_neg(dd_mul(LU(i, k), b[k])));
      b[i] = dd_div(b[i], LU(i, i));
    }
    std::copy(b.begin(), b.end(), tv.begin() + (size_t)j * n);
  }
  // A = V^-1 TV in double-double, then w' and G
  std::vector<double> a((size_t)n * n), wn(n);
  for (int i = 0; i < n; ++i) {
    const double* wi = &vinv[(size_t)i * n];
    for (int j = 0; j < n; ++j) {
      const DD* tj = &tv[(size_t)j * n];
      DD s = {0.0, 0.0};
      for (int k = 0; k < n; ++k) {
        DD p = dd_prod(wi[k], tj[k].hi);
        p.lo += wi[k] * tj[k].lo;
        s = dd_add(s, p);
      }
      a[(size_t)i * n + j] = s.hi + s.lo;
    }
    wn[i] = a[(size_t)i * n + i];
  }
  std::vector<double> g((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (i == j) continue;
      const double aij = a[(size_t)i * n + j];
      const double gap = wn[j] - wn[i];
      if (std::fabs(aij) <= 1e-3 * std::fabs(gap)) {
        g[(size_t)i * n + j] = aij / gap;
        continue;
      }
      // near-degenerate pair (stretched grids have them among the high
      // modes, localised at either wall): no first-order rotation exists;
      // the coupling is left in place when it is negligible next to the
      // eigenvalues, otherwise the tables stay unrefined
      if (!(std::fabs(aij) <= 1e-13 * std::max(std::fabs(wn[i]), std::fabs(wn[j])))) return false;
    }
  std::vector<double> vn(v);
  for (int r = 0; r < n; ++r) {
    const double* vr = &v[(size_t)r * n];
    double* out = &vn[(size_t)r * n];
    for (int i = 0; i < n; ++i) {
      const double vri = vr[i];
      if (vri == 0.0) continue;
      const double* gi = &g[(size_t)i * n];
      for (int j = 0; j < n; ++j) out[j] += vri * gi[j];
    }
  }
  std::vector<double> vi(vn);
  if (!invert(n, vi.data())) return false;
  v.swap(vn);
  vinv.swap(vi);
  w.swap(wn);
  return true;
}

int solver_axis_setup(const double* grid, int nall, const int bct[2], int so,
                      SolverAxisHost& o, std::string& msg) {
  if (nall < 9) { msg = "solver axis needs at least 9 nodes"; return MF_ERR_ARG; }
  if (so != 2 && so != 4 && so != 6 && so != 8) { msg = "so must be 2, 4, 6 or 8"; return MF_ERR_ARG; }
  for (int s = 0; s < 2; ++s)
    if (bct[s] < 1 || bct[s] > 3) { msg = "bct must be 1, 2 or 3"; return MF_ERR_ARG; }
  const int n = nall - 2;
  o.nall = nall; o.n = n; o.so = so; o.bc[0] = bct[0]; o.bc[1] = bct[1];
  o.ddl.assign(5 * n, 0.0);
  o.ddr.assign(8 * n, 0.0);
  if (!solver_dder_coeffs(grid, nall, bct, so, o.ddl.data(), o.ddr.data())) {
    msg = "singular Taylor system in solver coefficients (grid nodes coincide?)";
    return MF_ERR_SINGULAR;
  }
  o.ddl_lu = o.ddl;
  pentalu(n, o.ddl_lu.data());
  std::vector<double> lhs((size_t)n * n), rhs((size_t)n * n);
  solver_lhs_rhs(n, o.ddl.data(), o.ddr.data(), lhs.data(), rhs.data());
  o.inv_lhs = lhs;
  if (!invert(n, o.inv_lhs.data())) { msg = "singular lhs in solver set-up"; return MF_ERR_SINGULAR; }
  std::vector<double> temp((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      const double a = o.inv_lhs[(size_t)i * n + k];
      if (a == 0.0) continue;
      const double* rr = &rhs[(size_t)k * n];
      double* tt = &temp[(size_t)i * n];
      for (int j = 0; j < n; ++j) tt[j] += a * rr[j];
    }
  o.eigen.assign(n, 0.0);
  o.vect.assign((size_t)n * n, 0.0);
  int rc = eig_real(n, temp.data(), o.eigen.data(), o.vect.data(), &o.max_imag);
  if (rc == 1 || o.max_imag > 1e-13) {
    msg = "complex eigenvalues in the 1D operator (the grid is too irregular)";
    return MF_ERR_COMPLEX_EIG;
  }
  if (rc != 0) { msg = "eigenvalue QR iteration did not converge"; return MF_ERR_NOT_CONVERGED; }
  o.inv_vect = o.vect;
  if (!invert(n, o.inv_vect.data())) { msg = "singular eigenvector matrix"; return MF_ERR_SINGULAR; }
  o.eigen_refined = refine_eigen(n, lhs.data(), rhs.data(), o.vect, o.inv_vect, o.eigen);
  o.neum.assign(14, 0.0);
  if (!solver_extrapolation_coeffs(grid, nall, bct, so, o.neum.data())) {
    msg = "singular extrapolation system";
    return MF_ERR_SINGULAR;
  }
  return MF_OK;
}

}  // namespace mf
