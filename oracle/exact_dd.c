/* Oracle helper (test infrastructure only): the residual of the solver's
 * interior operator in double-double arithmetic.
 *
 *   r = g - sigma*u - sum_axes lhs_a^-1 (rhs_a u + boundary column * bc)
 *
 * The 1D operators are the ones solver_matrix_init diagonalises
 * (src/class_solver/class_solver_3d.f90:468-521: lhs and rhs assembled from
 * ddl(n,5) and ddr(n,8) of dder_coeffs, :568-619), with the boundary data
 * added as solve_3d folds it (:104-175: ddr(1,1), ddr(2,1) times the left
 * value, ddr(n-1,8), ddr(n,7) times the right one).  lhs is solved by a
 * band LU without pivoting (lower and upper bandwidth 3: the quasi-penta
 * corners alpha at (1,4) and beta at (n,n-3)) carried out in double-double,
 * so the residual of an FP64 iterate is exact to ~1e-30 relative.  One
 * correction solve with it turns any FP64 solution into the exactly rounded
 * solution of the discrete problem: the yardstick that separates the
 * rounding of two FP64 implementations from their distance to each other.
 *
 * Double-double: unevaluated sums hi + lo, error-free transformations by
 * Knuth's TwoSum and an fma-based TwoProduct (Dekker/Knuth; the algorithms
 * of Hida, Li and Bailey's QD library, written here from their published
 * description).  Built with -ffp-contract=off so that no other expression
 * is fused: the results are the same on every IEEE-754 machine. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double hi, lo; } dd;

static inline dd two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  dd r = {s, (a - (s - bb)) + (b - bb)};
  return r;
}
static inline dd quick_two_sum(double a, double b) {
  double s = a + b;
  dd r = {s, b - (s - a)};
  return r;
}
static inline dd two_prod(double a, double b) {
  double p = a * b;
  dd r = {p, fma(a, b, -p)};
  return r;
}
static inline dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
static inline dd dd_neg(dd a) { dd r = {-a.hi, -a.lo}; return r; }
static inline dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
static inline dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
static inline dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
static inline dd dd_div(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul_d(b, q1));
  double q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul_d(b, q2));
  double q3 = r.hi / b.hi;
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, (dd){q3, 0.0});
}
static inline dd dd_from(double a) { dd r = {a, 0.0}; return r; }

/* Band storage of an n x n matrix with bandwidths 3/3: B[i*7 + (j-i+3)]. */
#define BW 3
#define BL (2 * BW + 1)

typedef struct {
  int n;
  dd* lu;        /* band LU factors of lhs, n*BL */
  double bcc[4]; /* ddr(1,1), ddr(2,1), ddr(n-1,8), ddr(n,7) */
} axis_op;

/* ddl(n,5), ddr(n,8) Fortran-ordered: ddl[i + n*c], ddr[i + n*c]. */
static int axis_op_init(axis_op* op, int n, const double* ddl, const double* ddr) {
  if (n < 8) return 1;
  op->n = n;
  op->lu = (dd*)calloc((size_t)n * BL, sizeof(dd));
  if (!op->lu) return 2;
#define L(i, j) op->lu[(size_t)(i) * BL + ((j) - (i) + BW)]
#define DL(i, c) ddl[(size_t)(i) + (size_t)n * (c)]
#define DR(i, c) ddr[(size_t)(i) + (size_t)n * (c)]
  /* lhs rows, class_solver_3d.f90:484-502 */
  for (int c = 0; c < 3; ++c) L(0, c) = dd_from(DL(0, 2 + c));
  L(0, 3) = dd_from(DL(0, 0));
  for (int c = 0; c < 4; ++c) L(1, c) = dd_from(DL(1, 1 + c));
  for (int i = 2; i < n - 2; ++i)
    for (int c = 0; c < 5; ++c) L(i, i - 2 + c) = dd_from(DL(i, c));
  for (int c = 0; c < 4; ++c) L(n - 2, n - 4 + c) = dd_from(DL(n - 2, c));
  L(n - 1, n - 4) = dd_from(DL(n - 1, 4));
  for (int c = 0; c < 3; ++c) L(n - 1, n - 3 + c) = dd_from(DL(n - 1, c));
  /* boundary column of the rhs rows (rows themselves: rhs_row, :503-521) */
  op->bcc[0] = DR(0, 0);
  op->bcc[1] = DR(1, 0);
  op->bcc[2] = DR(n - 2, 7);
  op->bcc[3] = DR(n - 1, 6);
  /* band LU without pivoting, in double-double */
  for (int k = 0; k < n; ++k) {
    const dd piv = L(k, k);
    if (piv.hi == 0.0) return 3;
    for (int i = k + 1; i <= k + BW && i < n; ++i) {
      dd m = dd_div(L(i, k), piv);
      L(i, k) = m;
      for (int j = k + 1; j <= k + BW && j < n; ++j) L(i, j) = dd_sub(L(i, j), dd_mul(m, L(k, j)));
    }
  }
#undef L
#undef DL
#undef DR
  return 0;
}

static void axis_op_free(axis_op* op) { free(op->lu); }

/* Row i of rhs times the line u (stride s), exact products summed in
 * double-double; rows 0, 1, n-2 and n-1 hold 6 or 7 one-sided entries,
 * the others the 5-point stencil (class_solver_3d.f90:503-521). */
static dd rhs_row(const axis_op* op, const double* ddr, int i, const double* u, long s) {
  const int n = op->n;
  dd acc = dd_from(0.0);
#define DR(i, c) ddr[(size_t)(i) + (size_t)n * (c)]
  if (i == 0) {
    for (int c = 0; c < 6; ++c) acc = dd_add(acc, two_prod(DR(0, 1 + c), u[c * s]));
  } else if (i == 1) {
    for (int c = 0; c < 7; ++c) acc = dd_add(acc, two_prod(DR(1, 1 + c), u[c * s]));
  } else if (i == n - 2) {
    for (int c = 0; c < 7; ++c) acc = dd_add(acc, two_prod(DR(n - 2, c), u[(n - 7 + c) * s]));
  } else if (i == n - 1) {
    for (int c = 0; c < 6; ++c) acc = dd_add(acc, two_prod(DR(n - 1, c), u[(n - 6 + c) * s]));
  } else {
    for (int c = 0; c < 5; ++c) acc = dd_add(acc, two_prod(DR(i, c), u[(i - 2 + c) * s]));
  }
#undef DR
  return acc;
}

/* y = lhs^-1 (rhs u + bc column), one line u of stride s; y has n entries. */
static void apply_line(const axis_op* op, const double* ddr, const double* u, long s, double bl,
                       double bh, dd* y) {
  const int n = op->n;
  for (int i = 0; i < n; ++i) y[i] = rhs_row(op, ddr, i, u, s);
  y[0] = dd_add(y[0], two_prod(op->bcc[0], bl));
  y[1] = dd_add(y[1], two_prod(op->bcc[1], bl));
  y[n - 2] = dd_add(y[n - 2], two_prod(op->bcc[2], bh));
  y[n - 1] = dd_add(y[n - 1], two_prod(op->bcc[3], bh));
#define L(i, j) op->lu[(size_t)(i) * BL + ((j) - (i) + BW)]
  for (int i = 1; i < n; ++i)
    for (int k = (i - BW > 0 ? i - BW : 0); k < i; ++k) y[i] = dd_sub(y[i], dd_mul(L(i, k), y[k]));
  for (int i = n - 1; i >= 0; --i) {
    for (int j = i + 1; j <= i + BW && j < n; ++j) y[i] = dd_sub(y[i], dd_mul(L(i, j), y[j]));
    y[i] = dd_div(y[i], L(i, i));
  }
#undef L
}

/* r_hi + r_lo = g - sigma*u - (Lx + Ly + Lz) u over the n1 x n2 x n3 interior
 * (x fastest).  ddl[a], ddr[a]: the axis's Fortran ddl(n_a,5), ddr(n_a,8);
 * bcx (n2,n3,2), bcy (n1,n3,2), bcz (n1,n2,2) Fortran-ordered, may be NULL
 * (zero data).  Returns 0, or nonzero on bad sizes / singular pivots. */
int mfo_residual_dd(int n1, int n2, int n3, const double* g, const double* u, double sigma,
                    const double* ddl0, const double* ddr0, const double* ddl1, const double* ddr1,
                    const double* ddl2, const double* ddr2, const double* bcx, const double* bcy,
                    const double* bcz, double* r_hi, double* r_lo) {
  const int ns[3] = {n1, n2, n3};
  const double* ddl[3] = {ddl0, ddl1, ddl2};
  const double* ddr[3] = {ddr0, ddr1, ddr2};
  const double* bcs[3] = {bcx, bcy, bcz};
  axis_op op[3];
  memset(op, 0, sizeof(op));
  int rc = 0;
  for (int a = 0; a < 3 && rc == 0; ++a) rc = axis_op_init(&op[a], ns[a], ddl[a], ddr[a]);
  if (rc != 0) {
    for (int a = 0; a < 3; ++a) axis_op_free(&op[a]);
    return rc;
  }
  const long total = (long)n1 * n2 * n3;
#pragma omp parallel for schedule(static)
  for (long p = 0; p < total; ++p) {
    dd t = dd_sub(dd_from(g[p]), two_prod(sigma, u[p]));
    r_hi[p] = t.hi;
    r_lo[p] = t.lo;
  }
  const long stride[3] = {1, (long)n1, (long)n1 * n2};
  for (int a = 0; a < 3; ++a) {
    const int n = ns[a];
    const int o1 = (a == 0) ? 1 : 0, o2 = (a == 2) ? 1 : 2; /* the two other axes */
    const int m1 = ns[o1], m2 = ns[o2];
    const long lines = (long)m1 * m2;
#pragma omp parallel
    {
      dd* y = (dd*)malloc((size_t)n * sizeof(dd));
#pragma omp for schedule(static)
      for (long q = 0; q < lines; ++q) {
        const int i1 = (int)(q % m1), i2 = (int)(q / m1);
        const long base = i1 * stride[o1] + i2 * stride[o2];
        /* bc(a_other1, a_other2, 2) of this axis, Fortran-ordered */
        double bl = 0.0, bh = 0.0;
        if (bcs[a]) {
          bl = bcs[a][i1 + (long)m1 * i2];
          bh = bcs[a][i1 + (long)m1 * i2 + lines];
        }
        apply_line(&op[a], ddr[a], u + base, stride[a], bl, bh, y);
        for (int i = 0; i < n; ++i) {
          const long p = base + i * stride[a];
          dd t = dd_sub((dd){r_hi[p], r_lo[p]}, y[i]);
          r_hi[p] = t.hi;
          r_lo[p] = t.lo;
        }
      }
      free(y);
    }
  }
  for (int a = 0; a < 3; ++a) axis_op_free(&op[a]);
  return 0;
}
