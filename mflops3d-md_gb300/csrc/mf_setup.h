// Host-side (CPU, FP64) set-up of the compact-scheme coefficients and of the
// per-axis eigen-decomposition used by the matrix-diagonalisation solver.
// Everything here runs once per operator; the results are uploaded to HBM.
#pragma once
#include <vector>
#include <string>

namespace mf {

// Solves a (n x n, row-major, n <= 10) x = b in place with partial pivoting.
// Replaces the LAPACK dgesv of class_derivatives_coefficient.f90:180 and
// class_solver_coefficient_3d.f90:212.  Returns false when a pivot is zero.
bool small_solve(int n, double* a, double* b);

// One row of the class_derivatives compact scheme
// (class_derivatives_coefficient.f90:53-212).
bool der_coeffs_generic(const double h0[7], int cl, int der, int so,
                        double coef_imp[5], double coef_exp[7]);

// One row of the class_solver compact second-derivative scheme with boundary
// type bct (class_solver_coefficient_3d.f90:30-245); cl = 4 is the 7-point
// extrapolation row.
bool solver_coeffs_generic(const double h0[7], int cl, int der, int bct, int so,
                           double coef_imp[5], double coef_exp[8]);

// dl[n][5] (p,f,c,d,e), dr[n][7] for a whole line (class_derivatives.f90:330-377).
bool der_line_coeffs(const double* grid, int n, int der, int so,
                     double* dl, double* dr);

// In-place quasi-pentadiagonal LU of dl[n][5] (class_derivatives.f90:379-423).
void pentalu(int n, double* dl);

// ddl[n][5], ddr[n][8] for the n = nall-2 interior rows (class_solver_3d.f90:568-619).
bool solver_dder_coeffs(const double* grid, int nall, const int bct[2], int so,
                        double* ddl, double* ddr);

// neum[2][7] Neumann extrapolation rows (class_solver_3d.f90:622-656).
bool solver_extrapolation_coeffs(const double* grid, int nall, const int bct[2], int so,
                                 double* neum);

// Dense lhs/rhs (row-major n x n) of the interior operator (class_solver_3d.f90:484-521).
void solver_lhs_rhs(int n, const double* ddl, const double* ddr, double* lhs, double* rhs);

// In-place inverse of a row-major n x n matrix by LU with partial pivoting.
bool invert(int n, double* a);

// Real eigen-decomposition of a general row-major n x n matrix:
// a = V diag(w) V^-1.  V is row-major with eigenvectors in its columns, each
// of unit 2-norm.  Returns 0 on success, 1 if a complex pair was found
// (max_imag receives the largest imaginary part), 2 if QR did not converge.
int eig_real(int n, const double* a, double* w, double* v, double* max_imag);

// Full per-axis set-up (solver_coeffs_init, class_solver_3d.f90:413-466).
struct SolverAxisHost {
  int nall = 0, n = 0, so = 6;
  int bc[2] = {1, 1};
  std::vector<double> ddl, ddr;        // [n][5], [n][8]
  std::vector<double> ddl_lu;          // pentalu(ddl)
  std::vector<double> inv_lhs;         // [n][n] row-major
  std::vector<double> eigen;           // [n]
  std::vector<double> vect, inv_vect;  // [n][n] row-major, V and V^-1
  std::vector<double> neum;            // [2][7]
  double max_imag = 0.0;
  bool eigen_refined = false;          // the double-double refinement applied
};
// Returns 0 on success or an MF_ERR_* code; msg receives a description.
int solver_axis_setup(const double* grid, int nall, const int bct[2], int so,
                      SolverAxisHost& out, std::string& msg);

}  // namespace mf
