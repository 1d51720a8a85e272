// Least-squares B-spline filter (class_filter) on GB300.
//
// Reference: LSQUnivariateSpline (class_filter.f90:104-174: fixed-knot
// weighted least squares, FITPACK curfit iopt=-1, then splev / splder) and
// interp_period (class_filter.f90:267-347: periodic quintic least squares,
// FITPACK percur iopt=-1, then splev), applied pencil by pencil.
//
// For fixed data sites, weights and knots the fit is linear in the data, so
// every pencil of an axis shares one operator  yo = P y  (and yo' = P' y).
// Set-up (host, FP64): the weighted observation matrix is reduced to a band
// triangle by Givens rotations in FITPACK's row order, with the identity as
// right-hand side, giving R^-1 Q^T W for all unit data vectors at once; the
// evaluation rows (B-spline values / derivatives at the output sites) times
// that matrix give P.  The periodic fit folds the k wrapped coefficients and
// uses a Householder QR.  Apply (GPU, FP64): one kernel per axis, thread per
// output point, operator rows broadcast, data reads coalesced along x.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mf_internal.h"

namespace mf {

// Non-zero B-splines of degree k at x with t[l] <= x < t[l+1] (de Boor-Cox).
static void bspline_row(const std::vector<double>& t, int off, int k, double x, int l, double* h) {
  double hh[20];
  h[0] = 1.0;
  for (int j = 1; j <= k; ++j) {
    for (int i = 0; i < j; ++i) hh[i] = h[i];
    h[0] = 0.0;
    for (int i = 0; i < j; ++i) {
      const int li = off + l + i + 1, lj = li - j;
      const double f = hh[i] / (t[li] - t[lj]);
      h[i] = h[i] + f * (t[li] - x);
      h[i + 1] = f * (x - t[lj]);
    }
  }
}

static int knot_interval(const std::vector<double>& t, int k, double x) {
  const int n = (int)t.size();
  int l = k;
  while (x >= t[l + 1] && l != n - k - 2) ++l;
  return l;
}

// Rows of the evaluation operators at xo: value and first derivative of the
// spline in terms of its coefficients (splev / splder).
static void eval_rows(const std::vector<double>& t, int k, const double* xo, int no,
                      std::vector<double>& E, std::vector<double>& Ed) {
  const int nk1 = (int)t.size() - k - 1;
  E.assign((size_t)no * nk1, 0.0);
  Ed.assign((size_t)no * nk1, 0.0);
  double h[20];
  for (int p = 0; p < no; ++p) {
    const int l = knot_interval(t, k, xo[p]);
    bspline_row(t, 0, k, xo[p], l, h);
    for (int i = 0; i <= k; ++i) E[(size_t)p * nk1 + l - k + i] = h[i];
    // derivative: degree k-1 B-splines on t[1..n-2], coefficients
    // k (c_i - c_{i-1}) / (t_{i+k} - t_i)
    bspline_row(t, 1, k - 1, xo[p], l - 1, h);
    for (int i = 0; i < k; ++i) {
      const int ii = l - k + 1 + i;
      const double s = k / (t[ii + k] - t[ii]);
      Ed[(size_t)p * nk1 + ii] += h[i] * s;
      Ed[(size_t)p * nk1 + ii - 1] -= h[i] * s;
    }
  }
}

// Coefficient operator G (nk1 x ni): c = G y for the fixed-knot weighted
// least-squares fit (fpcurf, iopt = -1), Givens rotations in FITPACK's order.
static bool lsq_coeff_operator(const double* xi, const double* wi, int ni, const std::vector<double>& t,
                               int k, std::vector<double>& G) {
  const int n = (int)t.size(), nk1 = n - k - 1, k1 = k + 1;
  std::vector<double> a((size_t)nk1 * k1, 0.0), z((size_t)nk1 * ni, 0.0), yw(ni);
  double h[20];
  for (int it = 0; it < ni; ++it) {
    const double w = wi ? wi[it] : 1.0;
    std::fill(yw.begin(), yw.end(), 0.0);
    yw[it] = w;  // right-hand side of this data point for every unit vector
    const int l = knot_interval(t, k, xi[it]);
    bspline_row(t, 0, k, xi[it], l, h);
    for (int i = 0; i < k1; ++i) h[i] *= w;
    int j = l - k;
    for (int i = 0; i < k1; ++i, ++j) {
      const double piv = h[i];
      if (piv == 0.0) continue;
      double& ajj = a[(size_t)j * k1];
      const double store = std::fabs(piv);
      const double dd = store >= ajj ? store * std::sqrt(1.0 + (ajj / piv) * (ajj / piv))
                                     : ajj * std::sqrt(1.0 + (piv / ajj) * (piv / ajj));
      const double cs = ajj / dd, sn = piv / dd;
      ajj = dd;
      double* zj = &z[(size_t)j * ni];
      for (int q = 0; q < ni; ++q) {
        const double y0 = yw[q], z0 = zj[q];
        zj[q] = cs * z0 + sn * y0;
        yw[q] = cs * y0 - sn * z0;
      }
      for (int i1 = i + 1, i2 = 1; i1 < k1; ++i1, ++i2) {
        double& ab = a[(size_t)j * k1 + i2];
        const double h0 = h[i1], a0 = ab;
        ab = cs * a0 + sn * h0;
        h[i1] = cs * h0 - sn * a0;
      }
    }
  }
  G.assign((size_t)nk1 * ni, 0.0);
  for (int i = nk1 - 1; i >= 0; --i) {
    const double diag = a[(size_t)i * k1];
    if (diag == 0.0) return false;
    for (int q = 0; q < ni; ++q) {
      double s = z[(size_t)i * ni + q];
      for (int m = 1; m < k1 && i + m < nk1; ++m) s -= a[(size_t)i * k1 + m] * G[(size_t)(i + m) * ni + q];
      G[(size_t)i * ni + q] = s / diag;
    }
  }
  return true;
}

// Periodic fit (percur, iopt = -1): coefficient operator on the full
// (wrapped) coefficient vector.  The last data point only fixes the period.
static bool periodic_coeff_operator(const double* xi, int ni, const std::vector<double>& t, int k,
                                    std::vector<double>& G) {
  const int n = (int)t.size(), nk1 = n - k - 1, nfree = n - 2 * k - 1;
  const int mrows = ni - 1;
  if (nfree < 1 || mrows < nfree) return false;
  // A (mrows x nfree), row-major, with wrapped columns
  std::vector<double> A((size_t)mrows * nfree, 0.0);
  double h[20];
  for (int r = 0; r < mrows; ++r) {
    const int l = knot_interval(t, k, xi[r]);
    bspline_row(t, 0, k, xi[r], l, h);
    for (int i = 0; i <= k; ++i) A[(size_t)r * nfree + (l - k + i) % nfree] += h[i];
  }
  // Householder QR of A; Q^T applied to the identity (mrows x mrows)
  std::vector<double> QtI((size_t)mrows * mrows, 0.0);
  for (int r = 0; r < mrows; ++r) QtI[(size_t)r * mrows + r] = 1.0;
  std::vector<double> v(mrows);
  for (int c = 0; c < nfree; ++c) {
    double nrm = 0.0;
    for (int r = c; r < mrows; ++r) nrm += A[(size_t)r * nfree + c] * A[(size_t)r * nfree + c];
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) return false;
    const double a0 = A[(size_t)c * nfree + c];
    const double alpha = a0 > 0 ? -nrm : nrm;
    for (int r = c; r < mrows; ++r) v[r] = A[(size_t)r * nfree + c];
    v[c] -= alpha;
    double vv = 0.0;
    for (int r = c; r < mrows; ++r) vv += v[r] * v[r];
    if (vv == 0.0) continue;
    auto reflect = [&](double* col, int stride) {
      double s = 0.0;
      for (int r = c; r < mrows; ++r) s += v[r] * col[(size_t)r * stride];
      s = 2.0 * s / vv;
      for (int r = c; r < mrows; ++r) col[(size_t)r * stride] -= s * v[r];
    };
    for (int cc = c; cc < nfree; ++cc) reflect(&A[cc], nfree);
    for (int q = 0; q < mrows; ++q) reflect(&QtI[q], mrows);
  }
  // free coefficients F (nfree x ni): R F = (Q^T)[0:nfree, :], last column 0
  std::vector<double> F((size_t)nfree * ni, 0.0);
  for (int i = nfree - 1; i >= 0; --i) {
    const double diag = A[(size_t)i * nfree + i];
    if (diag == 0.0) return false;
    for (int q = 0; q < mrows; ++q) {
      double s = QtI[(size_t)i * mrows + q];
      for (int m = i + 1; m < nfree; ++m) s -= A[(size_t)i * nfree + m] * F[(size_t)m * ni + q];
      F[(size_t)i * ni + q] = s / diag;
    }
  }
  G.assign((size_t)nk1 * ni, 0.0);
  for (int i = 0; i < nk1; ++i)
    for (int q = 0; q < ni; ++q) G[(size_t)i * ni + q] = F[(size_t)(i % nfree) * ni + q];
  return true;
}

// out along `axis` (length no) = P (no x ni) applied to in (length ni).
__global__ void k_apply_axis(const double* __restrict__ PT, int ni, int no, const double* __restrict__ in,
                             double* __restrict__ out, int n0, int n1, int n2, int axis) {
  // output shape: axis length replaced by no; thread index over the output, x fastest
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int o0 = axis == 0 ? no : n0, o1 = axis == 1 ? no : n1, o2 = axis == 2 ? no : n2;
  if (t >= (long long)o0 * o1 * o2) return;
  const int a = (int)(t % o0);
  const long long bc = t / o0;
  const int b = (int)(bc % o1), c = (int)(bc / o1);
  const int o = axis == 0 ? a : axis == 1 ? b : c;
  long long base, s;
  if (axis == 0) { base = (long long)n0 * (b + (long long)n1 * c); s = 1; }
  else if (axis == 1) { base = a + (long long)n0 * n1 * c; s = n0; }
  else { base = a + (long long)n0 * b; s = (long long)n0 * n1; }
  double acc = 0.0;
  for (int i = 0; i < ni; ++i) acc = fma(PT[(size_t)i * no + o], in[base + i * s], acc);
  out[t] = acc;
}

}  // namespace mf

using namespace mf;

struct mf_filter {
  int ni = 0, no = 0;
  std::vector<double> P, Pd;  // host (no x ni), row-major
  DevBuf PT, PdT;             // device, transposed (ni x no)
  DevBuf st_in, st_out;
};

static int filter_upload(mf_filter* f) {
  const int ni = f->ni, no = f->no;
  std::vector<double> T((size_t)ni * no), Td((size_t)ni * no);
  for (int p = 0; p < no; ++p)
    for (int q = 0; q < ni; ++q) {
      T[(size_t)q * no + p] = f->P[(size_t)p * ni + q];
      Td[(size_t)q * no + p] = f->Pd[(size_t)p * ni + q];
    }
  int rc;
  if ((rc = f->PT.ensure(T.size() * 8)) || (rc = f->PdT.ensure(Td.size() * 8))) return rc;
  MF_CUDA(cudaMemcpy(f->PT.ptr, T.data(), T.size() * 8, cudaMemcpyHostToDevice));
  MF_CUDA(cudaMemcpy(f->PdT.ptr, Td.data(), Td.size() * 8, cudaMemcpyHostToDevice));
  return MF_OK;
}

namespace mf {

// P = E G and P' = E' G (host, row-major no x ni).
static void assemble(const std::vector<double>& t, int k, const std::vector<double>& G, int ni,
                     const double* xo, int no, std::vector<double>& P, std::vector<double>& Pd) {
  std::vector<double> E, Ed;
  eval_rows(t, k, xo, no, E, Ed);
  const int nk1 = (int)t.size() - k - 1;
  P.assign((size_t)no * ni, 0.0);
  Pd.assign((size_t)no * ni, 0.0);
  for (int p = 0; p < no; ++p)
    for (int i = 0; i < nk1; ++i) {
      const double e = E[(size_t)p * nk1 + i], ed = Ed[(size_t)p * nk1 + i];
      if (e == 0.0 && ed == 0.0) continue;
      for (int q = 0; q < ni; ++q) {
        P[(size_t)p * ni + q] += e * G[(size_t)i * ni + q];
        Pd[(size_t)p * ni + q] += ed * G[(size_t)i * ni + q];
      }
    }
}

static int build_lsq(const double* xi, int ni, const double* wi, const double* xn, int nn,
                     const double* xo, int no, int k, std::vector<double>& P, std::vector<double>& Pd) {
  if (!xi || !xn || !xo) return set_error(MF_ERR_ARG, "spline filter: null argument");
  if (k < 1 || k > 5 || nn < 2 || ni < nn + k - 1 || no < 1)
    return set_error(MF_ERR_ARG, "spline filter: need 1 <= k <= 5, nn >= 2, ni >= nn+k-1");
  for (int i = 1; i < ni; ++i)
    if (!(xi[i] > xi[i - 1])) return set_error(MF_ERR_ARG, "spline filter: xi must increase");
  // knots (class_filter.f90:147-153): (k+1) xb, xn(2:nn-1), (k+1) xe
  std::vector<double> t;
  for (int i = 0; i <= k; ++i) t.push_back(xi[0]);
  for (int i = 1; i < nn - 1; ++i) t.push_back(xn[i]);
  for (int i = 0; i <= k; ++i) t.push_back(xi[ni - 1]);
  std::vector<double> G;
  if (!lsq_coeff_operator(xi, wi, ni, t, k, G))
    return set_error(MF_ERR_SINGULAR, "spline filter: singular least-squares system (check knots)");
  assemble(t, k, G, ni, xo, no, P, Pd);
  return MF_OK;
}

static int build_period(const double* xi, int ni, const double* xos, int nos, std::vector<double>& P,
                        std::vector<double>& Pd) {
  if (!xi || !xos) return set_error(MF_ERR_ARG, "periodic spline filter: null argument");
  const int k = 5;
  const int nn = ni - k - 1;
  if (nn < 3 || nos < 1) return set_error(MF_ERR_ARG, "periodic spline filter: ni too small");
  for (int i = 1; i < ni; ++i)
    if (!(xi[i] > xi[i - 1])) return set_error(MF_ERR_ARG, "periodic spline filter: xi must increase");
  // nodes as the reference (class_filter.f90:304-307): not offset by xi(1)
  std::vector<double> xn(nn);
  for (int i = 0; i < nn; ++i) xn[i] = (xi[ni - 1] - xi[0]) * (double)i / (double)(nn - 1);
  const double xb = xi[0], xe = xi[ni - 1], per = xe - xb;
  const int n = nn + 2 * k;
  std::vector<double> t(n, 0.0);
  t[k] = xb;
  for (int i = 1; i < nn - 1; ++i) t[k + i] = xn[i];
  t[n - k - 1] = xe;
  for (int j = 1; j <= k; ++j) {
    t[k - j] = t[n - k - 1 - j] - per;
    t[n - k - 1 + j] = t[k + j] + per;
  }
  std::vector<double> G;
  if (!periodic_coeff_operator(xi, ni, t, k, G))
    return set_error(MF_ERR_SINGULAR, "periodic spline filter: singular least-squares system");
  assemble(t, k, G, ni, xos, nos, P, Pd);
  return MF_OK;
}

static void to_fortran(const std::vector<double>& S, int no, int ni, double* out) {
  for (int p = 0; p < no; ++p)
    for (int q = 0; q < ni; ++q) out[p + (size_t)no * q] = S[(size_t)p * ni + q];
}

}  // namespace mf

extern "C" {

int mf_filter_lsq_matrix(const double* xi, int ni, const double* wi, const double* xn, int nn,
                         const double* xo, int no, int k, double* P, double* Pd) {
  std::vector<double> A, Ad;
  int rc = build_lsq(xi, ni, wi, xn, nn, xo, no, k, A, Ad);
  if (rc) return rc;
  if (P) to_fortran(A, no, ni, P);
  if (Pd) to_fortran(Ad, no, ni, Pd);
  return MF_OK;
}

int mf_filter_period_matrix(const double* xi, int ni, const double* xos, int nos, double* P,
                            double* Pd) {
  std::vector<double> A, Ad;
  int rc = build_period(xi, ni, xos, nos, A, Ad);
  if (rc) return rc;
  if (P) to_fortran(A, nos, ni, P);
  if (Pd) to_fortran(Ad, nos, ni, Pd);
  return MF_OK;
}

int mf_filter_lsq_init(const double* xi, int ni, const double* wi, const double* xn, int nn,
                       const double* xo, int no, int k, mf_filter_t** out) {
  if (!out) return set_error(MF_ERR_ARG, "mf_filter_lsq_init: null handle pointer");
  *out = nullptr;
  mf_filter* f = new mf_filter();
  int rc = build_lsq(xi, ni, wi, xn, nn, xo, no, k, f->P, f->Pd);
  f->ni = ni;
  f->no = no;
  if (!rc) rc = filter_upload(f);
  if (rc) {
    mf_filter_destroy(f);
    return rc;
  }
  *out = f;
  return MF_OK;
}

int mf_filter_period_init(const double* xi, int ni, const double* xos, int nos, mf_filter_t** out) {
  if (!out) return set_error(MF_ERR_ARG, "mf_filter_period_init: null handle pointer");
  *out = nullptr;
  mf_filter* f = new mf_filter();
  int rc = build_period(xi, ni, xos, nos, f->P, f->Pd);
  f->ni = ni;
  f->no = nos;
  if (!rc) rc = filter_upload(f);
  if (rc) {
    mf_filter_destroy(f);
    return rc;
  }
  *out = f;
  return MF_OK;
}

int mf_filter_destroy(mf_filter_t* f) {
  if (!f) return MF_OK;
  f->PT.release();
  f->PdT.release();
  f->st_in.release();
  f->st_out.release();
  delete f;
  return MF_OK;
}

int mf_filter_matrix(const mf_filter_t* f, int deriv, double* P) {
  if (!f || !P) return set_error(MF_ERR_ARG, "mf_filter_matrix: null argument");
  const std::vector<double>& S = deriv ? f->Pd : f->P;
  for (int p = 0; p < f->no; ++p)
    for (int q = 0; q < f->ni; ++q) P[p + (size_t)f->no * q] = S[(size_t)p * f->ni + q];
  return MF_OK;
}

int mf_filter_apply(const mf_filter_t* fc, int axis, int deriv, const double* in, int nx, int ny, int nz,
                    double* out, void* stream) {
  mf_filter_t* f = const_cast<mf_filter_t*>(fc);
  if (!f || !in || !out || axis < 0 || axis > 2) return set_error(MF_ERR_ARG, "mf_filter_apply: bad arguments");
  const int nin[3] = {nx, ny, nz};
  if (nin[axis] != f->ni)
    return set_error(MF_ERR_ARG, "mf_filter_apply: axis length %d differs from the filter's %d", nin[axis], f->ni);
  int nout[3] = {nx, ny, nz};
  nout[axis] = f->no;
  const size_t in_bytes = (size_t)nx * ny * nz * 8;
  const long long tot = (long long)nout[0] * nout[1] * nout[2];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_in = is_device_ptr(in), dev_out = is_device_ptr(out);
  const double* din = in;
  double* dout = out;
  int rc;
  if (!dev_in) {
    if ((rc = stage_in(f->st_in, in, in_bytes, st))) return rc;
    din = f->st_in.as<double>();
  }
  if (!dev_out) {
    if ((rc = f->st_out.ensure((size_t)tot * 8))) return rc;
    dout = f->st_out.as<double>();
  }
  const double* PT = deriv ? f->PdT.as<double>() : f->PT.as<double>();
  k_apply_axis<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(PT, f->ni, f->no, din, dout, nx, ny, nz, axis);
  MF_CUDA(cudaGetLastError());
  if (!dev_out) MF_CUDA(cudaMemcpyAsync(out, dout, (size_t)tot * 8, cudaMemcpyDeviceToHost, st));
  if (!dev_in || !dev_out) MF_CUDA(cudaStreamSynchronize(st));
  return MF_OK;
}

int mf_lsq_univariate_spline(int ni, const double* xi, const double* yi, const double* wi, int nn,
                             const double* xn, int no, const double* xo, double* yo, double* ypo, int k) {
  mf_filter_t* f = nullptr;
  int rc = mf_filter_lsq_init(xi, ni, wi, xn, nn, xo, no, k, &f);
  if (rc) return rc;
  if (yo && (rc = mf_filter_apply(f, 0, 0, yi, ni, 1, 1, yo, nullptr))) { mf_filter_destroy(f); return rc; }
  if (ypo && (rc = mf_filter_apply(f, 0, 1, yi, ni, 1, 1, ypo, nullptr))) { mf_filter_destroy(f); return rc; }
  return mf_filter_destroy(f);
}

int mf_interp_period(int ni, const double* xi, const double* yi, int nos, const double* xos, double* yos) {
  mf_filter_t* f = nullptr;
  int rc = mf_filter_period_init(xi, ni, xos, nos, &f);
  if (rc) return rc;
  if ((rc = mf_filter_apply(f, 0, 0, yi, ni, 1, 1, yos, nullptr))) { mf_filter_destroy(f); return rc; }
  return mf_filter_destroy(f);
}

}  // extern "C"
