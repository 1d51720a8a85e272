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
//
// The least-squares filter also has a banded form, used by mf_filter_apply:
// c solves the normal equations (A^T W^2 A) c = A^T W^2 y, whose matrix is
// banded (half-bandwidth k) and factored once by Cholesky on the host; per
// pencil the kernel streams A^T W^2 y into a forward substitution, then
// back-substitutes and evaluates, about (ni + 3 nc + no)(k + 1) FP64 FMA
// instead of no * ni for the dense operator (2.7k vs 37k per pencil for
// 384 -> 96).  The normal equations square the condition of the B-spline
// observation matrix, which is small (cond(A) < 15 for k <= 5 with several
// data points per knot interval, so rounding stays near 1e-14); when the
// Cholesky pivots show a poorly determined fit, the dense operator is used.
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

// Banded least-squares filter (device tables, all FP64):
//   lq[q]             first basis index of data point q (non-decreasing)
//   aw[q*(K+1)+m]     w_q^2 B_{lq+m}(x_q)
//   lo[j*(K+1)]       1 / L_jj, lo[j*(K+1)+m] = L_{j,j-m}    (Cholesky, lower)
//   up[j*(K+1)+m]     L_{j+m,j}                              (m = 1..K)
//   ep[p], ev[p*(K+1)+m]  first coefficient and the K+1 evaluation weights
//                         of output p (values or first derivatives)
struct FiltBand {
  const int* lq;
  const double* aw;
  const double* lo;
  const double* up;
  const int* ep;
  const double* ev;
  int ni, nc, no;
};

template <int K>
__global__ void __launch_bounds__(64) k_filter_banded(FiltBand fb, const double* __restrict__ in,
                                                      double* __restrict__ out, int n0, int n1, int n2,
                                                      int axis) {
  extern __shared__ double zs[];  // nc values per thread, thread-interleaved
  const int na = axis == 0 ? n1 : n0, nb = axis == 2 ? n1 : n2;
  const long long pid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = pid < (long long)na * nb;
  const int a = live ? (int)(pid % na) : 0, b = live ? (int)(pid / na) : 0;
  long long base, s, obase, os;
  if (axis == 0) {
    base = (long long)n0 * (a + (long long)n1 * b);
    s = 1;
    obase = (long long)fb.no * (a + (long long)n1 * b);
    os = 1;
  } else if (axis == 1) {
    base = a + (long long)n0 * n1 * b;
    s = n0;
    obase = a + (long long)n0 * fb.no * b;
    os = n0;
  } else {
    base = a + (long long)n0 * b;
    s = (long long)n0 * n1;
    obase = base;
    os = (long long)n0 * n1;
  }
  const int stride = blockDim.x;
  double* z = zs + threadIdx.x;
  // forward: r = A^T W^2 y streamed into L z = r
  double win[K + 1], zp[K];
#pragma unroll
  for (int m = 0; m <= K; ++m) win[m] = 0.0;
#pragma unroll
  for (int m = 0; m < K; ++m) zp[m] = 0.0;
  int jlo = 0;
  auto finalize = [&](int j) {
    double v = win[0];
#pragma unroll
    for (int m = 1; m <= K; ++m) v = fma(-fb.lo[j * (K + 1) + m], zp[m - 1], v);
    v *= fb.lo[j * (K + 1)];
    z[(long long)j * stride] = v;
#pragma unroll
    for (int m = K - 1; m > 0; --m) zp[m] = zp[m - 1];
    zp[0] = v;
#pragma unroll
    for (int m = 0; m < K; ++m) win[m] = win[m + 1];
    win[K] = 0.0;
  };
  for (int q = 0; q < fb.ni; ++q) {
    const int l = fb.lq[q];
    while (jlo < l) finalize(jlo++);
    const double y = live ? in[base + (long long)q * s] : 0.0;
#pragma unroll
    for (int m = 0; m <= K; ++m) win[m] = fma(fb.aw[q * (K + 1) + m], y, win[m]);
  }
  while (jlo < fb.nc) finalize(jlo++);
  // backward: L^T c = z, outputs emitted once their K+1 coefficients exist
  double cw[K + 1];
#pragma unroll
  for (int m = 0; m <= K; ++m) cw[m] = 0.0;
  int p = fb.no - 1;
  for (int j = fb.nc - 1; j >= 0; --j) {
    double v = z[(long long)j * stride];
#pragma unroll
    for (int m = 1; m <= K; ++m) v = fma(-fb.up[j * (K + 1) + m], cw[m - 1], v);
    v *= fb.lo[j * (K + 1)];
#pragma unroll
    for (int m = K; m > 0; --m) cw[m] = cw[m - 1];
    cw[0] = v;
    while (p >= 0 && fb.ep[p] == j) {
      double o = 0.0;
#pragma unroll
      for (int m = 0; m <= K; ++m) o = fma(fb.ev[p * (K + 1) + m], cw[m], o);
      if (live) out[obase + (long long)p * os] = o;
      --p;
    }
  }
}

}  // namespace mf

using namespace mf;

struct mf_filter {
  int ni = 0, no = 0;
  std::vector<double> P, Pd;  // host (no x ni), row-major
  DevBuf PT, PdT;             // device, transposed (ni x no)
  DevBuf st_in, st_out;
  // banded least-squares form (k > 0 when available)
  int band_k = 0, nc = 0;
  DevBuf lq, aw, lo, up, ep, ev, evd;
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

// Host tables of the banded least-squares form; false (dense operator only)
// when the output sites are not sorted, an evaluation row leaves its band,
// or a Cholesky pivot loses more than 10 digits of its diagonal.
struct BandTables {
  int k = 0, nc = 0;
  std::vector<int> lq, ep;
  std::vector<double> aw, lo, up, ev, evd;
};

static bool build_band(const double* xi, const double* wi, int ni, const double* xn, int nn, const double* xo,
                       int no, int k, BandTables& B) {
  std::vector<double> t;
  for (int i = 0; i <= k; ++i) t.push_back(xi[0]);
  for (int i = 1; i < nn - 1; ++i) t.push_back(xn[i]);
  for (int i = 0; i <= k; ++i) t.push_back(xi[ni - 1]);
  const int nc = (int)t.size() - k - 1, k1 = k + 1;
  for (int p = 1; p < no; ++p)
    if (!(xo[p] >= xo[p - 1])) return false;
  B.k = k;
  B.nc = nc;
  B.lq.assign(ni, 0);
  B.aw.assign((size_t)ni * k1, 0.0);
  std::vector<double> G((size_t)nc * k1, 0.0);  // G[j][j+m] at j*k1 + m
  double h[20];
  for (int q = 0; q < ni; ++q) {
    const int l = knot_interval(t, k, xi[q]);
    bspline_row(t, 0, k, xi[q], l, h);
    const double w = wi ? wi[q] : 1.0, w2 = w * w;
    B.lq[q] = l - k;
    for (int m = 0; m <= k; ++m) B.aw[(size_t)q * k1 + m] = w2 * h[m];
    for (int a = 0; a <= k; ++a)
      for (int b = a; b <= k; ++b) G[(size_t)(l - k + a) * k1 + (b - a)] += w2 * h[a] * h[b];
  }
  auto g = [&](int i, int j) {  // symmetric banded access, |i - j| <= k
    return i <= j ? G[(size_t)i * k1 + (j - i)] : G[(size_t)j * k1 + (i - j)];
  };
  // banded Cholesky G = L L^T; Lr[j*k1 + m] = L[j][j-m]
  std::vector<double> Lr((size_t)nc * k1, 0.0);
  for (int j = 0; j < nc; ++j) {
    for (int m = k; m >= 1; --m) {
      const int i = j - m;
      if (i < 0) continue;
      double s = g(j, i);
      for (int r = 1; r <= k; ++r) {
        const int c = i - r;  // column shared by rows j and i
        if (c < 0 || j - c > k) continue;
        s -= Lr[(size_t)j * k1 + (j - c)] * Lr[(size_t)i * k1 + (i - c)];
      }
      Lr[(size_t)j * k1 + m] = s / Lr[(size_t)i * k1];
    }
    double d = g(j, j);
    for (int m = 1; m <= k; ++m) d -= Lr[(size_t)j * k1 + m] * Lr[(size_t)j * k1 + m];
    if (!(d > 1e-10 * g(j, j))) return false;
    Lr[(size_t)j * k1] = std::sqrt(d);
  }
  B.lo.assign((size_t)nc * k1, 0.0);
  B.up.assign((size_t)nc * k1, 0.0);
  for (int j = 0; j < nc; ++j) {
    B.lo[(size_t)j * k1] = 1.0 / Lr[(size_t)j * k1];
    for (int m = 1; m <= k; ++m) {
      if (j - m >= 0) B.lo[(size_t)j * k1 + m] = Lr[(size_t)j * k1 + m];
      if (j + m < nc) B.up[(size_t)j * k1 + m] = Lr[(size_t)(j + m) * k1 + m];
    }
  }
  std::vector<double> E, Ed;
  eval_rows(t, k, xo, no, E, Ed);
  B.ep.assign(no, 0);
  B.ev.assign((size_t)no * k1, 0.0);
  B.evd.assign((size_t)no * k1, 0.0);
  for (int p = 0; p < no; ++p) {
    const int e0 = knot_interval(t, k, xo[p]) - k;
    B.ep[p] = e0;
    for (int i = 0; i < nc; ++i) {
      const double e = E[(size_t)p * nc + i], ed = Ed[(size_t)p * nc + i];
      if (i >= e0 && i <= e0 + k) {
        B.ev[(size_t)p * k1 + (i - e0)] = e;
        B.evd[(size_t)p * k1 + (i - e0)] = ed;
      } else if (e != 0.0 || ed != 0.0) {
        return false;
      }
    }
  }
  return true;
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
  BandTables B;
  if (!rc && build_band(xi, wi, ni, xn, nn, xo, no, k, B)) {
    auto up_i = [&](DevBuf& d, const std::vector<int>& v) {
      int r = d.ensure(v.size() * sizeof(int));
      if (!r && cudaMemcpy(d.ptr, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        r = set_error(MF_ERR_CUDA, "mf_filter_lsq_init: upload failed");
      return r;
    };
    auto up_d = [&](DevBuf& d, const std::vector<double>& v) {
      int r = d.ensure(v.size() * sizeof(double));
      if (!r && cudaMemcpy(d.ptr, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        r = set_error(MF_ERR_CUDA, "mf_filter_lsq_init: upload failed");
      return r;
    };
    if (!(rc = up_i(f->lq, B.lq)) && !(rc = up_i(f->ep, B.ep)) && !(rc = up_d(f->aw, B.aw)) &&
        !(rc = up_d(f->lo, B.lo)) && !(rc = up_d(f->up, B.up)) && !(rc = up_d(f->ev, B.ev)) &&
        !(rc = up_d(f->evd, B.evd))) {
      f->band_k = k;
      f->nc = B.nc;
    }
  }
  if (!rc && cudaDeviceSynchronize() != cudaSuccess)  // uploads complete before use on any stream
    rc = set_error(MF_ERR_CUDA, "filter set-up: upload failed");
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
  if (!rc && cudaDeviceSynchronize() != cudaSuccess)  // uploads complete before use on any stream
    rc = set_error(MF_ERR_CUDA, "filter set-up: upload failed");
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
  for (DevBuf* b : {&f->lq, &f->aw, &f->lo, &f->up, &f->ep, &f->ev, &f->evd}) b->release();
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
  HostCopyWait wait(st);
  wait.armed = !dev_in || !dev_out;
  if (!dev_in) {
    if ((rc = stage_in(f->st_in, in, in_bytes, st))) return rc;
    din = f->st_in.as<double>();
  }
  if (!dev_out) {
    if ((rc = f->st_out.ensure((size_t)tot * 8))) return rc;
    dout = f->st_out.as<double>();
  }
  // banded form: one thread per pencil, nc coefficients per thread in shared memory
  const int threads = f->nc <= 400 ? 64 : 32;
  const size_t smem = (size_t)threads * f->nc * sizeof(double);
  if (f->band_k > 0 && smem <= 208 * 1024) {
    FiltBand fb{f->lq.as<int>(), f->aw.as<double>(), f->lo.as<double>(), f->up.as<double>(), f->ep.as<int>(),
                deriv ? f->evd.as<double>() : f->ev.as<double>(), f->ni, f->nc, f->no};
    const long long pencils = (long long)nx * ny * nz / nin[axis];
    const unsigned grid = (unsigned)((pencils + threads - 1) / threads);
    switch (f->band_k) {
#define MF_BAND_CASE(K)                                                                                    \
  case K:                                                                                                  \
    MF_CUDA(cudaFuncSetAttribute(k_filter_banded<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    k_filter_banded<K><<<grid, threads, smem, st>>>(fb, din, dout, nx, ny, nz, axis);                    \
    break;
      MF_BAND_CASE(1)
      MF_BAND_CASE(2)
      MF_BAND_CASE(3)
      MF_BAND_CASE(4)
      MF_BAND_CASE(5)
#undef MF_BAND_CASE
      default:
        return set_error(MF_ERR_UNSUPPORTED, "mf_filter_apply: spline degree %d", f->band_k);
    }
  } else {
    const double* PT = deriv ? f->PdT.as<double>() : f->PT.as<double>();
    k_apply_axis<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(PT, f->ni, f->no, din, dout, nx, ny, nz, axis);
  }
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
