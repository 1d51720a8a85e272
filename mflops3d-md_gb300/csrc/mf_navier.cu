// Navier-Stokes time step on one domain: the caller of the derivative and
// solver entry points, src/main/navier3d.f90:48-274 built from
// src/class_navier/class_navier_3D.f90 (one domain, mapt = 0, pressure types
// 1 to 4, les_type 0..3, sub-iterations).
//
// Time levels: nt = 4 slots per variable (u, v, w, p, phi) addressed through
// the permutation it(1..nt) of the reference (it(1) = the slot a step
// writes, it(nt) = the newest); the host keeps `it` and rotates it after each
// step (navier3d.f90:256-261).  The nonlinear term of a slot depends only on
// that slot's u, v, w, which do not change once the slot is final, so it is
// cached per slot: each step computes it for the newest slot only, where the
// reference recomputes all nt slots and reads two or three of them
// (class_navier_3D.f90:1169-1222); the values read are the same.
//
// The exact solution `sol` of the reference (class_navier_3D.f90:927-1041) is
// steady (wt = 0: cos(wt t) = 1, sin(wt t) = 0 at every t), so its boundary
// values and sources are evaluated once, at set-up, on the device.
//
// Stages per step (device work only, on the caller's stream):
//   flow-rate term   weighted sum of extrapol(u) (k_ns_wsum) -> k_ns_flow
//   presolve         k_ns_advect / k_ns_products / k_ns_skew (newest slot,
//                    eighteen sweeps in two launches); with LES, the nine
//                    velocity gradients, the viscosity (k_les_nu) and the
//                    nine sweeps of nu (du_ij + du_ji); k_ns_presolve
//   boundary values  k_ns_bc_velocity (+ gradient of extrapol(phi), pt = 1)
//   velocity solves  k_ns_fu (interior rhs) + three Helmholtz solves, u on
//                    the caller's stream, v and w on forked streams (before
//                    the pressure for pt 1, 2; after the projection, with the
//                    new pressure gradient, for pt 3, 4)
//   pressure         k_ns_scale / k_ns_phi_rhs, div of rhs_p, k_ns_fphi,
//                    k_ns_bc_phi (+ k_ns_rot_sums, k_ns_bc_rotrot for pt 3),
//                    one all-Neumann Poisson solve at sigma = 0
//   projection       k_ns_pressure, k_ns_velocity
// Pointwise kernels fuse the edge zeroing of field_zero_edges
// (class_field.f90:366-391) into their stores.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mf_internal.h"

namespace mf {
namespace {

constexpr int kNsThreads = 256;
constexpr int kNt = 4;
constexpr int kDiagSums = 11;
constexpr int kWRows = 16;  // y rows per CTA of the weighted sums

inline unsigned ns_blocks(long long n) { return (unsigned)((n + kNsThreads - 1) / kNsThreads); }

__device__ __forceinline__ void idx3(long long q, int nx, int ny, int& i, int& j, int& k) {
  i = (int)(q % nx);
  const long long r = q / nx;
  j = (int)(r % ny);
  k = (int)(r / ny);
}

// A point on an edge or a corner: at least two indices on the boundary.
__device__ __forceinline__ bool on_edge(int i, int j, int k, int nx, int ny, int nz) {
  return (i == 0 || i == nx - 1) + (j == 0 || j == ny - 1) + (k == 0 || k == nz - 1) >= 2;
}

// Exact solution and sources of the reference at grid points, t with
// cos(wt t) = 1, sin(wt t) = 0 (wt = 0): ex[0] = u, ex[1] = v, ex[2] = p,
// ex[3] = rhsu, ex[4] = rhsv (w and rhsw are 0).  Same expression order as
// sol (class_navier_3D.f90:1005-1036).
__global__ void k_ns_exact(const double* __restrict__ gx, const double* __restrict__ gy,
                           const double* __restrict__ gz, int nx, int ny, int nz, int nmodes, double pi,
                           double rey, double* __restrict__ ex) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  const double x = gx[i], y = gy[j];
  (void)gz;
  double u = 0.0, v = 0.0, p = 0.0, fu = 0.0, fv = 0.0;
  const double a = 1.0, b = 1.0, ct = 1.0, st = 0.0;
  for (int m = 1; m <= nmodes; ++m) {
    const double wx = pi * m, wy = pi * m, wp = pi * m, wt = 0.0 * m * pi;
    const double sx = sin(wx * x), cx = cos(wx * x), sy = sin(wy * y), cy = cos(wy * y);
    const double cyx = cos(wp * (y - x));
    u = u + a * sx * cy * ct / wx;
    v = v - a * cx * sy * ct / wy;
    p = p + b * sin(wp * (x - y)) * ct;
    fu = fu + (b * wp * ct * cyx + a * a * (ct * ct) * cx * sx * (sy * sy + cy * cy) / wx +
               a * ct * sx * cy * (wy * wy / wx + wx) / rey - a * wt * st * sx * cy / wx);
    fv = fv + (-b * wp * ct * cyx + a * a * (ct * ct) * cy * sy * (sx * sx + cx * cx) / wy -
               a * ct * cx * sy * (wy + wx * wx / wy) / rey + a * wt * st * cx * sy / wy);
  }
  ex[q] = u;
  ex[n + q] = v;
  ex[2 * n + q] = p;
  ex[3 * n + q] = fu;
  ex[4 * n + q] = fv;
}

// Face arrays of one variable: bcx (ny-2, nz-2, 2), bcy (nx-2, nz-2, 2),
// bcz (nx-2, ny-2, 2), stored one after the other (Fortran order each).
struct Faces {
  int nx, ny, nz;
  long long sx, sy, sz;  // sizes of bcx, bcy, bcz
  __device__ __forceinline__ long long total() const { return sx + sy + sz; }
  // Face point q -> grid index (i, j, k) and the tangential derivative
  // axis selector a (0 = x face, 1 = y face, 2 = z face).
  __device__ __forceinline__ void point(long long q, int& a, int& i, int& j, int& k) const {
    if (q < sx) {
      a = 0;
      const int n2 = ny - 2, n3 = nz - 2;
      j = (int)(q % n2) + 1;
      k = (int)((q / n2) % n3) + 1;
      i = (q / ((long long)n2 * n3)) ? nx - 1 : 0;
    } else if (q < sx + sy) {
      q -= sx;
      a = 1;
      const int n1 = nx - 2, n3 = nz - 2;
      i = (int)(q % n1) + 1;
      k = (int)((q / n1) % n3) + 1;
      j = (q / ((long long)n1 * n3)) ? ny - 1 : 0;
    } else {
      q -= sx + sy;
      a = 2;
      const int n1 = nx - 2, n2 = ny - 2;
      i = (int)(q % n1) + 1;
      j = (int)((q / n1) % n2) + 1;
      k = (q / ((long long)n1 * n2)) ? nz - 1 : 0;
    }
  }
};

// Exact face values of u, v (w = 0): bcex[c * total + q] from the exact fields.
__global__ void k_ns_bc_exact(Faces F, const double* __restrict__ ex, long long n, double* __restrict__ bcex) {
  const long long tot = F.total();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tot) return;
  int a, i, j, k;
  F.point(q, a, i, j, k);
  const long long g = i + (long long)F.nx * (j + (long long)F.ny * k);
  bcex[q] = ex[g];
  bcex[tot + q] = ex[n + g];
  bcex[2 * tot + q] = 0.0;
}

// navier_bc_velocity + add_boundary_gradient (class_navier_3D.f90:395-433,
// 695-791): bc of u, v, w = exact values; with d (pt = 1) the tangential
// components get + d_t(extrapol(phi)) / fac(1): v and w on the x faces, u and
// w on the y faces, u and v on the z faces.  d[0..2] = d/dx, d/dy, d/dz.
__global__ void k_ns_bc_velocity(Faces F, const double* __restrict__ bcex, const double* __restrict__ dx,
                                 const double* __restrict__ dy, const double* __restrict__ dz, double fac1,
                                 double* __restrict__ bc) {
  const long long tot = F.total();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tot) return;
  int a, i, j, k;
  F.point(q, a, i, j, k);
  const long long g = i + (long long)F.nx * (j + (long long)F.ny * k);
  for (int c = 0; c < 3; ++c) {
    double val = bcex[c * tot + q];
    if (dx && c != a) {
      const double* d = c == 0 ? dx : c == 1 ? dy : dz;
      val = val + d[g] / fac1;
    }
    bc[c * tot + q] = val;
  }
}

// navier_bc_pressure (class_navier_3D.f90:342-393), one domain:
// bcphi on the faces normal to axis a = rhs_p(a)(face) - fac(1) bc of the
// normal velocity component.
__global__ void k_ns_bc_phi(Faces F, const double* __restrict__ rpx, const double* __restrict__ rpy,
                            const double* __restrict__ rpz, const double* __restrict__ bcvel, double fac1,
                            double* __restrict__ bcphi) {
  const long long tot = F.total();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tot) return;
  int a, i, j, k;
  F.point(q, a, i, j, k);
  const long long g = i + (long long)F.nx * (j + (long long)F.ny * k);
  const double* rp = a == 0 ? rpx : a == 1 ? rpy : rpz;
  bcphi[q] = rp[g] - fac1 * bcvel[a * tot + q];
}

// Linear combination of up to three time levels (navier_extrapol,
// class_navier_3D.f90:2010-2050): out = c0 a0 + c1 a1 + c2 a2 (m terms, m = 0
// gives 0), edges zeroed.
struct Lin {
  int m;
  double c[3];
  const double* a[3];
};

__device__ __forceinline__ double lin_at(const Lin& L, long long q) {
  if (L.m == 0) return 0.0;
  double acc = L.c[0] * L.a[0][q];
  if (L.m > 1) acc = acc + L.c[1] * L.a[1][q];
  if (L.m > 2) acc = acc + L.c[2] * L.a[2][q];
  return acc;
}

__global__ void k_ns_extrapol(Lin L, int nx, int ny, int nz, double* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  out[q] = on_edge(i, j, k, nx, ny, nz) ? 0.0 : lin_at(L, q);
}

// The three components c of navier_nonlinear at one slot in one launch
// (blockIdx.y = c).  D holds the nine derivatives d x_c / d x_d at
// D + (3 d + c) n; out_c = out + c ostride.  nlt 1: u dx + v dy + w dz;
// nlt 2: half of it (class_navier_3D.f90:1195-1206); nlt 0: 0.
__global__ void k_ns_advect(long long n, int nlt, const double* __restrict__ u, const double* __restrict__ v,
                            const double* __restrict__ w, const double* __restrict__ D,
                            double* __restrict__ out, long long ostride) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int c = blockIdx.y;
  double* o = out + c * ostride;
  if (nlt != 1 && nlt != 2) {
    o[q] = 0.0;
    return;
  }
  double t = u[q] * D[c * n + q] + v[q] * D[(3 + c) * n + q] + w[q] * D[(6 + c) * n + q];
  if (nlt == 2) t = t * 0.5;
  o[q] = t;
}

// Products of the skew-symmetric form: P + (3 d + c) n = x_c u_d with
// x_c = x + c xstride (u, v, w of one slot), u_d = u, v, w (blockIdx.y = c).
__global__ void k_ns_products(long long n, const double* __restrict__ x, long long xstride,
                              const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, double* __restrict__ P) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int c = blockIdx.y;
  const double xv = x[c * xstride + q];
  P[c * n + q] = xv * u[q];
  P[(3 + c) * n + q] = xv * v[q];
  P[(6 + c) * n + q] = xv * w[q];
}

// nlt 2, second half (:1208-1213): out_c += d(x_c u)/dx 0.5, then
// d(x_c v)/dy 0.5, then d(x_c w)/dz 0.5, with E + (3 d + c) n the
// derivatives of the products.
__global__ void k_ns_skew(long long n, const double* __restrict__ E, double* __restrict__ out, long long ostride) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int c = blockIdx.y;
  double* o = out + c * ostride;
  double t = o[q];
  t = t + E[c * n + q] * 0.5;
  t = t + E[(3 + c) * n + q] * 0.5;
  t = t + E[(6 + c) * n + q] * 0.5;
  o[q] = t;
}

// LES stress products (class_navier_3D.f90:1090-1094):
// P + (3 j + i) n = nu (du_ij + du_ji), du_ij at D + (3 j + i) n.
__global__ void k_ns_les_products(long long n, const double* __restrict__ nu, const double* __restrict__ D,
                                  double* __restrict__ P) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double v = nu[q];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) P[(3 * j + i) * n + q] = v * (D[(3 * j + i) * n + q] + D[(3 * i + j) * n + q]);
}

// navier_presolve_{u,v,w} (class_navier_3D.f90:1528-1595):
// rhs = zero_edges(f - zero_edges(extrapol(nonlinear))) with f the exact
// source (src, null for w), minus the LES term les_f = -sum_j E_j (E: the
// three sweeps of component c, E + j n3 with n3 = 3 n, null without LES),
// plus the flow-rate term g (u only, *g).
__global__ void k_ns_presolve(Lin L, int nx, int ny, int nz, const double* __restrict__ src,
                              const double* __restrict__ E, const double* __restrict__ g,
                              double* __restrict__ rhs) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  if (on_edge(i, j, k, nx, ny, nz)) {
    rhs[q] = 0.0;
    return;
  }
  double f = src ? src[q] : 0.0;
  if (E) {
    double lf = 0.0;
    lf = lf - E[q];
    lf = lf - E[3 * n + q];
    lf = lf - E[6 * n + q];
    f = f - lf;
  }
  if (g) f = f + g[0];
  rhs[q] = f - lin_at(L, q);
}

// navier_solve_{u,v,w} right-hand side (class_navier_3D.f90:1612-1635) at the
// interior points, written as the solver's interior array (full = 0) or at
// the interior points of a full field (full = 1, the multidomain solve):
// fu = Re (((fac2 x_n + fac3 x_n-1) [+ fac4 x_n-2] [+ grad]) - rhs).
__global__ void k_ns_fu(int nx, int ny, int nz, const double* __restrict__ x0, const double* __restrict__ x1,
                        const double* __restrict__ x2, double f2, double f3, double f4,
                        const double* __restrict__ grad, const double* __restrict__ rhs, double rey, int full,
                        double* __restrict__ out) {
  const int n1 = nx - 2, n2 = ny - 2, n3 = nz - 2;
  const long long n = (long long)n1 * n2 * n3;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, n1, n2, i, j, k);
  const long long g = (i + 1) + (long long)nx * ((j + 1) + (long long)ny * (k + 1));
  double f = 0.0;
  f = f + f2 * x0[g] + f3 * x1[g];
  if (x2) f = f + f4 * x2[g];
  if (grad) f = f + grad[g];
  f = f - rhs[g];
  out[full ? g : q] = rey * f;
}

// out = zero_edges(s x)  (navier_phi_rhs, pt <= 2: fac(1) u*).
__global__ void k_ns_scale(int nx, int ny, int nz, double s, const double* __restrict__ x,
                           double* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  out[q] = on_edge(i, j, k, nx, ny, nz) ? 0.0 : s * x[q];
}

// navier_phi_rhs for pt = 3, 4 (class_navier_3D.f90:1983-2003):
// pt 3: f1 - fac2 x(it(nt)) - fac3 x(it(nt-1)) - fac4 x(it(nt-2));
// pt 4: that - f2 + fac1 x(it(nt)) + fac2 x(it(nt-1)) + fac3 x(it(nt-2)) + fac4 x(it(1));
// edges zeroed.  f1, f2 = rhs(1), rhs(2) of the component.
__global__ void k_ns_phi_rhs(int nx, int ny, int nz, int pt, const double* __restrict__ f1,
                             const double* __restrict__ f2, const double* __restrict__ x0,
                             const double* __restrict__ x1, const double* __restrict__ x2,
                             const double* __restrict__ x3, double fa, double fb, double fc, double fd,
                             double* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  if (on_edge(i, j, k, nx, ny, nz)) {
    out[q] = 0.0;
    return;
  }
  double t;
  if (pt == 5) {  // pt 4 from the second sub-iteration on: f1 - f2 + fac1 x(it(1))
    t = f1[q] - f2[q] + fa * x3[q];
  } else {
    t = f1[q] - fb * x0[q] - fc * x1[q] - fd * x2[q];
    if (pt == 4) t = t - f2[q] + fa * x0[q] + fb * x1[q] + fc * x2[q] + fd * x3[q];
  }
  out[q] = t;
}

// add_boundary_rotrot, first half (class_navier_3D.f90:819-840): with
// A = d eu/dx, B = d ev/dy, C = d ew/dz of the extrapolated velocity,
// ax = B + C, ay = A + C, az = A + B.
__global__ void k_ns_rot_sums(long long n, const double* __restrict__ A, const double* __restrict__ B,
                              const double* __restrict__ C, double* __restrict__ ax, double* __restrict__ ay,
                              double* __restrict__ az) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  ax[q] = B[q] + C[q];
  ay[q] = A[q] + C[q];
  az[q] = A[q] + B[q];
}

// add_boundary_rotrot, second half: on the faces normal to axis a,
// bcphi -= (d(a_a)/dx_a - dd1 - dd2) / Re with d[a] = d(a_a)/dx_a and
// dd[2a], dd[2a+1] the two second derivatives of that face's normal velocity
// component (x: u_yy, u_zz; y: v_xx, v_zz; z: w_xx, w_yy).
struct RotRot {
  const double* d[3];
  const double* dd[6];
};
__global__ void k_ns_bc_rotrot(Faces F, RotRot R, double rey, double* __restrict__ bcphi) {
  const long long tot = F.total();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tot) return;
  int a, i, j, k;
  F.point(q, a, i, j, k);
  const long long g = i + (long long)F.nx * (j + (long long)F.ny * k);
  const double aux = R.d[a][g] - R.dd[2 * a][g] - R.dd[2 * a + 1][g];
  bcphi[q] = bcphi[q] - aux / rey;
}

// navier_solve_phi right-hand side at the interior points
// (class_navier_3D.f90:1808-1813): sigmap extrapol(phi) + d rhs_px/dx +
// d rhs_py/dy + d rhs_pz/dz.
__global__ void k_ns_fphi(int nx, int ny, int nz, double sigmap, const double* __restrict__ ext,
                          const double* __restrict__ ddx, const double* __restrict__ ddy,
                          const double* __restrict__ ddz, int full, double* __restrict__ out) {
  const int n1 = nx - 2, n2 = ny - 2, n3 = nz - 2;
  const long long n = (long long)n1 * n2 * n3;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, n1, n2, i, j, k);
  const long long g = (i + 1) + (long long)nx * ((j + 1) + (long long)ny * (k + 1));
  double f = sigmap * ext[g];
  f = f + ddx[g] + ddy[g] + ddz[g];
  out[full ? g : q] = f;
}

// In-place field_zero_edges.
__global__ void k_ns_zero_edges(int nx, int ny, int nz, double* __restrict__ f) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  if (on_edge(i, j, k, nx, ny, nz)) f[q] = 0.0;
}

// navier_projection, pressure (class_navier_3D.f90:1878-1896):
// p = zero_edges(zero_edges(phi [+ aux]) [- (div_x + div_y + div_z) / Re])
// (no divergence term when ddx is null: pt = 3).
__global__ void k_ns_pressure(int nx, int ny, int nz, const double* __restrict__ phi,
                              const double* __restrict__ aux, const double* __restrict__ ddx,
                              const double* __restrict__ ddy, const double* __restrict__ ddz, double rey,
                              double* __restrict__ p) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  if (on_edge(i, j, k, nx, ny, nz)) {
    p[q] = 0.0;
    return;
  }
  double v = phi[q];
  if (aux) v = v + aux[q];
  if (ddx) v = v - (ddx[q] + ddy[q] + ddz[q]) / rey;
  p[q] = v;
}

// navier_projection, velocity (:1943-1949): x = zero_edges((rhs_p - dphi) / fac(1)).
__global__ void k_ns_velocity(int nx, int ny, int nz, const double* __restrict__ rp,
                              const double* __restrict__ dphi, double fac1, double* __restrict__ x) {
  const long long n = (long long)nx * ny * nz;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int i, j, k;
  idx3(q, nx, ny, i, j, k);
  x[q] = on_edge(i, j, k, nx, ny, nz) ? 0.0 : (rp[q] - dphi[q]) / fac1;
}

// Quadrature weight of integrale / norme2 (class_navier_3D.f90:2419-2603):
// half widths w_x(i) w_y(j) w_z(k) at the interior and face points, 0 on
// edges and corners.
struct Weights {
  const double *wx, *wy, *wz;
  int nx, ny, nz;
  __device__ __forceinline__ double at(int i, int j, int k) const {
    return on_edge(i, j, k, nx, ny, nz) ? 0.0 : wx[i] * wy[j] * wz[k];
  }
};

// Block sums of kS quantities in a fixed order; thread 0 writes them.
template <int kS>
__device__ __forceinline__ void block_sums(double (&acc)[kS], double* __restrict__ out) {
  __shared__ double red[kS][kNsThreads];
#pragma unroll
  for (int s = 0; s < kS; ++s) red[s][threadIdx.x] = acc[s];
  __syncthreads();
  for (int h = kNsThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int s = 0; s < kS; ++s) red[s][threadIdx.x] += red[s][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int s = 0; s < kS; ++s) out[s] = red[s][0];
}

// part[k * G + g] = sum over the y rows of chunk g of plane k of W f.
// Grid (nz, G = ceil(ny / kWRows)).
__global__ void __launch_bounds__(kNsThreads) k_ns_wsum(Weights W, const double* __restrict__ f,
                                                        double* __restrict__ part) {
  const int k = blockIdx.x, j0 = blockIdx.y * kWRows, j1 = min(W.ny, j0 + kWRows);
  double acc[1] = {0.0};
  for (int j = j0; j < j1; ++j)
    for (int i = threadIdx.x; i < W.nx; i += kNsThreads)
      acc[0] += W.at(i, j, k) * f[i + (long long)W.nx * (j + (long long)W.ny * k)];
  block_sums<1>(acc, part + (long long)k * gridDim.y + blockIdx.y);
}

// out[s] = sum over p of part[p * nsum + s], one CTA, fixed order.
__global__ void __launch_bounds__(kNsThreads) k_ns_sum_parts(const double* __restrict__ part, int count,
                                                             int nsum, double* __restrict__ out) {
  __shared__ double red[kNsThreads];
  for (int s = 0; s < nsum; ++s) {
    double acc = 0.0;
    for (int p = threadIdx.x; p < count; p += kNsThreads) acc += part[(long long)p * nsum + s];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kNsThreads / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = red[0];
    __syncthreads();
  }
}

// out = x[0] + x[1] + ... + x[n-1] in this order (the per-subdomain sums
// of the flow-rate integral), one thread.
__global__ void k_ns_sum_small(const double* __restrict__ x, int n, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i];
  out[0] = s;
}

// Flow-rate term of f for u (class_navier_3D.f90:1140-1164), one thread:
// err = integrale(extrapol(u)) / integrale(1); on the first call debit = err
// (1 when <= 1e-10, a single-precision literal) and g = 3 debit; then
// g -= (err - debit) fac(1).  state = {g, debit, initialised}.
__global__ void k_ns_flow(const double* __restrict__ isum, double reft, double fac1, double thresh,
                          double* __restrict__ state) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double err = isum[0] / reft;
  if (state[2] == 0.0) {
    double debit = err;
    if (debit <= thresh) debit = 1.0;
    state[1] = debit;
    state[0] = 3.0 * debit;
    state[2] = 1.0;
  }
  err = err - state[1];
  state[0] = state[0] - err * fac1;
}

// Driver diagnostics (navier3d.f90:120-254), weighted sums in three phases.
struct DiagIn {
  const double *u, *v, *w, *p, *up, *vp, *wp, *pp;  // levels it(nt) and it(nt-1)
  const double *dx, *dy, *dz;                       // du/dx, dv/dy, dw/dz of it(nt)
  const double *ue, *ve, *pex;                      // exact fields
  double pexm, auxm;                                // means removed in phases 1, 2
  const double *su, *sv, *sw, *sp;                  // testconv: last sub-iterate
  double spm;                                       // testconv: mean shift of sp
};

// Grid (nz, G); part[(k G + g) kDiagSums + s].
template <int kPhase>
__global__ void __launch_bounds__(kNsThreads) k_ns_diag(Weights W, DiagIn D, double* __restrict__ part) {
  const int k = blockIdx.x, j0 = blockIdx.y * kWRows, j1 = min(W.ny, j0 + kWRows);
  double acc[kDiagSums];
#pragma unroll
  for (int s = 0; s < kDiagSums; ++s) acc[s] = 0.0;
  for (int j = j0; j < j1; ++j)
    for (int i = threadIdx.x; i < W.nx; i += kNsThreads) {
      const double wq = W.at(i, j, k);
      const long long q = i + (long long)W.nx * (j + (long long)W.ny * k);
      if (kPhase == 0) {
        const double div = D.dx[q] + D.dy[q] + D.dz[q];
        const double ue = D.ue[q], ve = D.ve[q], we = 0.0;
        const double r1 = sqrt(ue * ue + ve * ve + we * we);
        const double eu = ue - D.u[q], ev = ve - D.v[q], ew = we - D.w[q];
        const double r2 = sqrt(eu * eu + ev * ev + ew * ew);
        const double du = D.u[q] - D.up[q], dv = D.v[q] - D.vp[q], dw = D.w[q] - D.wp[q];
        acc[0] += wq * div * div;
        acc[1] += wq * r1 * r1;
        acc[2] += wq * r2 * r2;
        acc[3] += wq * D.p[q];
        acc[4] += wq * D.u[q] * D.u[q];
        acc[5] += wq * D.v[q] * D.v[q];
        acc[6] += wq * D.w[q] * D.w[q];
        acc[7] += wq * du * du;
        acc[8] += wq * dv * dv;
        acc[9] += wq * dw * dw;
        acc[10] += wq * D.pex[q];
      } else if (kPhase == 1) {
        const double pe = D.pex[q] - D.pexm;
        const double e = D.p[q] - pe;
        acc[0] += wq * e * e;
        acc[1] += wq * pe * pe;
        acc[2] += wq * (D.p[q] - D.pp[q]);
      } else if (kPhase == 2) {
        const double a = (D.p[q] - D.pp[q]) - D.auxm;
        acc[0] += wq * a * a;
      } else if (kPhase == 3) {  // testconv (navier3d.f90:394-403), u..p = it(1)
        const double u = D.u[q], v = D.v[q], w = D.w[q];
        const double r = sqrt(u * u + v * v + w * w);
        const double eu = D.su[q] - u, ev = D.sv[q] - v, ew = D.sw[q] - w;
        const double e = sqrt(eu * eu + ev * ev + ew * ew);
        acc[0] += wq * r * r;
        acc[1] += wq * e * e;
        acc[2] += wq * (D.p[q] - D.sp[q]);
      } else {  // testconv (:405-407)
        const double sp = D.sp[q] + D.spm;
        const double e = D.p[q] - sp;
        acc[0] += wq * sp * sp;
        acc[1] += wq * e * e;
      }
    }
  block_sums<kDiagSums>(acc, part + ((long long)k * gridDim.y + blockIdx.y) * kDiagSums);
}

// f += s at every point (the driver's removal of the pressure mean).
__global__ void k_ns_shift(long long n, double s, double* __restrict__ f) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) f[q] = f[q] + s;
}

}  // namespace
}  // namespace mf

using namespace mf;

// One subdomain of the step: its fields, work arrays and coefficients (one
// domain: the whole box).
struct NsDom {
  int nx = 0, ny = 0, nz = 0, n1 = 0, n2 = 0, n3 = 0;
  long long np = 0, nin = 0;
  mf_der_t *dcx = nullptr, *dcy = nullptr, *dcz = nullptr;
  // one domain: velocity solver sets scu, scv, scw (as the reference keeps
  // them; the three velocity solves run on forked streams) and the pressure set
  mf_solver3d_t* sc[4] = {nullptr, nullptr, nullptr, nullptr};
  mf_les_t* les = nullptr;  // les_type != 0
  DevBuf nu;                // eddy viscosity of the step
  DevBuf fields;  // [5 vars][kNt slots] fields
  DevBuf nl;      // [3][kNt] cached nonlinear terms
  DevBuf rhs;     // [3][2] rhs_u(1), rhs_u(2) ...
  DevBuf rp;      // rhs_px, rhs_py, rhs_pz
  DevBuf tmp;     // 18 work fields
  DevBuf fin;     // right-hand sides of the solves: three interior arrays (one domain) or three full fields
  DevBuf exact;   // u, v, p, rhsu, rhsv of the exact solution
  DevBuf bcex;    // exact face values of u, v, w
  DevBuf bc;      // face values of u, v, w, phi
  DevBuf grid;    // gx, gy, gz
  DevBuf wts;     // half widths wx, wy, wz
  DevBuf part;    // partial sums
  DevBuf sums;    // summed values
  DevBuf sub;     // last sub-iterate u, v, w, p (nsubite > 1)
  Faces faces{};
  double reft = 0.0;  // integrale(1) over this subdomain

  double* F(int var, int slot) const { return fields.as<double>() + ((size_t)var * kNt + slot) * np; }
  double* NL(int c, int slot) const { return nl.as<double>() + ((size_t)c * kNt + slot) * np; }
  double* RHS(int c, int which) const { return rhs.as<double>() + ((size_t)c * 2 + which) * np; }
  double* RP(int c) const { return rp.as<double>() + (size_t)c * np; }
  double* T(int t) const { return tmp.as<double>() + (size_t)t * np; }
  double* EX(int q) const { return exact.as<double>() + (size_t)q * np; }
  double* BC(int c) const { return bc.as<double>() + (size_t)c * (faces.sx + faces.sy + faces.sz); }
  Weights weights() const {
    const double* w = wts.as<double>();
    return Weights{w, w + nx, w + nx + ny, nx, ny, nz};
  }
  void release() {
    mf_der_destroy(dcx);
    mf_der_destroy(dcy);
    mf_der_destroy(dcz);
    for (mf_solver3d_t* s : sc) mf_solver3d_destroy(s);
    mf_les_destroy(les);
    for (DevBuf* b : {&nu, &fields, &nl, &rhs, &rp, &tmp, &fin, &exact, &bcex, &bc, &grid, &wts, &part, &sums, &sub})
      b->release();
  }
};

struct mf_navier {
  mf_navier_params_t prm;
  double fac[4] = {0, 0, 0, 0};
  double sigmau = 0.0, sigmap = 0.0, time = 0.0;
  int it[kNt] = {0, 1, 2, 3};
  int subite = 1, subiterations = 0;
  bool nl_ok[kNt] = {false, false, false, false};
  int rhs_cur = 0;
  std::vector<NsDom> dom;  // subdomains, index i + nd1 (j + nd2 k)
  int nd[3] = {1, 1, 1};
  mf_md_t *mdu = nullptr, *mdp = nullptr;  // multidomain: velocity and pressure influence-matrix solves
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
  DevBuf state;  // flow-rate term: g, debit, initialised
  DevBuf dsum;   // per-subdomain sums of the flow-rate integral, then their total
  double reft = 0.0;  // integrale(1) over all subdomains
  double err_vts = 0.0, err_pre = 0.0;
  const mf_mlp_t* les_mlp = nullptr;  // les_type 4: the caller's network (not owned)
  bool md() const { return mdu != nullptr; }
};

namespace {

constexpr int kVarU = 0, kVarP = 3, kVarPhi = 4;

// extrapol of var (navier_extrapol) of the given order: -1 -> it(1); 1 ->
// it(nt); 2 -> 2 it(nt) - it(nt-1); 3 -> 3 it(nt) - 3 it(nt-1) + it(nt-2);
// else 0; from the second sub-iteration on it(1) whatever the order.
Lin extrapol_of(const mf_navier* nv, const NsDom& d, int order, bool nonlin, int var) {
  Lin L{};
  const int* it = nv->it;
  auto P = [&](int s) { return nonlin ? d.NL(var, s) : d.F(var, s); };
  if (nv->subite > 1) {  // from the second sub-iteration on: the current iterate
    L.m = 1; L.c[0] = 1.0; L.a[0] = P(it[0]);
  } else if (order == -1) {
    L.m = 1; L.c[0] = 1.0; L.a[0] = P(it[0]);
  } else if (order == 1) {
    L.m = 1; L.c[0] = 1.0; L.a[0] = P(it[kNt - 1]);
  } else if (order == 2) {
    L.m = 2; L.c[0] = 2.0; L.a[0] = P(it[kNt - 1]); L.c[1] = -1.0; L.a[1] = P(it[kNt - 2]);
  } else if (order == 3) {
    L.m = 3; L.c[0] = 3.0; L.a[0] = P(it[kNt - 1]); L.c[1] = -3.0; L.a[1] = P(it[kNt - 2]);
    L.c[2] = 1.0; L.a[2] = P(it[kNt - 3]);
  } else {
    L.m = 0;
  }
  return L;
}

// Slots whose nonlinear terms extrapol('v') reads.
int extrapol_slots(const mf_navier* nv, int order, int slots[3]) {
  const int* it = nv->it;
  if (nv->subite > 1 || order == -1) {
    slots[0] = it[0];
    return 1;
  }
  if (order < 1 || order > 3) return 0;
  for (int t = 0; t < order; ++t) slots[t] = it[kNt - 1 - t];
  return order;
}

int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MF_OK : cuda_error(e, what);
}

int extrapol_into(const NsDom& d, const Lin& L, double* out, cudaStream_t st) {
  k_ns_extrapol<<<ns_blocks(d.np), kNsThreads, 0, st>>>(L, d.nx, d.ny, d.nz, out);
  return launch_check("k_ns_extrapol");
}

// Independent derivative sweeps of a subdomain's fields, launched together
// (mf_der_apply_many): the lines of one 128 x 129 x 128 sweep alone fill a
// GB300 only to ~3 warps per SM.
struct Sweeps {
  int n = 0;
  const mf_der_t* dc[9];
  int axis[9], order[9];
  const double* f[9];
  double* df[9];
  void add(const NsDom& d, int ax, const double* in, double* out, int ord = 1) {
    dc[n] = ax == 0 ? d.dcx : ax == 1 ? d.dcy : d.dcz;
    axis[n] = ax;
    order[n] = ord;
    f[n] = in;
    df[n] = out;
    ++n;
  }
  int run(const NsDom& d, cudaStream_t st) const {
    return mf_der_apply_many(n, dc, axis, order, f, df, d.nx, d.ny, d.nz, st);
  }
};

// Gradient of f: d/dx, d/dy, d/dz into out0, out1, out2.
int gradient(const NsDom& d, const double* f, double* out0, double* out1, double* out2, cudaStream_t st) {
  Sweeps S;
  S.add(d, 0, f, out0);
  S.add(d, 1, f, out1);
  S.add(d, 2, f, out2);
  return S.run(d, st);
}

// navier_nonlinear of the three components at `slot` into their cache
// entries: nine sweeps d x_c / d x_d in one launch, and for nlt 2 the nine
// products x_c u_d and their sweeps in another.
int nonlinear_slot(const mf_navier* nv, NsDom& d, int slot, cudaStream_t st) {
  const long long n = d.np;
  const double *u = d.F(0, slot), *v = d.F(1, slot), *w = d.F(2, slot);
  const long long xstride = d.F(1, slot) - d.F(0, slot);
  const long long ostride = d.NL(1, slot) - d.NL(0, slot);
  const dim3 grid(ns_blocks(n), 3);
  const int nlt = nv->prm.nlt;
  int rc;
  if (nlt == 1 || nlt == 2) {
    Sweeps S;
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) S.add(d, a, d.F(c, slot), d.T(3 * a + c));
    if ((rc = S.run(d, st))) return rc;
  }
  k_ns_advect<<<grid, kNsThreads, 0, st>>>(n, nlt, u, v, w, d.T(0), d.NL(0, slot), ostride);
  if ((rc = launch_check("k_ns_advect"))) return rc;
  if (nlt == 2) {
    k_ns_products<<<grid, kNsThreads, 0, st>>>(n, u, xstride, u, v, w, d.T(9));
    if ((rc = launch_check("k_ns_products"))) return rc;
    Sweeps S;
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) S.add(d, a, d.T(9 + 3 * a + c), d.T(3 * a + c));
    if ((rc = S.run(d, st))) return rc;
    k_ns_skew<<<grid, kNsThreads, 0, st>>>(n, d.T(0), d.NL(0, slot), ostride);
    if ((rc = launch_check("k_ns_skew"))) return rc;
  }
  return MF_OK;
}

// Face-array pointers of variable c (0..3 = u, v, w, phi) of every subdomain.
struct FacePtrs {
  std::vector<const double*> x, y, z;
};
FacePtrs face_ptrs(const mf_navier* nv, int c) {
  FacePtrs p;
  for (const NsDom& d : nv->dom) {
    const double* b = d.BC(c);
    p.x.push_back(b);
    p.y.push_back(b + d.faces.sx);
    p.z.push_back(b + d.faces.sx + d.faces.sy);
  }
  return p;
}

// Weighted sum of f over subdomain d into d.sums[0] (device).
int wsum(NsDom& d, const double* f, double* out, cudaStream_t st) {
  const int groups = (d.ny + kWRows - 1) / kWRows;
  k_ns_wsum<<<dim3(d.nz, groups), kNsThreads, 0, st>>>(d.weights(), f, d.part.as<double>());
  k_ns_sum_parts<<<1, kNsThreads, 0, st>>>(d.part.as<double>(), d.nz * groups, 1, out);
  return launch_check("k_ns_wsum");
}

}  // namespace

namespace {

// One domain: the solver's own solve of the interior right-hand side rhs.
int solve_one(const mf_navier* nv, const NsDom& d, mf_solver3d_t* sc, const double* rhs, double sigma,
              double* solf, int c, cudaStream_t st) {
  const double* b = d.BC(c);
  const double* bx = b;
  const double* by = b + d.faces.sx;
  const double* bz = b + d.faces.sx + d.faces.sy;
  if (nv->prm.precision == MF_PREC_FP64) return mf_solve_3d(sc, rhs, sigma, solf, bx, by, bz, d.n1, d.n2, d.n3, st);
  return mf_solve_3d_mixed(sc, rhs, sigma, solf, bx, by, bz, d.n1, d.n2, d.n3, nv->prm.precision, nv->prm.refine,
                           st);
}

// Multidomain: one multidomain_solve of variable var (face arrays of c) with
// the full right-hand-side fields in each subdomain's fin.
int solve_md(mf_navier* nv, mf_md_t* md, int var, int c, int slot, cudaStream_t st) {
  std::vector<const double*> g;
  std::vector<double*> u;
  for (NsDom& d : nv->dom) {
    g.push_back(d.fin.as<double>());
    u.push_back(d.F(var, slot));
  }
  FacePtrs b = face_ptrs(nv, c);
  return mf_md_solve(md, g.data(), u.data(), b.x.data(), b.y.data(), b.z.data(), st);
}

// navier_solve_{u,v,w}: the three Helmholtz solves into slot it(1); with
// grad, each subdomain's T(1 + c) is added to the right-hand side.  One
// domain: u on the caller's stream, v and w on forked streams joined back.
int velocity_solves(mf_navier* nv, bool grad, cudaStream_t st) {
  const mf_navier_params_t& P = nv->prm;
  const int nw = nv->it[0], s0 = nv->it[kNt - 1], s1 = nv->it[kNt - 2], s2 = nv->it[kNt - 3];
  int rc;
  auto fu = [&](NsDom& d, int c, int full, double* out, cudaStream_t sc) {
    k_ns_fu<<<ns_blocks(full ? d.np : d.nin), kNsThreads, 0, sc>>>(
        d.nx, d.ny, d.nz, d.F(c, s0), d.F(c, s1), P.tou == 3 ? d.F(c, s2) : nullptr, nv->fac[1], nv->fac[2],
        nv->fac[3], grad ? d.T(1 + c) : nullptr, d.RHS(c, nv->rhs_cur), P.reynolds, full, out);
    return launch_check("k_ns_fu");
  };
  if (nv->md()) {
    // the three right-hand sides first, then one multidomain solve for all
    // of them (one pass over the interface inverse)
    std::vector<const double*> g;
    std::vector<double*> u;
    std::vector<const double*> bx, by, bz;
    for (int c = 0; c < 3; ++c) {
      for (NsDom& d : nv->dom) {
        double* rhs = d.fin.as<double>() + (size_t)c * d.np;
        if ((rc = fu(d, c, 1, rhs, st))) return rc;
        g.push_back(rhs);
        u.push_back(d.F(c, nw));
      }
      FacePtrs b = face_ptrs(nv, c);
      bx.insert(bx.end(), b.x.begin(), b.x.end());
      by.insert(by.end(), b.y.begin(), b.y.end());
      bz.insert(bz.end(), b.z.begin(), b.z.end());
    }
    return mf_md_solve_many(nv->mdu, 3, g.data(), u.data(), bx.data(), by.data(), bz.data(), st);
  }
  NsDom& d = nv->dom[0];
  MF_CUDA(cudaEventRecord(nv->fork, st));
  for (int q = 0; q < 2; ++q) MF_CUDA(cudaStreamWaitEvent(nv->side[q], nv->fork, 0));
  for (int c = 0; c < 3; ++c) {
    cudaStream_t sc = c == 0 ? st : nv->side[c - 1];
    double* rhs = d.fin.as<double>() + (size_t)c * d.nin;
    if ((rc = fu(d, c, 0, rhs, sc)) || (rc = solve_one(nv, d, d.sc[c], rhs, nv->sigmau, d.F(c, nw), c, sc)))
      return rc;
  }
  for (int q = 0; q < 2; ++q) {
    MF_CUDA(cudaEventRecord(nv->join[q], nv->side[q]));
    MF_CUDA(cudaStreamWaitEvent(st, nv->join[q], 0));
  }
  return MF_OK;
}

// Presolve of one subdomain: navier_LES and the stress sweeps of f, then
// rhs = f - extrapol(nonlinear) for u, v, w (class_navier_3D.f90:1528-1595).
int presolve(const mf_navier* nv, NsDom& d, const double* g, cudaStream_t st) {
  const mf_navier_params_t& P = nv->prm;
  const int s0 = nv->it[kNt - 1];
  const unsigned gb = ns_blocks(d.np);
  int rc;
  if (P.les_type != 0) {
    Sweeps S;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) S.add(d, j, d.F(i, s0), d.T(3 * j + i));
    if ((rc = S.run(d, st))) return rc;
    const double* du[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) du[3 * i + j] = d.T(3 * j + i);
    // les_type 4: the learned coefficient where the features are inside the
    // network's training range, Smagorinsky with les_c^2 elsewhere
    if (P.les_type == MF_LES_LEARNED) {
      if (!nv->les_mlp)
        return set_error(MF_ERR_ARG, "mf_navier_step: les_type 4 needs a network (mf_navier_set_les_network)");
      if ((rc = mf_les_nu_mlp(d.les, nv->les_mlp, P.les_c * P.les_c, du, d.nu.as<double>(), nullptr, st)))
        return rc;
    } else if ((rc = mf_les_nu(d.les, P.les_type, P.les_c * P.les_c, du, d.nu.as<double>(), st))) {
      return rc;
    }
    k_ns_les_products<<<gb, kNsThreads, 0, st>>>(d.np, d.nu.as<double>(), d.T(0), d.T(9));
    if ((rc = launch_check("k_ns_les_products"))) return rc;
    Sweeps E;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) E.add(d, j, d.T(9 + 3 * j + i), d.T(3 * j + i));
    if ((rc = E.run(d, st))) return rc;
  }
  for (int c = 0; c < 3; ++c) {
    const double* src = c == 0 ? d.EX(3) : c == 1 ? d.EX(4) : nullptr;
    k_ns_presolve<<<gb, kNsThreads, 0, st>>>(extrapol_of(nv, d, P.tou, true, c), d.nx, d.ny, d.nz, src,
                                             P.les_type != 0 ? d.T(c) : nullptr, c == 0 ? g : nullptr,
                                             d.RHS(c, nv->rhs_cur));
    if ((rc = launch_check("k_ns_presolve"))) return rc;
  }
  return MF_OK;
}

// Velocity boundary values (+ gradient of extrapol(phi) for pt = 1).
int velocity_bc(const mf_navier* nv, NsDom& d, cudaStream_t st) {
  const double fac1 = nv->fac[0];
  const unsigned fb = ns_blocks(d.faces.sx + d.faces.sy + d.faces.sz);
  int rc;
  if (nv->prm.pt == 1) {
    if ((rc = extrapol_into(d, extrapol_of(nv, d, nv->prm.top - 1, false, kVarPhi), d.T(0), st)) ||
        (rc = gradient(d, d.T(0), d.T(1), d.T(2), d.T(3), st)))
      return rc;
    k_ns_bc_velocity<<<fb, kNsThreads, 0, st>>>(d.faces, d.bcex.as<double>(), d.T(1), d.T(2), d.T(3), fac1,
                                                d.bc.as<double>());
  } else {
    k_ns_bc_velocity<<<fb, kNsThreads, 0, st>>>(d.faces, d.bcex.as<double>(), nullptr, nullptr, nullptr, fac1,
                                                d.bc.as<double>());
  }
  return launch_check("k_ns_bc_velocity");
}

// Presolve phi and the right-hand side and Neumann data of the phi solve
// (navier_phi_rhs, navier_solve_phi, navier_bc_pressure, add_boundary_rotrot).
int phi_stage(const mf_navier* nv, NsDom& d, cudaStream_t st) {
  const mf_navier_params_t& P = nv->prm;
  const int nw = nv->it[0], s0 = nv->it[kNt - 1], s1 = nv->it[kNt - 2], s2 = nv->it[kNt - 3];
  const double fac1 = nv->fac[0];
  const unsigned gb = ns_blocks(d.np), fb = ns_blocks(d.faces.sx + d.faces.sy + d.faces.sz);
  int rc;
  for (int c = 0; c < 3; ++c) {
    if (P.pt <= 2)
      k_ns_scale<<<gb, kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, fac1, d.F(c, nw), d.RP(c));
    else
      k_ns_phi_rhs<<<gb, kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, P.pt == 4 && nv->subite > 1 ? 5 : P.pt,
                                              d.RHS(c, nv->rhs_cur), d.RHS(c, nv->rhs_cur ^ 1), d.F(c, s0),
                                              d.F(c, s1), d.F(c, s2), d.F(c, nw), nv->fac[0], nv->fac[1],
                                              nv->fac[2], nv->fac[3], d.RP(c));
    if ((rc = launch_check("k_ns_phi_rhs"))) return rc;
  }
  {
    Sweeps S;
    for (int c = 0; c < 3; ++c) S.add(d, c, d.RP(c), d.T(4 + c));
    if ((rc = S.run(d, st)) ||
        (rc = extrapol_into(d, extrapol_of(nv, d, P.top - 1, false, kVarPhi), d.T(0), st)))
      return rc;
  }
  const int full = nv->md() ? 1 : 0;
  k_ns_fphi<<<ns_blocks(full ? d.np : d.nin), kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, nv->sigmap, d.T(0), d.T(4),
                                                                    d.T(5), d.T(6), full, d.fin.as<double>());
  k_ns_bc_phi<<<fb, kNsThreads, 0, st>>>(d.faces, d.RP(0), d.RP(1), d.RP(2), d.bc.as<double>(), fac1, d.BC(3));
  if ((rc = launch_check("k_ns_fphi"))) return rc;
  if (P.pt == 3) {
    // add_boundary_rotrot: extrapolated velocity (T7..T9), its first
    // derivatives A, B, C (T10..T12) and six second derivatives, then the
    // sums, their three sweeps and the face update
    for (int c = 0; c < 3; ++c)
      if ((rc = extrapol_into(d, extrapol_of(nv, d, P.top - 1, false, c), d.T(7 + c), st))) return rc;
    Sweeps S;
    S.add(d, 0, d.T(7), d.T(10));
    S.add(d, 1, d.T(8), d.T(11));
    S.add(d, 2, d.T(9), d.T(12));
    S.add(d, 1, d.T(7), d.T(13), 2);  // u_yy
    S.add(d, 2, d.T(7), d.T(14), 2);  // u_zz
    S.add(d, 0, d.T(8), d.T(15), 2);  // v_xx
    S.add(d, 2, d.T(8), d.T(16), 2);  // v_zz
    S.add(d, 0, d.T(9), d.T(17), 2);  // w_xx
    S.add(d, 1, d.T(9), d.T(1), 2);   // w_yy
    if ((rc = S.run(d, st))) return rc;
    k_ns_rot_sums<<<gb, kNsThreads, 0, st>>>(d.np, d.T(10), d.T(11), d.T(12), d.T(2), d.T(3), d.T(4));
    if ((rc = launch_check("k_ns_rot_sums"))) return rc;
    Sweeps S2;
    S2.add(d, 0, d.T(2), d.T(5));
    S2.add(d, 1, d.T(3), d.T(6));
    S2.add(d, 2, d.T(4), d.T(0));
    if ((rc = S2.run(d, st))) return rc;
    RotRot R{{d.T(5), d.T(6), d.T(0)}, {d.T(13), d.T(14), d.T(15), d.T(16), d.T(17), d.T(1)}};
    k_ns_bc_rotrot<<<fb, kNsThreads, 0, st>>>(d.faces, R, P.reynolds, d.BC(3));
    if ((rc = launch_check("k_ns_bc_rotrot"))) return rc;
  }
  return MF_OK;
}

// navier_projection (class_navier_3D.f90:1847-1959).
int projection(const mf_navier* nv, NsDom& d, cudaStream_t st) {
  const mf_navier_params_t& P = nv->prm;
  const int nw = nv->it[0];
  const unsigned gb = ns_blocks(d.np);
  int rc;
  k_ns_zero_edges<<<gb, kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, d.F(kVarPhi, nw));
  if ((rc = launch_check("k_ns_zero_edges"))) return rc;
  const bool add_p = P.pt == 2 || P.pt == 4;
  if (add_p && (rc = extrapol_into(d, extrapol_of(nv, d, P.top - 1, false, kVarP), d.T(0), st))) return rc;
  if (P.pt == 4)
    for (int c = 0; c < 3; ++c)
      if ((rc = extrapol_into(d, extrapol_of(nv, d, P.top - 1, false, c), d.T(7 + c), st))) return rc;
  {
    // divergence (of u*, pt <= 2; of the extrapolated velocity, pt = 4) and
    // gradient of phi: up to six sweeps in one launch
    Sweeps S;
    if (P.pt <= 2)
      for (int c = 0; c < 3; ++c) S.add(d, c, d.F(c, nw), d.T(1 + c));
    else if (P.pt == 4)
      for (int c = 0; c < 3; ++c) S.add(d, c, d.T(7 + c), d.T(1 + c));
    for (int c = 0; c < 3; ++c) S.add(d, c, d.F(kVarPhi, nw), d.T(4 + c));
    if ((rc = S.run(d, st))) return rc;
  }
  const bool div = P.pt != 3;
  k_ns_pressure<<<gb, kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, d.F(kVarPhi, nw), add_p ? d.T(0) : nullptr,
                                           div ? d.T(1) : nullptr, div ? d.T(2) : nullptr, div ? d.T(3) : nullptr,
                                           P.reynolds, d.F(kVarP, nw));
  if ((rc = launch_check("k_ns_pressure"))) return rc;
  for (int c = 0; c < 3; ++c) {
    k_ns_velocity<<<gb, kNsThreads, 0, st>>>(d.nx, d.ny, d.nz, d.RP(c), d.T(4 + c), nv->fac[0], d.F(c, nw));
    if ((rc = launch_check("k_ns_velocity"))) return rc;
  }
  return MF_OK;
}

// One pass of the step (navier3d.f90:63-102) over all subdomains.
int ns_step(mf_navier* nv, cudaStream_t st) {
  const mf_navier_params_t& P = nv->prm;
  const int nw = nv->it[0];
  const int ndom = (int)nv->dom.size();
  int rc;
  // nonlinear terms of the slots that extrapol('v') reads
  int slots[3];
  const int nslots = extrapol_slots(nv, P.tou, slots);
  for (int t = 0; t < nslots; ++t)
    if (!nv->nl_ok[slots[t]]) {
      for (NsDom& d : nv->dom)
        if ((rc = nonlinear_slot(nv, d, slots[t], st))) return rc;
      nv->nl_ok[slots[t]] = true;
    }
  // flow-rate term of f for u: integral of extrapol(u) over all subdomains
  const double* g = nullptr;
  if (P.flow_rate) {
    double* ds = nv->dsum.as<double>();
    for (int q = 0; q < ndom; ++q) {
      NsDom& d = nv->dom[q];
      if ((rc = extrapol_into(d, extrapol_of(nv, d, P.tou, false, kVarU), d.T(0), st)) ||
          (rc = wsum(d, d.T(0), ds + q, st)))
        return rc;
    }
    k_ns_sum_small<<<1, 1, 0, st>>>(ds, ndom, ds + ndom);
    k_ns_flow<<<1, 1, 0, st>>>(ds + ndom, nv->reft, nv->fac[0], (double)1e-10f, nv->state.as<double>());
    if ((rc = launch_check("k_ns_flow"))) return rc;
    g = nv->state.as<double>();
  }
  nv->rhs_cur ^= 1;  // rhs(2) = rhs(1): the other buffer keeps the previous step's
  for (NsDom& d : nv->dom)
    if ((rc = presolve(nv, d, g, st)) || (rc = velocity_bc(nv, d, st))) return rc;
  // pt = 1, 2: velocity before the pressure (pt = 2: + gradient of extrapol(p))
  if (P.pt == 2)
    for (NsDom& d : nv->dom)
      if ((rc = extrapol_into(d, extrapol_of(nv, d, P.top - 1, false, kVarP), d.T(0), st)) ||
          (rc = gradient(d, d.T(0), d.T(1), d.T(2), d.T(3), st)))
        return rc;
  if (P.pt <= 2 && (rc = velocity_solves(nv, P.pt == 2, st))) return rc;
  // pressure increment
  for (NsDom& d : nv->dom)
    if ((rc = phi_stage(nv, d, st))) return rc;
  if (nv->md()) {
    if ((rc = solve_md(nv, nv->mdp, kVarPhi, 3, nw, st))) return rc;
  } else {
    NsDom& d = nv->dom[0];
    if ((rc = solve_one(nv, d, d.sc[3], d.fin.as<double>(), nv->sigmap, d.F(kVarPhi, nw), 3, st))) return rc;
  }
  for (NsDom& d : nv->dom)
    if ((rc = projection(nv, d, st))) return rc;
  // pt = 3, 4: velocity correction with the gradient of the new pressure
  if (P.pt >= 3) {
    for (NsDom& d : nv->dom)
      if ((rc = gradient(d, d.F(kVarP, nw), d.T(1), d.T(2), d.T(3), st))) return rc;
    if ((rc = velocity_solves(nv, true, st))) return rc;
  }
  nv->nl_ok[nw] = false;
  return MF_OK;
}

}  // namespace

namespace {

// Weighted sums of one k_ns_diag phase over all subdomains (each subdomain's
// sums in a fixed order, then added in subdomain order) into out[kDiagSums]
// on the host; synchronises.
int diag_sums(mf_navier* nv, int phase, const std::vector<DiagIn>& Ds, double* out, cudaStream_t st) {
  for (int s = 0; s < kDiagSums; ++s) out[s] = 0.0;
  for (size_t q = 0; q < nv->dom.size(); ++q) {
    NsDom& d = nv->dom[q];
    const DiagIn& D = Ds[q];
    const int groups = (d.ny + kWRows - 1) / kWRows, count = d.nz * groups;
    const dim3 grid(d.nz, groups);
    double* part = d.part.as<double>();
    switch (phase) {
      case 0: k_ns_diag<0><<<grid, kNsThreads, 0, st>>>(d.weights(), D, part); break;
      case 1: k_ns_diag<1><<<grid, kNsThreads, 0, st>>>(d.weights(), D, part); break;
      case 2: k_ns_diag<2><<<grid, kNsThreads, 0, st>>>(d.weights(), D, part); break;
      case 3: k_ns_diag<3><<<grid, kNsThreads, 0, st>>>(d.weights(), D, part); break;
      default: k_ns_diag<4><<<grid, kNsThreads, 0, st>>>(d.weights(), D, part); break;
    }
    k_ns_sum_parts<<<1, kNsThreads, 0, st>>>(part, count, kDiagSums, d.sums.as<double>());
    int r = launch_check("k_ns_diag");
    if (r) return r;
    double h[kDiagSums];
    MF_CUDA(cudaMemcpyAsync(h, d.sums.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
    MF_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < kDiagSums; ++s) out[s] += h[s];
  }
  return MF_OK;
}

// testconv (navier3d.f90:366-412) of the iterate it(1) against the last
// sub-iterate: true when both relative changes are below eps.
int ns_testconv(mf_navier* nv, double eps, bool* test, cudaStream_t st) {
  const int nw = nv->it[0];
  std::vector<DiagIn> Ds(nv->dom.size());
  for (size_t q = 0; q < nv->dom.size(); ++q) {
    NsDom& d = nv->dom[q];
    DiagIn& D = Ds[q];
    D = DiagIn{};
    D.u = d.F(0, nw); D.v = d.F(1, nw); D.w = d.F(2, nw); D.p = d.F(kVarP, nw);
    const double* sb = d.sub.as<double>();
    D.su = sb; D.sv = sb + d.np; D.sw = sb + 2 * d.np; D.sp = sb + 3 * d.np;
  }
  double a[kDiagSums], b[kDiagSums];
  int rc;
  if ((rc = diag_sums(nv, 3, Ds, a, st))) return rc;
  const double e1 = std::sqrt(a[1]) / std::sqrt(a[0]);
  for (DiagIn& D : Ds) D.spm = a[2] / nv->reft;
  if ((rc = diag_sums(nv, 4, Ds, b, st))) return rc;
  const double e2 = std::sqrt(b[1]) / std::sqrt(b[0]);
  *test = e1 < eps && e2 < eps;
  return MF_OK;
}

// Driver diagnostics of level it(nt) (navier3d.f90:120-254) over all
// subdomains; diag[12].
int ns_diagnostics(mf_navier* nv, double* diag, cudaStream_t st) {
  const int cur = nv->it[kNt - 1], prev = nv->it[kNt - 2];
  int rc;
  std::vector<DiagIn> Ds(nv->dom.size());
  for (size_t q = 0; q < nv->dom.size(); ++q) {
    NsDom& d = nv->dom[q];
    Sweeps S;
    for (int c = 0; c < 3; ++c) S.add(d, c, d.F(c, cur), d.T(1 + c));
    if ((rc = S.run(d, st))) return rc;
    DiagIn& D = Ds[q];
    D = DiagIn{};
    D.u = d.F(0, cur); D.v = d.F(1, cur); D.w = d.F(2, cur); D.p = d.F(kVarP, cur);
    D.up = d.F(0, prev); D.vp = d.F(1, prev); D.wp = d.F(2, prev); D.pp = d.F(kVarP, prev);
    D.dx = d.T(1); D.dy = d.T(2); D.dz = d.T(3);
    D.ue = d.EX(0); D.ve = d.EX(1); D.pex = d.EX(2);
  }
  double s0[kDiagSums], s1[kDiagSums], s2[kDiagSums];
  if ((rc = diag_sums(nv, 0, Ds, s0, st))) return rc;
  const double reft = nv->reft, ts = nv->prm.ts;
  const double ref1 = std::sqrt(reft);  // norme(1)
  diag[0] = std::sqrt(s0[0]) / ref1;
  const double refv = std::sqrt(s0[1]), errv = std::sqrt(s0[2]);
  nv->err_vts += errv * errv * ts;
  diag[1] = errv;
  diag[2] = errv / refv;
  diag[3] = std::sqrt(nv->err_vts);
  // pressure: remove the weighted mean of p(it(nt)) (the driver stores it back)
  for (NsDom& d : nv->dom) {
    k_ns_shift<<<ns_blocks(d.np), kNsThreads, 0, st>>>(d.np, -(s0[3] / reft), d.F(kVarP, cur));
    if ((rc = launch_check("k_ns_shift"))) return rc;
  }
  for (DiagIn& D : Ds) D.pexm = s0[10] / reft;
  if ((rc = diag_sums(nv, 1, Ds, s1, st))) return rc;
  const double errp = std::sqrt(s1[0]), refp = std::sqrt(s1[1]);
  nv->err_pre += errp * errp * ts;
  diag[4] = errp;
  diag[5] = errp / refp;
  diag[6] = std::sqrt(nv->err_pre);
  const double nu = std::sqrt(s0[4]), nvv = std::sqrt(s0[5]), nww = std::sqrt(s0[6]);
  diag[7] = 0.5 * (nu * nu + nvv * nvv + nww) / reft;
  for (DiagIn& D : Ds) D.auxm = s1[2] / reft;
  if ((rc = diag_sums(nv, 2, Ds, s2, st))) return rc;
  const double sp = std::sqrt(s2[0]);
  diag[8] = sp;
  diag[9] = sp / reft;
  const double du = std::sqrt(s0[7]), dv = std::sqrt(s0[8]), dw = std::sqrt(s0[9]);
  const double sv = std::sqrt(du * du + dv * dv + dw);
  diag[10] = sv;
  diag[11] = sv / reft;
  return MF_OK;
}

// Set-up of one subdomain's coefficients, buffers and exact solution.
int dom_setup(NsDom& d, const mf_navier_params_t* p, const double* gx, int nx, const double* gy, int ny,
              const double* gz, int nz, bool md) {
  d.nx = nx; d.ny = ny; d.nz = nz;
  d.n1 = nx - 2; d.n2 = ny - 2; d.n3 = nz - 2;
  d.np = (long long)nx * ny * nz;
  d.nin = (long long)d.n1 * d.n2 * d.n3;
  d.faces = Faces{nx, ny, nz, 2LL * d.n2 * d.n3, 2LL * d.n1 * d.n3, 2LL * d.n1 * d.n2};
  const long long ftot = d.faces.sx + d.faces.sy + d.faces.sz;
  const int groups = (ny + kWRows - 1) / kWRows;
  const size_t fb = (size_t)d.np * sizeof(double);
  const int bctu[6] = {1, 1, 1, 1, 1, 1}, bctp[6] = {2, 2, 2, 2, 2, 2};
  int rc;
  if ((rc = mf_der_coeffs_init(gx, nx, 1, p->so_der, &d.dcx)) || (rc = mf_der_coeffs_init(gy, ny, 1, p->so_der, &d.dcy)) ||
      (rc = mf_der_coeffs_init(gz, nz, 1, p->so_der, &d.dcz)))
    return rc;
  if (!md)
    for (int q = 0; q < 4; ++q)
      if ((rc = mf_solver_coeffs_init_3d(gx, gy, gz, nx, ny, nz, q < 3 ? bctu : bctp, p->so_solver, &d.sc[q])))
        return rc;
  if (p->les_type != 0 && ((rc = mf_les_create(gx, nx, gy, ny, gz, nz, &d.les)) || (rc = d.nu.ensure(fb))))
    return rc;
  if (p->nsubite > 1 && (rc = d.sub.ensure(fb * 4))) return rc;
  if ((rc = d.fields.ensure(fb * 5 * kNt)) || (rc = d.nl.ensure(fb * 3 * kNt)) || (rc = d.rhs.ensure(fb * 6)) ||
      (rc = d.rp.ensure(fb * 3)) || (rc = d.tmp.ensure(fb * 18)) ||
      (rc = d.fin.ensure(md ? 3 * fb : (size_t)d.nin * sizeof(double) * 3)) || (rc = d.exact.ensure(fb * 5)) ||
      (rc = d.bcex.ensure(sizeof(double) * 3 * ftot)) || (rc = d.bc.ensure(sizeof(double) * 4 * ftot)) ||
      (rc = d.grid.ensure(sizeof(double) * (nx + ny + nz))) || (rc = d.wts.ensure(sizeof(double) * (nx + ny + nz))) ||
      (rc = d.part.ensure(sizeof(double) * kDiagSums * (size_t)nz * groups)) ||
      (rc = d.sums.ensure(sizeof(double) * kDiagSums)))
    return rc;
  // host-side set-up: grids, half widths, integrale(1) of this subdomain
  std::vector<double> g(nx + ny + nz), w(nx + ny + nz);
  const double* src[3] = {gx, gy, gz};
  const int n[3] = {nx, ny, nz};
  for (int a = 0, off = 0; a < 3; off += n[a], ++a) {
    for (int i = 0; i < n[a]; ++i) g[off + i] = src[a][i];
    for (int i = 1; i < n[a] - 1; ++i) w[off + i] = (src[a][i + 1] - src[a][i - 1]) * 0.5;
    w[off] = (src[a][1] - src[a][0]) * 0.5;
    w[off + n[a] - 1] = (src[a][n[a] - 1] - src[a][n[a] - 2]) * 0.5;
  }
  double reft = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int b = (i == 0 || i == nx - 1) + (j == 0 || j == ny - 1) + (k == 0 || k == nz - 1);
        if (b <= 1) reft += w[i] * w[nx + j] * w[nx + ny + k];
      }
  d.reft = reft;
  if (cudaMemcpy(d.grid.ptr, g.data(), g.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d.wts.ptr, w.data(), w.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(d.fields.ptr, 0, fb * 5 * kNt) != cudaSuccess || cudaMemset(d.rhs.ptr, 0, fb * 6) != cudaSuccess)
    return set_error(MF_ERR_CUDA, "mf_navier_create: upload failed");
  const double* dg = d.grid.as<double>();
  k_ns_exact<<<ns_blocks(d.np), kNsThreads>>>(dg, dg + nx, dg + nx + ny, nx, ny, nz, p->nmodes, 4.0 * std::atan(1.0),
                                              p->reynolds, d.exact.as<double>());
  k_ns_bc_exact<<<ns_blocks(ftot), kNsThreads>>>(d.faces, d.exact.as<double>(), d.np, d.bcex.as<double>());
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
    return set_error(MF_ERR_CUDA, "mf_navier_create: exact-solution kernels failed");
  return MF_OK;
}

int navier_check_params(const mf_navier_params_t* p) {
  if (!(p->ts > 0.0) || !(p->reynolds > 0.0) || p->nlt < 0 || p->nlt > 2 || p->pt < 1 || p->pt > 4 ||
      p->tou < 1 || p->tou > 3 || p->nmodes < 0 || p->les_type < 0 || p->les_type > MF_LES_LEARNED || p->nsubite < 1)
    return set_error(MF_ERR_ARG,
                     "mf_navier_create: bad parameters (ts, reynolds > 0; nlt 0..2; pt 1..4; tou 1..3; les_type 0..4)");
  if (p->precision != MF_PREC_FP64 && p->precision != MF_PREC_SPLIT_BF16 && p->precision != MF_PREC_3XTF32)
    return set_error(MF_ERR_ARG, "mf_navier_create: unknown precision %d", p->precision);
  return MF_OK;
}

int navier_build(const int nd[3], const int periods[3], const double* const* gx, const int* nx,
                 const double* const* gy, const int* ny, const double* const* gz, const int* nz,
                 const mf_navier_params_t* p, mf_navier_t** out) {
  *out = nullptr;
  int rc;
  if ((rc = navier_check_params(p))) return rc;
  for (int l = 0; l < 3; ++l)
    if (nd[l] < 1) return set_error(MF_ERR_ARG, "mf_navier_create: at least one subdomain per axis");
  const int* sizes[3] = {nx, ny, nz};
  for (int l = 0; l < 3; ++l)
    for (int q = 0; q < nd[l]; ++q)
      if (sizes[l][q] < 9) return set_error(MF_ERR_ARG, "mf_navier_create: at least 9 nodes per axis");
  const bool md = nd[0] * nd[1] * nd[2] > 1 || periods[0] || periods[1] || periods[2];
  mf_navier* nv = new mf_navier();
  nv->prm = *p;
  for (int l = 0; l < 3; ++l) nv->nd[l] = nd[l];
  const double ts = p->ts;
  if (p->tou == 1) {
    nv->fac[0] = 1.0 / ts; nv->fac[1] = -1.0 / ts; nv->fac[2] = 0.0; nv->fac[3] = 0.0;
  } else if (p->tou == 2) {
    nv->fac[0] = 1.5 / ts; nv->fac[1] = -2.0 / ts; nv->fac[2] = 0.5 / ts; nv->fac[3] = 0.0;
  } else {
    nv->fac[0] = 11.0 / (6.0 * ts); nv->fac[1] = -18.0 / (6.0 * ts);
    nv->fac[2] = 9.0 / (6.0 * ts); nv->fac[3] = -2.0 / (6.0 * ts);
  }
  nv->sigmau = -p->reynolds * nv->fac[0];
  nv->sigmap = 0.0;
  auto fail = [&](int r) {
    mf_navier_destroy(nv);
    return r;
  };
  nv->dom.resize((size_t)nd[0] * nd[1] * nd[2]);
  for (int k = 0; k < nd[2]; ++k)
    for (int j = 0; j < nd[1]; ++j)
      for (int i = 0; i < nd[0]; ++i) {
        NsDom& d = nv->dom[i + nd[0] * (j + nd[1] * k)];
        if ((rc = dom_setup(d, p, gx[i], nx[i], gy[j], ny[j], gz[k], nz[k], md))) return fail(rc);
      }
  for (const NsDom& d : nv->dom) nv->reft += d.reft;
  if ((rc = nv->state.ensure(sizeof(double) * 3)) || (rc = nv->dsum.ensure(sizeof(double) * (nv->dom.size() + 1))))
    return fail(rc);
  if (cudaMemset(nv->state.ptr, 0, sizeof(double) * 3) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
    return fail(set_error(MF_ERR_CUDA, "mf_navier_create: upload failed"));
  if (md) {
    // the influence matrices of the velocity (Dirichlet outer faces, sigmau)
    // and of the pressure (Neumann, sigma 0, constant null space)
    const int bctu[6] = {1, 1, 1, 1, 1, 1}, bctp[6] = {2, 2, 2, 2, 2, 2};
    if ((rc = mf_md_create(nd, periods, gx, nx, gy, ny, gz, nz, bctu, p->so_solver, &nv->mdu)) ||
        (rc = mf_md_create(nd, periods, gx, nx, gy, ny, gz, nz, bctp, p->so_solver, &nv->mdp)))
      return fail(rc);
    auto build = [&](mf_md_t* m, double sigma, int null_mode) {
      return p->md_cache_dir ? mf_md_influence_matrix_cached(m, sigma, null_mode, p->md_cache_dir, nullptr)
                             : mf_md_influence_matrix_set(m, sigma, null_mode, nullptr);
    };
    for (mf_md_t* m : {nv->mdu, nv->mdp})
      if ((rc = mf_md_set_interface_solve(m, p->md_interface)) ||
          (rc = mf_md_set_precision(m, p->precision, p->refine)))
        return fail(rc);
    if ((rc = build(nv->mdu, nv->sigmau, 0)) || (rc = build(nv->mdp, 0.0, 1))) return fail(rc);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(set_error(MF_ERR_CUDA, "influence matrices failed"));
  } else {
    for (int q = 0; q < 2; ++q)
      if (cudaStreamCreateWithFlags(&nv->side[q], cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&nv->join[q], cudaEventDisableTiming) != cudaSuccess)
        return fail(set_error(MF_ERR_CUDA, "mf_navier_create: stream set-up failed"));
    if (cudaEventCreateWithFlags(&nv->fork, cudaEventDisableTiming) != cudaSuccess)
      return fail(set_error(MF_ERR_CUDA, "mf_navier_create: stream set-up failed"));
  }
  *out = nv;
  return MF_OK;
}

int dom_field(mf_navier* nv, int sub, int var, int level, double** ptr, NsDom** dp) {
  if (!nv || !ptr || sub < 0 || sub >= (int)nv->dom.size() || var < 0 || var > 4 || level < 0 || level >= kNt)
    return set_error(MF_ERR_ARG, "mf_navier field access: subdomain, var 0..4, level 0..3");
  NsDom& d = nv->dom[sub];
  *ptr = d.F(var, nv->it[level]);
  if (dp) *dp = &d;
  return MF_OK;
}

}  // namespace

extern "C" {

int mf_navier_defaults(mf_navier_params_t* p) {
  if (!p) return set_error(MF_ERR_ARG, "mf_navier_defaults: null argument");
  p->ts = 1.0;
  p->reynolds = 1.0;
  p->nlt = 2;
  p->pt = 1;
  p->tou = 2;
  p->top = 2;
  p->so_solver = 6;
  p->so_der = 6;
  p->flow_rate = 1;
  p->nmodes = 5;
  p->precision = MF_PREC_FP64;
  p->refine = -1;
  p->les_type = 0;
  p->les_c = 0.0;
  p->nsubite = 1;
  p->md_cache_dir = nullptr;
  p->md_interface = MF_MD_IFACE_AUTO;
  return MF_OK;
}

int mf_navier_destroy(mf_navier_t* nv) {
  if (!nv) return MF_OK;
  for (NsDom& d : nv->dom) d.release();
  mf_md_destroy(nv->mdu);
  mf_md_destroy(nv->mdp);
  for (int q = 0; q < 2; ++q) {
    if (nv->side[q]) cudaStreamDestroy(nv->side[q]);
    if (nv->join[q]) cudaEventDestroy(nv->join[q]);
  }
  if (nv->fork) cudaEventDestroy(nv->fork);
  nv->state.release();
  nv->dsum.release();
  delete nv;
  return MF_OK;
}

int mf_navier_create(const double* gx, int nx, const double* gy, int ny, const double* gz, int nz,
                     const mf_navier_params_t* p, mf_navier_t** out) {
  if (!gx || !gy || !gz || !p || !out) return set_error(MF_ERR_ARG, "mf_navier_create: null argument");
  const int nd[3] = {1, 1, 1}, periods[3] = {0, 0, 0};
  return navier_build(nd, periods, &gx, &nx, &gy, &ny, &gz, &nz, p, out);
}

int mf_navier_create_md(const int nd[3], const int periods[3], const double* const* gridx, const int* nx,
                        const double* const* gridy, const int* ny, const double* const* gridz, const int* nz,
                        const mf_navier_params_t* p, mf_navier_t** out) {
  if (!nd || !periods || !gridx || !nx || !gridy || !ny || !gridz || !nz || !p || !out)
    return set_error(MF_ERR_ARG, "mf_navier_create_md: null argument");
  return navier_build(nd, periods, gridx, nx, gridy, ny, gridz, nz, p, out);
}

int mf_navier_subdomains(const mf_navier_t* nv, int* count) {
  if (!nv || !count) return set_error(MF_ERR_ARG, "mf_navier_subdomains: null argument");
  *count = (int)nv->dom.size();
  return MF_OK;
}

int mf_navier_sub_field(mf_navier_t* nv, int sub, int var, int level, double** ptr) {
  return dom_field(nv, sub, var, level, ptr, nullptr);
}

int mf_navier_field(mf_navier_t* nv, int var, int level, double** ptr) {
  return dom_field(nv, 0, var, level, ptr, nullptr);
}

int mf_navier_sub_set_field(mf_navier_t* nv, int sub, int var, int level, const double* f, void* stream) {
  double* d = nullptr;
  NsDom* dm = nullptr;
  int rc = dom_field(nv, sub, var, level, &d, &dm);
  if (rc) return rc;
  if (!f) return set_error(MF_ERR_ARG, "mf_navier_set_field: null field");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MF_CUDA(cudaMemcpyAsync(d, f, (size_t)dm->np * 8, cudaMemcpyDefault, st));
  if (!is_device_ptr(f)) MF_CUDA(cudaStreamSynchronize(st));
  if (var < 3) nv->nl_ok[nv->it[level]] = false;
  return MF_OK;
}

int mf_navier_set_field(mf_navier_t* nv, int var, int level, const double* f, void* stream) {
  return mf_navier_sub_set_field(nv, 0, var, level, f, stream);
}

int mf_navier_sub_get_field(mf_navier_t* nv, int sub, int var, int level, double* f, void* stream) {
  double* d = nullptr;
  NsDom* dm = nullptr;
  int rc = dom_field(nv, sub, var, level, &d, &dm);
  if (rc) return rc;
  if (!f) return set_error(MF_ERR_ARG, "mf_navier_get_field: null field");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MF_CUDA(cudaMemcpyAsync(f, d, (size_t)dm->np * 8, cudaMemcpyDefault, st));
  if (!is_device_ptr(f)) MF_CUDA(cudaStreamSynchronize(st));
  return MF_OK;
}

int mf_navier_get_field(mf_navier_t* nv, int var, int level, double* f, void* stream) {
  return mf_navier_sub_get_field(nv, 0, var, level, f, stream);
}

int mf_navier_step(mf_navier_t* nv, double* diag, void* stream) {
  if (!nv) return set_error(MF_ERR_ARG, "mf_navier_step: null handle");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = MF_OK;
  nv->time += nv->prm.ts;  // navier_time
  for (int subite = 1; subite <= nv->prm.nsubite; ++subite) {
    nv->subite = subite;
    nv->subiterations = subite;
    if ((rc = ns_step(nv, st))) break;
    bool test = false;
    if (subite > 1 && (rc = ns_testconv(nv, 1e-9, &test, st))) break;
    if (nv->prm.nsubite > 1) {
      const int nw = nv->it[0];
      for (NsDom& d : nv->dom) {
        for (int v = 0; v < 4 && !rc; ++v)
          if (cudaMemcpyAsync(d.sub.as<double>() + (size_t)v * d.np, d.F(v, nw), (size_t)d.np * 8,
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            rc = set_error(MF_ERR_CUDA, "mf_navier_step: copy of the sub-iterate failed");
        if (rc) break;
      }
      if (rc) break;
    }
    if (diag && (rc = ns_diagnostics(nv, diag, st))) break;
    if (test) break;
  }
  nv->subite = 1;
  if (rc) return rc;
  // slot rotation (navier3d.f90:256-261)
  const int first = nv->it[0];
  for (int i = 0; i < kNt - 1; ++i) nv->it[i] = nv->it[i + 1];
  nv->it[kNt - 1] = first;
  return MF_OK;
}

int mf_navier_subiterations(const mf_navier_t* nv, int* n) {
  if (!nv || !n) return set_error(MF_ERR_ARG, "mf_navier_subiterations: null argument");
  *n = nv->subiterations;
  return MF_OK;
}

int mf_navier_set_les_network(mf_navier_t* nv, const mf_mlp_t* mlp) {
  if (!nv) return set_error(MF_ERR_ARG, "mf_navier_set_les_network: null handle");
  if (nv->prm.les_type != MF_LES_LEARNED)
    return set_error(MF_ERR_ARG, "mf_navier_set_les_network: the step was created with les_type %d, not 4",
                     nv->prm.les_type);
  nv->les_mlp = mlp;
  return MF_OK;
}

int mf_navier_state(mf_navier_t* nv, double* time, double* debit, double* g) {
  if (!nv) return set_error(MF_ERR_ARG, "mf_navier_state: null handle");
  double s[3];
  MF_CUDA(cudaMemcpy(s, nv->state.ptr, sizeof(s), cudaMemcpyDeviceToHost));
  if (time) *time = nv->time;
  if (debit) *debit = s[1];
  if (g) *g = s[0];
  return MF_OK;
}

// Checkpoint (the role of restart_write / restart_read,
// class_navier_3D.f90:186-340, as one raw little-endian binary file instead
// of a NetCDF directory).  Layout: magic "MFNSCHK2", int32 nt, int32 number
// of subdomains, per subdomain int32 nx, ny, nz and its three grids (FP64),
// time, int32 it(1..nt) (0-based slots), int32 rhs_cur, err_vts, err_pre,
// the flow-rate state {g, debit, initialised}, then per subdomain the fields
// u, v, w, p, phi of each slot 0..nt-1 and rhs(1), rhs(2) of u, v, w (FP64,
// x fastest).  Beyond the reference's restart it keeps the right-hand-side
// history (read by pt 4) and the flow-rate state (saved variables of f), so
// a resumed run continues bit-identically.  The nonlinear terms are
// recomputed after a load.
constexpr char kChkMagic[8] = {'M', 'F', 'N', 'S', 'C', 'H', 'K', '2'};

int mf_navier_save(mf_navier_t* nv, const char* path, void* stream) {
  if (!nv || !path) return set_error(MF_ERR_ARG, "mf_navier_save: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MF_CUDA(cudaStreamSynchronize(st));
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(MF_ERR_ARG, "mf_navier_save: cannot open %s", path);
  double flow[3];
  bool ok = cudaMemcpy(flow, nv->state.ptr, sizeof(flow), cudaMemcpyDeviceToHost) == cudaSuccess;
  const int head[2] = {kNt, (int)nv->dom.size()};
  ok = ok && std::fwrite(kChkMagic, 1, 8, f) == 8 && std::fwrite(head, 4, 2, f) == 2;
  for (const NsDom& d : nv->dom) {
    std::vector<double> grid(d.nx + d.ny + d.nz);
    const int dims[3] = {d.nx, d.ny, d.nz};
    ok = ok && cudaMemcpy(grid.data(), d.grid.ptr, grid.size() * 8, cudaMemcpyDeviceToHost) == cudaSuccess &&
         std::fwrite(dims, 4, 3, f) == 3 && std::fwrite(grid.data(), 8, grid.size(), f) == grid.size();
  }
  ok = ok && std::fwrite(&nv->time, 8, 1, f) == 1 && std::fwrite(nv->it, 4, kNt, f) == (size_t)kNt &&
       std::fwrite(&nv->rhs_cur, 4, 1, f) == 1 && std::fwrite(&nv->err_vts, 8, 1, f) == 1 &&
       std::fwrite(&nv->err_pre, 8, 1, f) == 1 && std::fwrite(flow, 8, 3, f) == 3;
  for (const NsDom& d : nv->dom) {
    std::vector<double> buf(d.np);
    auto put = [&](const double* src) {
      return ok = ok && cudaMemcpy(buf.data(), src, buf.size() * 8, cudaMemcpyDeviceToHost) == cudaSuccess &&
                  std::fwrite(buf.data(), 8, buf.size(), f) == buf.size();
    };
    for (int slot = 0; slot < kNt && ok; ++slot)
      for (int v = 0; v < 5 && ok; ++v) put(d.F(v, slot));
    for (int c = 0; c < 3 && ok; ++c)
      for (int w = 0; w < 2 && ok; ++w) put(d.RHS(c, w));
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MF_OK : set_error(MF_ERR_CUDA, "mf_navier_save: writing %s failed", path);
}

int mf_navier_load(mf_navier_t* nv, const char* path, void* stream) {
  if (!nv || !path) return set_error(MF_ERR_ARG, "mf_navier_load: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MF_CUDA(cudaStreamSynchronize(st));
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(MF_ERR_ARG, "mf_navier_load: cannot open %s", path);
  char magic[8];
  int head[2];
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kChkMagic, 8) == 0 &&
            std::fread(head, 4, 2, f) == 2 && head[0] == kNt && head[1] == (int)nv->dom.size();
  for (size_t q = 0; ok && q < nv->dom.size(); ++q) {
    const NsDom& d = nv->dom[q];
    int dims[3];
    std::vector<double> grid(d.nx + d.ny + d.nz), mine(grid.size());
    ok = std::fread(dims, 4, 3, f) == 3 && dims[0] == d.nx && dims[1] == d.ny && dims[2] == d.nz &&
         std::fread(grid.data(), 8, grid.size(), f) == grid.size() &&
         cudaMemcpy(mine.data(), d.grid.ptr, mine.size() * 8, cudaMemcpyDeviceToHost) == cudaSuccess &&
         std::memcmp(grid.data(), mine.data(), grid.size() * 8) == 0;
  }
  if (!ok) {
    std::fclose(f);
    return set_error(MF_ERR_ARG, "mf_navier_load: %s is not a checkpoint of these grids", path);
  }
  double time, evts, epre, flow[3];
  int it[kNt], rhs_cur;
  ok = std::fread(&time, 8, 1, f) == 1 && std::fread(it, 4, kNt, f) == (size_t)kNt &&
       std::fread(&rhs_cur, 4, 1, f) == 1 && std::fread(&evts, 8, 1, f) == 1 && std::fread(&epre, 8, 1, f) == 1 &&
       std::fread(flow, 8, 3, f) == 3;
  int seen = 0;
  for (int i = 0; i < kNt && ok; ++i) {
    ok = it[i] >= 0 && it[i] < kNt && !(seen & (1 << it[i]));
    seen |= 1 << (ok ? it[i] : 0);
  }
  ok = ok && (rhs_cur == 0 || rhs_cur == 1);
  // every field is read and the file checked to its end before anything is
  // uploaded: a truncated or inconsistent file leaves the running state as
  // it was
  const int per_dom = kNt * 5 + 6;
  std::vector<std::vector<double>> fields;
  for (size_t q = 0; q < nv->dom.size() && ok; ++q)
    for (int k = 0; k < per_dom && ok; ++k) {
      fields.emplace_back(nv->dom[q].np);
      ok = std::fread(fields.back().data(), 8, fields.back().size(), f) == fields.back().size();
    }
  ok = ok && std::fgetc(f) == EOF;
  std::fclose(f);
  if (!ok) return set_error(MF_ERR_ARG, "mf_navier_load: %s is truncated or inconsistent", path);
  size_t idx = 0;
  for (NsDom& d : nv->dom) {
    auto put = [&](double* dst) {
      const std::vector<double>& b = fields[idx++];
      ok = ok && cudaMemcpy(dst, b.data(), b.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    for (int slot = 0; slot < kNt; ++slot)
      for (int v = 0; v < 5; ++v) put(d.F(v, slot));
    for (int c = 0; c < 3; ++c)
      for (int w = 0; w < 2; ++w) put(d.RHS(c, w));
  }
  ok = ok && cudaMemcpy(nv->state.ptr, flow, sizeof(flow), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaDeviceSynchronize() == cudaSuccess;
  if (!ok) return set_error(MF_ERR_CUDA, "mf_navier_load: upload of %s failed", path);
  nv->time = time;
  for (int i = 0; i < kNt; ++i) nv->it[i] = it[i];
  nv->rhs_cur = rhs_cur;
  nv->err_vts = evts;
  nv->err_pre = epre;
  for (int i = 0; i < kNt; ++i) nv->nl_ok[i] = false;
  return MF_OK;
}

}  // extern "C"
