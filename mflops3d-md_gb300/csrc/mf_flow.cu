// Fine-grid flow for the learned LES coefficient's training data (no
// reference counterpart).  A decaying flow in a closed no-slip box, advanced
// by an explicit Runge-Kutta method with a pressure projection after every
// stage; the derivatives are the compact sweeps of mf_der.cu and
// the projection is a Neumann Poisson solve of mf_solver.cu, so the pairs
// are generated by the same operators as the rest of the path.  The kernels
// here are the pointwise parts of one stage (all FP64):
//   k_flow_stage       out_i = a w_i + b (u_i + dt (-u_j d_j u_i + nu d_jj u_i)),
//                      zero on the walls
//   k_flow_divergence  interior Poisson right-hand side  scale * d_j u_j
//   k_flow_correct     u_i -= dt d_i phi in the interior, zero on the walls
//   k_flow_products    u_i u_j (six fields) for the filtered stresses
//   k_flow_curl        u_i = eps_ijk d_j psi_k (initial condition)
#include "mf_internal.h"

namespace mf {

struct Vec3 {
  const double* c[3];
};
struct Vec3Out {
  double* c[3];
};
struct Out6 {
  double* c[6];
};
struct Grad9 {
  const double* g[9];  // g[3*i + j] = d_j of component i
};

__device__ __forceinline__ bool on_wall(long long idx, int nx, int ny, int nz) {
  const int i = (int)(idx % nx);
  const long long jk = idx / nx;
  const int j = (int)(jk % ny), k = (int)(jk / ny);
  return i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
}

__global__ void k_flow_stage(int nx, int ny, int nz, double nu, double dt, double a, double b, Vec3 u, Vec3 w,
                             Grad9 du, Grad9 ddu, Vec3Out out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  if (on_wall(idx, nx, ny, nz)) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out.c[i][idx] = 0.0;
    return;
  }
  const double u0 = u.c[0][idx], u1 = u.c[1][idx], u2 = u.c[2][idx];
  double r[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double adv = u0 * du.g[3 * i][idx] + u1 * du.g[3 * i + 1][idx] + u2 * du.g[3 * i + 2][idx];
    const double lap = ddu.g[3 * i][idx] + ddu.g[3 * i + 1][idx] + ddu.g[3 * i + 2][idx];
    r[i] = u.c[i][idx] + dt * (nu * lap - adv);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) out.c[i][idx] = (a != 0.0 ? a * w.c[i][idx] : 0.0) + b * r[i];
}

__global__ void k_flow_divergence(int nx, int ny, int nz, double scale, const double* __restrict__ dx,
                                  const double* __restrict__ dy, const double* __restrict__ dz,
                                  double* __restrict__ rhs) {
  const int n1 = nx - 2, n2 = ny - 2, n3 = nz - 2;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)n1 * n2 * n3) return;
  const int i = (int)(q % n1);
  const long long jk = q / n1;
  const int j = (int)(jk % n2), k = (int)(jk / n2);
  const long long idx = (i + 1) + (long long)nx * ((j + 1) + (long long)ny * (k + 1));
  rhs[q] = scale * (dx[idx] + dy[idx] + dz[idx]);
}

__global__ void k_flow_correct(int nx, int ny, int nz, double dt, Vec3Out u, Vec3 dphi) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const bool wall = on_wall(idx, nx, ny, nz);
#pragma unroll
  for (int i = 0; i < 3; ++i) u.c[i][idx] = wall ? 0.0 : u.c[i][idx] - dt * dphi.c[i][idx];
}

__global__ void k_flow_products(long long tot, Vec3 u, Out6 uu) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= tot) return;
  const double a = u.c[0][idx], b = u.c[1][idx], c = u.c[2][idx];
  uu.c[0][idx] = a * a;
  uu.c[1][idx] = a * b;
  uu.c[2][idx] = a * c;
  uu.c[3][idx] = b * b;
  uu.c[4][idx] = b * c;
  uu.c[5][idx] = c * c;
}

__global__ void k_flow_curl(int nx, int ny, int nz, Grad9 dpsi, Vec3Out u) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const bool wall = on_wall(idx, nx, ny, nz);
  // u_0 = d_1 psi_2 - d_2 psi_1, u_1 = d_2 psi_0 - d_0 psi_2, u_2 = d_0 psi_1 - d_1 psi_0
  const double c0 = dpsi.g[3 * 2 + 1][idx] - dpsi.g[3 * 1 + 2][idx];
  const double c1 = dpsi.g[3 * 0 + 2][idx] - dpsi.g[3 * 2 + 0][idx];
  const double c2 = dpsi.g[3 * 1 + 0][idx] - dpsi.g[3 * 0 + 1][idx];
  u.c[0][idx] = wall ? 0.0 : c0;
  u.c[1][idx] = wall ? 0.0 : c1;
  u.c[2][idx] = wall ? 0.0 : c2;
}

static inline unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

static bool all_dev(const double* const* p, int n) {
  if (!p) return false;
  for (int q = 0; q < n; ++q)
    if (!p[q] || !is_device_ptr(p[q])) return false;
  return true;
}

static bool all_dev(double* const* p, int n) { return all_dev(const_cast<const double* const*>(p), n); }

}  // namespace mf

using namespace mf;

extern "C" {

int mf_flow_stage(int nx, int ny, int nz, double nu, double dt, double a, double b, const double* const* u,
                  const double* const* w, const double* const* du, const double* const* ddu, double* const* out,
                  void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !all_dev(u, 3) || !all_dev(du, 9) || !all_dev(ddu, 9) || !all_dev(out, 3) ||
      (a != 0.0 && !all_dev(w, 3)))
    return set_error(MF_ERR_ARG, "mf_flow_stage: bad arguments");
  Vec3 U, W{};
  Vec3Out O;
  Grad9 D, DD;
  for (int i = 0; i < 3; ++i) {
    U.c[i] = u[i];
    W.c[i] = a != 0.0 ? w[i] : nullptr;
    O.c[i] = out[i];
  }
  for (int q = 0; q < 9; ++q) {
    D.g[q] = du[q];
    DD.g[q] = ddu[q];
  }
  const long long tot = (long long)nx * ny * nz;
  k_flow_stage<<<nb(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, nz, nu, dt, a, b, U, W, D, DD, O);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_flow_divergence(int nx, int ny, int nz, double scale, const double* dudx, const double* dvdy,
                       const double* dwdz, double* rhs, void* stream) {
  const double* in[3] = {dudx, dvdy, dwdz};
  if (nx < 3 || ny < 3 || nz < 3 || !all_dev(in, 3) || !rhs || !is_device_ptr(rhs))
    return set_error(MF_ERR_ARG, "mf_flow_divergence: bad arguments");
  const long long tot = (long long)(nx - 2) * (ny - 2) * (nz - 2);
  k_flow_divergence<<<nb(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, nz, scale, dudx, dvdy, dwdz,
                                                                           rhs);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_flow_correct(int nx, int ny, int nz, double dt, double* const* u, const double* const* dphi, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !all_dev(u, 3) || !all_dev(dphi, 3))
    return set_error(MF_ERR_ARG, "mf_flow_correct: bad arguments");
  Vec3Out U;
  Vec3 P;
  for (int i = 0; i < 3; ++i) {
    U.c[i] = u[i];
    P.c[i] = dphi[i];
  }
  const long long tot = (long long)nx * ny * nz;
  k_flow_correct<<<nb(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, nz, dt, U, P);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_flow_products(int nx, int ny, int nz, const double* const* u, double* const* uu, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || !all_dev(u, 3) || !all_dev(uu, 6))
    return set_error(MF_ERR_ARG, "mf_flow_products: bad arguments");
  Vec3 U;
  Out6 O;
  for (int i = 0; i < 3; ++i) U.c[i] = u[i];
  for (int q = 0; q < 6; ++q) O.c[q] = uu[q];
  const long long tot = (long long)nx * ny * nz;
  k_flow_products<<<nb(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(tot, U, O);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_flow_curl(int nx, int ny, int nz, const double* const* dpsi, double* const* u, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !all_dev(dpsi, 9) || !all_dev(u, 3))
    return set_error(MF_ERR_ARG, "mf_flow_curl: bad arguments");
  Grad9 D;
  Vec3Out U;
  for (int q = 0; q < 9; ++q) D.g[q] = dpsi[q];
  for (int i = 0; i < 3; ++i) U.c[i] = u[i];
  const long long tot = (long long)nx * ny * nz;
  k_flow_curl<<<nb(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, nz, D, U);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

}  // extern "C"
