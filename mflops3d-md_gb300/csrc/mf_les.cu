// LES eddy viscosity on GB300: one fused pointwise kernel over the nine
// velocity-gradient fields (navier_LES, class_navier_3D.f90:1225-1455, and
// les_sigma, :1458-1502): Smagorinsky, WALE or sigma model, times
// Delta^2 = (dx^2 + dy^2 + dz^2)/3, zero on the edge lines (field_zero_edges,
// class_field.f90:366-391; gradients on edges count as zero as well).
// 72 bytes read + 8 written per point: HBM-bound except the sigma model's
// FP64 acos/cos, which the narrow FP64 pipe of GB300 makes compute-heavy.
#include <cmath>
#include <vector>

#include "mf_internal.h"
#include "mf_mlp.cuh"

namespace mf {

// The reference compares with default-kind (single precision) 1e-10.
static __device__ __constant__ double kLesThresh = (double)1e-10f;

struct LesGrad {
  const double* g[9];  // g[3*i + j] = d u_i / d x_j
};

__device__ __forceinline__ bool on_edge(int i, int j, int k, int nx, int ny, int nz) {
  const int e = (i == 0 || i == nx - 1) + (j == 0 || j == ny - 1) + (k == 0 || k == nz - 1);
  return e >= 2;
}

__device__ __forceinline__ void load_grad(const LesGrad& d, long long idx, double g[3][3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) g[a][b] = d.g[3 * a + b][idx];
}

// S:S and the Smagorinsky-form value c sqrt(2 S:S) Delta^2 with every
// rounding spelled out (no compiler contraction), so that every kernel that
// evaluates the plain model produces the same bits.
__device__ __forceinline__ double strain_ss(const double g[3][3]) {
  double ss = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ss = __fma_rn(g[a][a], g[a][a], ss);
#pragma unroll
    for (int b = a + 1; b < 3; ++b) {
      const double s = __dadd_rn(g[a][b], g[b][a]);
      ss = __fma_rn(__dmul_rn(0.5, s), s, ss);
    }
  }
  return ss;
}

__device__ __forceinline__ double smag_nu(double c, double ss, double dx2, double dy2, double dz2) {
  const double v = __dmul_rn(c, __dsqrt_rn(__dmul_rn(2.0, ss)));
  return __dmul_rn(v, __ddiv_rn(__dadd_rn(__dadd_rn(dx2, dy2), dz2), 3.0));
}

__global__ void k_les_nu(LesGrad d, const double* __restrict__ dx2, const double* __restrict__ dy2,
                         const double* __restrict__ dz2, int nx, int ny, int nz, int type, double c,
                         double* __restrict__ nu) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const int i = (int)(idx % nx);
  const long long jk = idx / nx;
  const int j = (int)(jk % ny), k = (int)(jk / ny);
  if (type == 0 || on_edge(i, j, k, nx, ny, nz)) {
    nu[idx] = 0.0;
    return;
  }
  double g[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) g[a][b] = d.g[3 * a + b][idx];
  double v = 0.0;
  if (type == 1 || type == 2) {
    const double ss = strain_ss(g);
    if (type == 1) {
      nu[idx] = smag_nu(c, ss, dx2[i], dy2[j], dz2[k]);
      return;
    } else {
      double g2[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) g2[a][b] = g[a][0] * g[0][b] + g[a][1] * g[1][b] + g[a][2] * g[2][b];
      const double tr = g2[0][0] + g2[1][1] + g2[2][2];
      double sd = 0.0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          double s = 0.5 * (g2[a][b] + g2[b][a]);
          if (a == b) s -= tr / 3.0;
          sd += s * s;
        }
      // x^1.5, x^2.5 and x^1.25 through square roots: FP64 pow costs tens of
      // operations on the narrow FP64 pipe, a square root a handful
      if (sd < kLesThresh) {
        v = 0.0;
      } else {
        const double rsd = sqrt(sd), rss = sqrt(ss);
        v = c * (sd * rsd) / (ss * ss * rss + sd * sqrt(rsd));  // sd^1.25 = sd sd^(1/4)
      }
    }
  } else {
    // sigma model: singular values of g from the invariants of g g^T
    double G[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) G[a][b] = g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2];
    const double i1 = G[0][0] + G[1][1] + G[2][2];
    const double i2 = G[0][0] * G[1][1] + G[0][0] * G[2][2] + G[1][1] * G[2][2] - G[0][1] * G[1][0] -
                      G[0][2] * G[2][0] - G[1][2] * G[2][1];
    const double i3 = G[0][0] * G[1][1] * G[2][2] + G[1][0] * G[2][1] * G[0][2] +
                      G[2][0] * G[0][1] * G[1][2] - G[0][2] * G[1][1] * G[2][0] -
                      G[1][2] * G[2][1] * G[0][0] - G[2][2] * G[0][1] * G[1][0];
    const double a1 = i1 * i1 / 9.0 - i2 / 3.0;
    const double a2 = i1 * i1 * i1 / 27.0 - i1 * i2 / 6.0 + i3 / 2.0;
    const double sq = sqrt(fmax(a1, 0.0));
    const double a3 = (a1 < kLesThresh) ? 0.0 : acos(a2 / (a1 * sq)) / 3.0;
    // cos(a3 + pi/3) = cos(a3)/2 - sin(a3) sqrt(3)/2: one sincos for both roots
    double sn, cs;
    sincos(a3, &sn, &cs);
    const double h3 = 0.86602540378443864676;  // sqrt(3)/2
    double s1 = i1 / 3.0 + 2.0 * sq * cs;
    double s2 = i1 / 3.0 - 2.0 * sq * (0.5 * cs - h3 * sn);
    double s3 = i1 - s1 - s2;
    s1 = sqrt(fmax(s1, 0.0));
    s2 = sqrt(fmax(s2, 0.0));
    s3 = sqrt(fmax(s3, 0.0));
    v = (s1 < kLesThresh) ? 0.0 : c * s3 * (s1 - s2) * (s2 - s3) / (s1 * s1);
  }
  nu[idx] = v * ((dx2[i] + dy2[j] + dz2[k]) / 3.0);
}

// Training inputs of the learned coefficient: the six invariant features
// (FP32) and b = Delta^2 sqrt(2 S:S), the factor multiplying C; zero on the
// edge lines and where the gradient vanishes.
__global__ void k_les_features(LesGrad d, const double* __restrict__ dx2, const double* __restrict__ dy2,
                               const double* __restrict__ dz2, int nx, int ny, int nz,
                               float* __restrict__ X, float* __restrict__ base) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const int i = (int)(idx % nx);
  const long long jk = idx / nx;
  const int j = (int)(jk % ny), k = (int)(jk / ny);
  float f[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  double b = 0.0;
  if (!on_edge(i, j, k, nx, ny, nz)) {
    double g[3][3];
    load_grad(d, idx, g);
    if (grad_features(g, f)) b = sqrt(2.0 * strain_ss(g)) * ((dx2[i] + dy2[j] + dz2[k]) / 3.0);
  }
#pragma unroll
  for (int q = 0; q < kMlpIn; ++q) X[idx * kMlpIn + q] = f[q];
  base[idx] = (float)b;
}

// A-priori target: the eddy viscosity that reproduces the local subgrid
// dissipation of the filtered field, nu = -tau^d : S / (2 S:S), with
// tau_ij = F(u_i u_j) - F(u_i) F(u_j) from filtered products.
struct SgsFields {
  const double* ub[3];
  const double* uu[6];  // F(u_i u_j): 00, 01, 02, 11, 12, 22
};

__global__ void k_sgs_target(SgsFields s, LesGrad d, int nx, int ny, int nz, float* __restrict__ nu) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const int i = (int)(idx % nx);
  const long long jk = idx / nx;
  const int j = (int)(jk % ny), k = (int)(jk / ny);
  if (on_edge(i, j, k, nx, ny, nz)) {
    nu[idx] = 0.f;
    return;
  }
  double g[3][3];
  load_grad(d, idx, g);
  const double u0 = s.ub[0][idx], u1 = s.ub[1][idx], u2 = s.ub[2][idx];
  double t[3][3];
  t[0][0] = s.uu[0][idx] - u0 * u0;
  t[0][1] = t[1][0] = s.uu[1][idx] - u0 * u1;
  t[0][2] = t[2][0] = s.uu[2][idx] - u0 * u2;
  t[1][1] = s.uu[3][idx] - u1 * u1;
  t[1][2] = t[2][1] = s.uu[4][idx] - u1 * u2;
  t[2][2] = s.uu[5][idx] - u2 * u2;
  const double tr = (t[0][0] + t[1][1] + t[2][2]) / 3.0;
  double ts = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) ts += (t[a][b] - (a == b ? tr : 0.0)) * 0.5 * (g[a][b] + g[b][a]);
  const double ss = strain_ss(g);
  nu[idx] = ss > 1e-300 ? (float)(-ts / (2.0 * ss)) : 0.f;
}

// Learned-coefficient eddy viscosity with per-point fallback: where all six
// features lie inside the training range nu = max(C(x), 0) Delta^2 sqrt(2 S:S)
// with C from the network (FP32, parameters staged in shared memory), else the
// plain Smagorinsky value with coefficient c_fallback, bit-identical to
// k_les_nu type 1.  Edge lines are zero.
__global__ void __launch_bounds__(128) k_les_nu_mlp(LesGrad d, const double* __restrict__ dx2,
                                                    const double* __restrict__ dy2,
                                                    const double* __restrict__ dz2, int nx, int ny, int nz,
                                                    const float* __restrict__ params, MlpScaling s,
                                                    double c_fallback, double* __restrict__ nu,
                                                    unsigned long long* __restrict__ n_fallback) {
  extern __shared__ __align__(16) float sp[];
  for (int q = threadIdx.x; q < kMlpParams; q += blockDim.x) sp[q] = params[q];
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nx * ny * nz) return;
  const int i = (int)(idx % nx);
  const long long jk = idx / nx;
  const int j = (int)(jk % ny), k = (int)(jk / ny);
  if (on_edge(i, j, k, nx, ny, nz)) {
    nu[idx] = 0.0;
    return;
  }
  double g[3][3];
  load_grad(d, idx, g);
  const double ss = strain_ss(g);
  float f[kMlpIn];
  float x[kMlpIn];
  double c = c_fallback;
  const bool in = grad_features(g, f) && mlp_input(s, f, x);
  if (in) {
    c = (double)fmaxf(s.cscale * mlp_forward(sp, x), 0.f);
  } else if (n_fallback) {
    atomicAdd(n_fallback, 1ull);
  }
  nu[idx] = smag_nu(c, ss, dx2[i], dy2[j], dz2[k]);
}

}  // namespace mf

using namespace mf;

struct mf_les {
  int n[3] = {0, 0, 0};
  DevBuf d2[3];  // squared spacings per axis
  DevBuf grad;   // nine gradient fields for mf_les_nu_velocity
  DevBuf count;  // fallback counter of mf_les_nu_mlp
};

extern "C" {

int mf_les_create(const double* gx, int nx, const double* gy, int ny, const double* gz, int nz,
                  mf_les_t** out) {
  if (!gx || !gy || !gz || !out || nx < 2 || ny < 2 || nz < 2)
    return set_error(MF_ERR_ARG, "mf_les_create: bad arguments");
  *out = nullptr;
  mf_les* les = new mf_les();
  const double* g[3] = {gx, gy, gz};
  const int n[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    les->n[a] = n[a];
    std::vector<double> d2(n[a]);
    for (int i = 0; i < n[a]; ++i) {
      double d;
      if (i == 0) d = g[a][1] - g[a][0];
      else if (i == n[a] - 1) d = g[a][i] - g[a][i - 1];
      else d = (g[a][i + 1] - g[a][i - 1]) * 0.5;
      d2[i] = d * d;
    }
    int rc = les->d2[a].ensure(n[a] * 8);
    if (!rc && cudaMemcpy(les->d2[a].ptr, d2.data(), n[a] * 8, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = set_error(MF_ERR_CUDA, "mf_les_create: upload failed");
    if (rc) {
      mf_les_destroy(les);
      return rc;
    }
  }
  *out = les;
  return MF_OK;
}

int mf_les_destroy(mf_les_t* les) {
  if (!les) return MF_OK;
  for (auto& b : les->d2) b.release();
  les->grad.release();
  les->count.release();
  delete les;
  return MF_OK;
}

int mf_les_nu(const mf_les_t* les, int les_type, double c, const double* const* du, double* nu,
              void* stream) {
  if (!les || !du || !nu || les_type < 0 || les_type > 3)
    return set_error(MF_ERR_ARG, "mf_les_nu: bad arguments");
  LesGrad d;
  for (int q = 0; q < 9; ++q) {
    if (!du[q] || !is_device_ptr(du[q])) return set_error(MF_ERR_ARG, "mf_les_nu: device gradients required");
    d.g[q] = du[q];
  }
  if (!is_device_ptr(nu)) return set_error(MF_ERR_ARG, "mf_les_nu: device output required");
  const long long tot = (long long)les->n[0] * les->n[1] * les->n[2];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_les_nu<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(
      d, les->d2[0].as<double>(), les->d2[1].as<double>(), les->d2[2].as<double>(), les->n[0],
      les->n[1], les->n[2], les_type, c, nu);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_les_nu_velocity(mf_les_t* les, const mf_der_t* dcx, const mf_der_t* dcy,
                       const mf_der_t* dcz, int les_type, double c, const double* u,
                       const double* v, const double* w, double* nu, void* stream) {
  if (!les || !dcx || !dcy || !dcz || !u || !v || !w || !nu)
    return set_error(MF_ERR_ARG, "mf_les_nu_velocity: bad arguments");
  const int nx = les->n[0], ny = les->n[1], nz = les->n[2];
  const size_t tot = (size_t)nx * ny * nz;
  int rc = les->grad.ensure(9 * tot * sizeof(double));
  if (rc) return rc;
  const double* vel[3] = {u, v, w};
  const mf_der_t* dc[3] = {dcx, dcy, dcz};
  const double* du[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double* g = les->grad.as<double>() + (3 * i + j) * tot;
      rc = mf_der_apply(dc[j], j, 1, vel[i], g, nx, ny, nz, stream);
      if (rc) return rc;
      du[3 * i + j] = g;
    }
  return mf_les_nu(les, les_type, c, du, nu, stream);
}

static int les_grad_args(const mf_les_t* les, const double* const* du, LesGrad& d, const char* who) {
  if (!les || !du) return set_error(MF_ERR_ARG, "%s: bad arguments", who);
  for (int q = 0; q < 9; ++q) {
    if (!du[q] || !is_device_ptr(du[q])) return set_error(MF_ERR_ARG, "%s: device gradients required", who);
    d.g[q] = du[q];
  }
  return MF_OK;
}

int mf_les_features(const mf_les_t* les, const double* const* du, float* X, float* base, void* stream) {
  LesGrad d;
  int rc = les_grad_args(les, du, d, "mf_les_features");
  if (rc) return rc;
  if (!X || !base || !is_device_ptr(X) || !is_device_ptr(base))
    return set_error(MF_ERR_ARG, "mf_les_features: device outputs required");
  const long long tot = (long long)les->n[0] * les->n[1] * les->n[2];
  k_les_features<<<(unsigned)((tot + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d, les->d2[0].as<double>(), les->d2[1].as<double>(), les->d2[2].as<double>(), les->n[0], les->n[1],
      les->n[2], X, base);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_les_sgs_target(const mf_les_t* les, const double* const* ubar, const double* const* uu,
                      const double* const* du, float* nu_true, void* stream) {
  LesGrad d;
  int rc = les_grad_args(les, du, d, "mf_les_sgs_target");
  if (rc) return rc;
  if (!ubar || !uu || !nu_true || !is_device_ptr(nu_true))
    return set_error(MF_ERR_ARG, "mf_les_sgs_target: bad arguments");
  SgsFields s;
  for (int q = 0; q < 3; ++q) {
    if (!ubar[q] || !is_device_ptr(ubar[q])) return set_error(MF_ERR_ARG, "mf_les_sgs_target: device fields required");
    s.ub[q] = ubar[q];
  }
  for (int q = 0; q < 6; ++q) {
    if (!uu[q] || !is_device_ptr(uu[q])) return set_error(MF_ERR_ARG, "mf_les_sgs_target: device fields required");
    s.uu[q] = uu[q];
  }
  const long long tot = (long long)les->n[0] * les->n[1] * les->n[2];
  k_sgs_target<<<(unsigned)((tot + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      s, d, les->n[0], les->n[1], les->n[2], nu_true);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

int mf_les_nu_mlp(mf_les_t* les, const mf_mlp_t* mlp, double c_fallback, const double* const* du, double* nu,
                  long long* n_fallback, void* stream) {
  LesGrad d;
  int rc = les_grad_args(les, du, d, "mf_les_nu_mlp");
  if (rc) return rc;
  if (!mlp || !nu || !is_device_ptr(nu)) return set_error(MF_ERR_ARG, "mf_les_nu_mlp: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long* cnt = nullptr;
  if (n_fallback) {
    if ((rc = les->count.ensure(sizeof(unsigned long long)))) return rc;
    cnt = les->count.as<unsigned long long>();
    MF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st));
  }
  const long long tot = (long long)les->n[0] * les->n[1] * les->n[2];
  k_les_nu_mlp<<<(unsigned)((tot + 127) / 128), 128, sizeof(float) * kMlpParams, st>>>(
      d, les->d2[0].as<double>(), les->d2[1].as<double>(), les->d2[2].as<double>(), les->n[0], les->n[1],
      les->n[2], mlp_device_params(mlp), mlp_scaling(mlp), c_fallback, nu, cnt);
  MF_CUDA(cudaGetLastError());
  if (n_fallback) {
    unsigned long long h = 0;
    MF_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
    MF_CUDA(cudaStreamSynchronize(st));
    *n_fallback = (long long)h;
  }
  return MF_OK;
}

}  // extern "C"
