// Channel-flow statistics on the GPU: mean, rms and cross-correlation
// profiles in the wall-normal direction and the friction velocity, the
// post-processing of src/main/post_prod.f90:40-238 on snapshots that are
// already in device memory.
//
// One CTA per y plane sums, over the interior (i, k) points and all
// snapshots, the weight s = (x(i+1) - x(i-1)) (z(k+1) - z(k-1)) times the
// field values (first pass) or the products of the normalised deviations
// from the mean (second pass), in FP64 and in a fixed order (per-thread
// strided sums, then a fixed shared-memory tree), so the profiles do not
// depend on scheduling.  A point counts where the first snapshot's u (the
// normalised u in the second pass) exceeds the single-precision literal
// 1e-10, and always on the two wall planes.  Between the passes and after
// the second the host applies the symmetrisation of the reference, takes
// du/dy of the mean u with the library's compact derivative and u_tau.
#include <cmath>
#include <vector>

#include "mf_internal.h"

namespace mf {

constexpr int kStatThreads = 256;
constexpr int kStatSums = 8;  // pass 1: u v w p n; pass 2: uu vv ww pp uv uw vw n

struct StatFields {
  const double* const* u;
  const double* const* v;
  const double* const* w;
  const double* const* p;
};

// pass 0: sums of s*f (f = u, v, w, p) and of s; pass 1: sums of s * products
// of the deviations (f / scale_f - mean_f), scale = u_tau (u_tau^2 for p).
__global__ void __launch_bounds__(kStatThreads) k_plane_sums(StatFields F, int nt, int nx, int ny, int nz,
                                                             const double* __restrict__ dx,
                                                             const double* __restrict__ dz, int pass,
                                                             const double* __restrict__ mean, double utau,
                                                             double* __restrict__ out) {
  __shared__ double red[kStatSums][kStatThreads];
  const int j = blockIdx.x;
  const float thresh = 1e-10f;
  const double su = pass ? utau : 1.0, sp = pass ? utau * utau : 1.0;
  double acc[kStatSums];
#pragma unroll
  for (int q = 0; q < kStatSums; ++q) acc[q] = 0.0;
  const bool wall = j == 0 || j == ny - 1;
  const double mu = pass ? mean[0 * ny + j] : 0.0, mv = pass ? mean[1 * ny + j] : 0.0;
  const double mw = pass ? mean[2 * ny + j] : 0.0, mp = pass ? mean[3 * ny + j] : 0.0;
  const long long ni = nx - 2, nk = nz - 2;
  for (long long q = threadIdx.x; q < ni * nk; q += kStatThreads) {
    const int i = (int)(q % ni) + 1, k = (int)(q / ni) + 1;
    const long long idx = i + (long long)nx * (j + (long long)ny * k);
    const double u0 = pass ? F.u[0][idx] / su : F.u[0][idx];
    if (!(wall || u0 > (double)thresh)) continue;
    const double s = dx[i - 1] * dz[k - 1];
    for (int t = 0; t < nt; ++t) {
      if (pass == 0) {
        acc[0] += F.u[t][idx] * s;
        acc[1] += F.v[t][idx] * s;
        acc[2] += F.w[t][idx] * s;
        acc[3] += F.p[t][idx] * s;
        acc[4] += s;
      } else {
        const double du = F.u[t][idx] / su - mu, dv = F.v[t][idx] / su - mv;
        const double dw = F.w[t][idx] / su - mw, dp = F.p[t][idx] / sp - mp;
        acc[0] += s * (du * du);
        acc[1] += s * (dv * dv);
        acc[2] += s * (dw * dw);
        acc[3] += s * (dp * dp);
        acc[4] += (du * dv) * s;
        acc[5] += (du * dw) * s;
        acc[6] += (dv * dw) * s;
        acc[7] += s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kStatSums; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int h = kStatThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int q = 0; q < kStatSums; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < kStatSums) out[(long long)threadIdx.x * ny + j] = red[threadIdx.x][0];
}

}  // namespace mf

using namespace mf;

extern "C" {

int mf_channel_stats(int nt, const double* const* u, const double* const* v, const double* const* w,
                     const double* const* p, int nx, int ny, int nz, const double* gx, const double* gy,
                     const double* gz, double re, int so, double* moy, double* rms, double* utau_out,
                     void* stream) {
  if (nt < 1 || !u || !v || !w || !p || nx < 3 || ny < 3 || nz < 3 || !gx || !gy || !gz || !moy || !rms ||
      !utau_out || !(re > 0.0))
    return set_error(MF_ERR_ARG, "mf_channel_stats: bad arguments");
  for (int t = 0; t < nt; ++t)
    for (const double* f : {u[t], v[t], w[t], p[t]})
      if (!f || !is_device_ptr(f)) return set_error(MF_ERR_ARG, "mf_channel_stats: device snapshots required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc;
  // device copies of the snapshot pointers and of the weight factors
  std::vector<const double*> ptrs;
  for (const double* const* a : {u, v, w, p})
    for (int t = 0; t < nt; ++t) ptrs.push_back(a[t]);
  std::vector<double> dx(nx - 2), dz(nz - 2);
  for (int i = 1; i < nx - 1; ++i) dx[i - 1] = gx[i + 1] - gx[i - 1];
  for (int k = 1; k < nz - 1; ++k) dz[k - 1] = gz[k + 1] - gz[k - 1];
  DevBuf dptr, ddx, ddz, dmean, dout;
  auto fail = [&](int r) {
    for (DevBuf* b : {&dptr, &ddx, &ddz, &dmean, &dout}) b->release();
    return r;
  };
  if ((rc = dptr.ensure(ptrs.size() * sizeof(double*))) || (rc = ddx.ensure(dx.size() * 8)) ||
      (rc = ddz.ensure(dz.size() * 8)) || (rc = dmean.ensure(4 * (size_t)ny * 8)) ||
      (rc = dout.ensure(kStatSums * (size_t)ny * 8)))
    return fail(rc);
  if (cudaMemcpyAsync(dptr.ptr, ptrs.data(), ptrs.size() * sizeof(double*), cudaMemcpyHostToDevice, st) ||
      cudaMemcpyAsync(ddx.ptr, dx.data(), dx.size() * 8, cudaMemcpyHostToDevice, st) ||
      cudaMemcpyAsync(ddz.ptr, dz.data(), dz.size() * 8, cudaMemcpyHostToDevice, st))
    return fail(set_error(MF_ERR_CUDA, "mf_channel_stats: upload failed"));
  const double* const* dp = dptr.as<const double*>();
  StatFields F{dp, dp + nt, dp + 2 * nt, dp + 3 * nt};
  std::vector<double> sums(kStatSums * (size_t)ny);
  // pass 1: means
  k_plane_sums<<<ny, kStatThreads, 0, st>>>(F, nt, nx, ny, nz, ddx.as<double>(), ddz.as<double>(), 0, nullptr,
                                            1.0, dout.as<double>());
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(sums.data(), dout.ptr, sums.size() * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(set_error(MF_ERR_CUDA, "mf_channel_stats: first pass failed"));
  std::vector<double> m(4 * (size_t)ny);
  for (int q = 0; q < 4; ++q)
    for (int j = 0; j < ny; ++j) m[(size_t)q * ny + j] = sums[(size_t)q * ny + j] / sums[4 * (size_t)ny + j];
  const double sign[4] = {1.0, -1.0, 1.0, 1.0};  // u, v, w, p
  for (int j = 0; j < ny / 2; ++j) {
    const int jj = ny - 1 - j;
    for (int q = 0; q < 4; ++q) {
      double& a = m[(size_t)q * ny + j];
      double& b = m[(size_t)q * ny + jj];
      a = (a + sign[q] * b) * 0.5;
      b = sign[q] * a;
    }
  }
  // u_tau from du/dy of the mean u (compact derivative of order `so`)
  mf_der_t* dc = nullptr;
  if ((rc = mf_der_coeffs_init(gy, ny, 0, so, &dc))) return fail(rc);
  std::vector<double> deru(ny);
  rc = mf_der_apply(dc, 0, 1, m.data(), deru.data(), ny, 1, 1, stream);
  mf_der_destroy(dc);
  if (rc) return fail(rc);
  const double utau = std::sqrt((deru[0] - deru[ny - 1]) * 0.5 / re);
  for (int j = 0; j < ny; ++j) {
    for (int q = 0; q < 3; ++q) m[(size_t)q * ny + j] /= utau;
    m[3 * (size_t)ny + j] /= utau * utau;
  }
  // pass 2: rms and cross terms of the normalised fields
  if (cudaMemcpyAsync(dmean.ptr, m.data(), m.size() * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail(set_error(MF_ERR_CUDA, "mf_channel_stats: upload failed"));
  k_plane_sums<<<ny, kStatThreads, 0, st>>>(F, nt, nx, ny, nz, ddx.as<double>(), ddz.as<double>(), 1,
                                            dmean.as<double>(), utau, dout.as<double>());
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(sums.data(), dout.ptr, sums.size() * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(set_error(MF_ERR_CUDA, "mf_channel_stats: second pass failed"));
  std::vector<double> r(7 * (size_t)ny);
  for (int j = 0; j < ny; ++j) {
    const double n = sums[7 * (size_t)ny + j];
    for (int q = 0; q < 4; ++q) r[(size_t)q * ny + j] = std::sqrt(sums[(size_t)q * ny + j] / n);
    for (int q = 4; q < 7; ++q) r[(size_t)q * ny + j] = sums[(size_t)q * ny + j] / n;
  }
  // symmetrisation: u, v, w, p and uw even as rms values, uv and vw odd
  const bool even_rms[7] = {true, true, true, true, false, true, false};
  for (int j = 0; j < ny / 2; ++j) {
    const int jj = ny - 1 - j;
    for (int q = 0; q < 7; ++q) {
      double& a = r[(size_t)q * ny + j];
      double& b = r[(size_t)q * ny + jj];
      if (even_rms[q]) {
        a = std::sqrt((a * a + b * b) * 0.5);
        b = a;
      } else {
        a = (a - b) * 0.5;
        b = -a;
      }
    }
  }
  for (size_t q = 0; q < m.size(); ++q) moy[q] = m[q];
  for (size_t q = 0; q < r.size(); ++q) rms[q] = r[q];
  *utau_out = utau;
  return fail(MF_OK);
}

}  // extern "C"
