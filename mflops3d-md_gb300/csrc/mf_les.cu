// LES eddy viscosity on GB300: one fused pointwise kernel over the nine
// velocity-gradient fields (navier_LES, class_navier_3D.f90:1225-1455, and
// les_sigma, :1458-1502): Smagorinsky, WALE or sigma model, times
// Delta^2 = (dx^2 + dy^2 + dz^2)/3, zero on the edge lines (field_zero_edges,
// class_field.f90:366-391; gradients on edges count as zero as well).
// 72 bytes read + 8 written per point: HBM-bound except the sigma model's
// FP64 acos/cos, which the narrow FP64 pipe of GB300 makes compute-heavy.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mf_internal.h"
#include "mf_mlp.cuh"
#include "mf_tcgen05.cuh"

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
// evaluates the plain model produces the same bits.  Delta^2 uses the
// rounded 1/3 (within an ulp of the division by 3).
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

// sqrt(x) from an FP32 seed and one Newton (Heron) step in FP64,
// y1 = y0 + (x - y0^2) / (2 y0) with the reciprocal taken in FP32: about
// 2^-48 relative, against ~20 FP64 operations for the correctly rounded
// square root on the narrow FP64 pipe.  Outside the FP32 range, sqrt().
__device__ __forceinline__ double sqrt_heron(double x) {
  if (!(x > 1e-30 && x < 1e30)) return x > 0.0 ? sqrt(x) : 0.0;
  const float y0f = sqrtf((float)x);
  const double y0 = (double)y0f;
  const double r = __fma_rn(-y0, y0, x);
  return __fma_rn(r, (double)(0.5f / y0f), y0);
}

__device__ __forceinline__ double smag_nu(double c, double ss, double dx2, double dy2, double dz2) {
  const double v = __dmul_rn(c, sqrt_heron(__dmul_rn(2.0, ss)));
  return __dmul_rn(v, __dmul_rn(__dadd_rn(__dadd_rn(dx2, dy2), dz2), 1.0 / 3.0));
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
    float gf[3][3], ssf;
    load_grad(d, idx, g);
    narrow_grad(g, gf);
    if (grad_features(gf, f, &ssf)) b = (double)sqrtf(2.f * ssf) * ((dx2[i] + dy2[j] + dz2[k]) * (1.0 / 3.0));
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
// with C from the network, else the plain Smagorinsky value with coefficient
// c_fallback, bit-identical to k_les_nu type 1 (smag_nu).  Edge lines are 0.
//
// The 64x64 hidden layer runs on the tensor cores, 128 points per tile
// (persistent CTAs, two per SM): every thread computes its point's strain
// (FP64), features and first layer (FP32) and writes its h1 row, split
// 3xTF32 (hi = h1 as stored, the hardware keeps its TF32 part; lo = the
// rounded remainder), into 128-byte-swizzled K-major tiles; one thread issues
// 24 tcgen05.mma (128 x 64 x 8: hi*hi + lo*hi + hi*lo over 8 K steps) against
// W2 tiles staged once per CTA, FP32 accumulation in 64 TMEM columns; every
// warp reads its 32 lanes back (tcgen05.ld) for the 64 -> 1 output layer.
// Accuracy ~1e-6 relative, like the FP32 CUDA-core network.
constexpr uint32_t kNuTcA = 0, kNuTcALo = 32768, kNuTcB = 65536, kNuTcBLo = 81920, kNuTcP = 98304;
constexpr uint32_t kNuTcBar = kNuTcP + 2320, kNuTcSlot = kNuTcP + 2336;
constexpr size_t kNuTcSmem = kNuTcP + 2344 + 1024;  // + alignment slack

// Byte offset of FP32 element (row, k) in a K-major 128-byte-swizzled tile
// of `rows` rows and K = 64 (two 32-wide K blocks of rows x 128 bytes).
__device__ __forceinline__ uint32_t sw128(int rows, int row, int k) {
  return (uint32_t)(k >> 5) * rows * 128 + (row >> 3) * 1024 + (row & 7) * 128 +
         ((((k >> 2) & 7) ^ (row & 7)) << 4) + ((k & 3) << 2);
}

__global__ void __launch_bounds__(128) k_les_nu_mlp(LesGrad d, const double* __restrict__ dx2,
                                                    const double* __restrict__ dy2,
                                                    const double* __restrict__ dz2, int nx, int ny, int nz,
                                                    const float* __restrict__ params, MlpScaling s,
                                                    double c_fallback, double* __restrict__ nu,
                                                    unsigned long long* __restrict__ n_fallback,
                                                    int* __restrict__ err) {
  using namespace tcg;
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  float* Ps = reinterpret_cast<float*>(sm + kNuTcP);  // W1[384], b1[64], b2[64], w3[64], b3
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kNuTcBar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kNuTcSlot);
  const int t = threadIdx.x, warp = t >> 5;
  for (int q = t; q < kMlpW2; q += 128) Ps[q] = params[q];  // W1, b1
  for (int q = t; q < kMlpH; q += 128) {
    Ps[448 + q] = params[kMlpB2 + q];
    Ps[512 + q] = params[kMlpW3 + q];
  }
  if (t == 0) Ps[576] = params[kMlpB3];
  for (int e = t; e < kMlpH * kMlpH; e += 128) {
    const float w = params[kMlpW2 + e];
    const uint32_t off = sw128(64, e >> 6, e & 63);
    *reinterpret_cast<float*>(sm + kNuTcB + off) = w;
    *reinterpret_cast<float*>(sm + kNuTcBLo + off) = tf32_lo(w);
  }
  if (t == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(64));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *slot;
  const uint32_t idesc = instr_desc(128, 64, true);
  const long long tot = (long long)nx * ny * nz;
  const long long ntiles = (tot + 127) / 128;
  uint32_t phase = 0;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long idx = tile * 128 + t;
    const bool live = idx < tot;
    int i = 0, j = 0, k = 0;
    if (live) {
      i = (int)(idx % nx);
      const long long jk = idx / nx;
      j = (int)(jk % ny);
      k = (int)(jk / ny);
    }
    const bool edge = live && on_edge(i, j, k, nx, ny, nz);
    double g[3][3];
    float ssf = 0.f;
    bool in = false;
    float h1[kMlpH];
#pragma unroll
    for (int q = 0; q < kMlpH; ++q) h1[q] = 0.f;
    if (live && !edge) {
      float gf[3][3];
      load_grad(d, idx, g);
      narrow_grad(g, gf);
      float f[kMlpIn], x[kMlpIn];
      in = grad_features(gf, f, &ssf) && mlp_input(s, f, x);
      if (in) {
#pragma unroll
        for (int q = 0; q < kMlpH; ++q) {
          float a = Ps[kMlpB1 + q];
#pragma unroll
          for (int m = 0; m < kMlpIn; ++m) a = fmaf(Ps[q * kMlpIn + m], x[m], a);
          h1[q] = fmaxf(a, 0.f);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < kMlpH / 4; ++c) {
      const uint32_t off = sw128(128, t, 4 * c);
      *reinterpret_cast<float4*>(sm + kNuTcA + off) = make_float4(h1[4 * c], h1[4 * c + 1], h1[4 * c + 2], h1[4 * c + 3]);
      *reinterpret_cast<float4*>(sm + kNuTcALo + off) =
          make_float4(tf32_lo(h1[4 * c]), tf32_lo(h1[4 * c + 1]), tf32_lo(h1[4 * c + 2]), tf32_lo(h1[4 * c + 3]));
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      fence_after();
      const uint32_t a0 = smem_u32(sm + kNuTcA), al = smem_u32(sm + kNuTcALo);
      const uint32_t b0 = smem_u32(sm + kNuTcB), bl = smem_u32(sm + kNuTcBLo);
#pragma unroll
      for (int kb = 0; kb < 2; ++kb)
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t ao = kb * 16384 + ks * 32, bo = kb * 8192 + ks * 32;
          mma<true>(tmem, smem_desc(a0 + ao), smem_desc(b0 + bo), idesc, (kb | ks) != 0);
          mma<true>(tmem, smem_desc(al + ao), smem_desc(b0 + bo), idesc, 1);
          mma<true>(tmem, smem_desc(a0 + ao), smem_desc(bl + bo), idesc, 1);
        }
      mma_commit(bar);
    }
    const bool ok = mbar_wait(bar, phase, err, 0);
    phase ^= 1u;
    fence_after();
    float a2[kMlpH];
    tmem_load32(tmem + ((uint32_t)(warp * 32) << 16), a2);
    tmem_load32(tmem + ((uint32_t)(warp * 32) << 16) + 32, a2 + 32);
    if (!ok) break;
    if (live) {
      if (edge) {
        nu[idx] = 0.0;
      } else {
        if (in) {
          // network points: C sqrt(2 S:S) in FP32 (the network's own accuracy)
          float y = Ps[576];
#pragma unroll
          for (int q = 0; q < kMlpH; ++q) y = fmaf(Ps[512 + q], fmaxf(a2[q] + Ps[448 + q], 0.f), y);
          const float v = fmaxf(s.cscale * y, 0.f) * sqrtf(2.f * ssf);
          nu[idx] = (double)v * ((dx2[i] + dy2[j] + dz2[k]) * (1.0 / 3.0));
        } else {
          // fallback points: the plain model's exact FP64 value
          if (n_fallback) atomicAdd(n_fallback, 1ull);
          nu[idx] = smag_nu(c_fallback, strain_ss(g), dx2[i], dy2[j], dz2[k]);
        }
      }
    }
    fence_before();
    __syncthreads();
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64));
  }
}

}  // namespace mf

using namespace mf;

struct mf_les {
  int n[3] = {0, 0, 0};
  DevBuf d2[3];  // squared spacings per axis
  DevBuf grad;   // nine gradient fields for mf_les_nu_velocity
  DevBuf count;  // fallback counter of mf_les_nu_mlp
  DevBuf err;    // bounded-wait flag of the tensor-core kernel
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
  if (cudaDeviceSynchronize() != cudaSuccess) {  // uploads complete before use on any stream
    mf_les_destroy(les);
    return set_error(MF_ERR_CUDA, "mf_les_create: upload failed");
  }
  *out = les;
  return MF_OK;
}

int mf_les_destroy(mf_les_t* les) {
  if (!les) return MF_OK;
  for (auto& b : les->d2) b.release();
  les->grad.release();
  les->count.release();
  les->err.release();
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
  if ((rc = les->err.ensure(sizeof(int)))) return rc;
  MF_CUDA(cudaMemsetAsync(les->err.ptr, 0, sizeof(int), st));
  const long long tiles = (tot + 127) / 128;
  const unsigned grid = (unsigned)std::min<long long>(tiles, 2LL * num_sms());
  MF_CUDA(cudaFuncSetAttribute(k_les_nu_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNuTcSmem));
  k_les_nu_mlp<<<grid, 128, kNuTcSmem, st>>>(d, les->d2[0].as<double>(), les->d2[1].as<double>(),
                                             les->d2[2].as<double>(), les->n[0], les->n[1], les->n[2],
                                             mlp_device_params(mlp), mlp_scaling(mlp), c_fallback, nu, cnt,
                                             les->err.as<int>());
  MF_CUDA(cudaGetLastError());
  if (n_fallback) {
    unsigned long long h = 0;
    int e = 0;
    MF_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
    MF_CUDA(cudaMemcpyAsync(&e, les->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    MF_CUDA(cudaStreamSynchronize(st));
    if (e) return set_error(MF_ERR_TIMEOUT, "mf_les_nu_mlp: tensor-core wait expired");
    *n_fallback = (long long)h;
  }
  return MF_OK;
}

}  // extern "C"
