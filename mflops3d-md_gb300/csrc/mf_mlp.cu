// Learned LES coefficient: the network object and its training kernels
// (no reference counterpart; see mf_mlp.cuh for the model).
//
// One training step over n points (an optional index list selects them):
//   k_mlp_grad   one CTA per 128 points: forward, loss, backward, and that
//                chunk's partial gradient of all 4,673 parameters, written to
//                its own row of a chunk-gradient table (no atomics, so the
//                sum is deterministic)
//   k_mlp_adam   one thread per parameter: sums the column of the table in
//                chunk order and applies Adam (Kingma & Ba 2015, bias-corrected)
// Loss: L = (1/n) sum_p (C_p b_p - nu_p)^2 * loss_scale, with C_p = cscale *
// net(x_p) and b_p = Delta^2 sqrt(2 S:S): the error of the eddy viscosity
// itself, so points with strong strain weigh most.
#include <cmath>
#include <cstdint>
#include <vector>

#include "mf_internal.h"
#include "mf_mlp.cuh"

namespace mf {

constexpr int kChunk = 128;                       // points per CTA
constexpr int kGradStride = 4676;                 // parameters + loss slot, 16-byte rows
constexpr int kParamsPad = 4676;                  // shared-memory copy of the parameters
constexpr int kHPad = kMlpH + 1;                  // row pitch of the activation tiles
constexpr size_t kGradSmem = sizeof(float) * (kParamsPad + 2 * kChunk * kHPad + kChunk * kMlpIn + 2 * kChunk);

__global__ void __launch_bounds__(kChunk) k_mlp_grad(const float* __restrict__ params, MlpScaling s,
                                                     float scale_over_n, const float* __restrict__ X,
                                                     const float* __restrict__ base,
                                                     const float* __restrict__ target,
                                                     const int* __restrict__ idx, long long n,
                                                     float* __restrict__ G) {
  extern __shared__ __align__(16) float sm[];
  float* P = sm;
  float* H1 = P + kParamsPad;       // h1, later dL/da1
  float* D2 = H1 + kChunk * kHPad;  // h2, later dL/da2
  float* XS = D2 + kChunk * kHPad;  // standardised inputs
  float* DY = XS + kChunk * kMlpIn; // dL/dy
  float* RL = DY + kChunk;          // squared residuals
  const int t = threadIdx.x;
  for (int q = t; q < kMlpParams; q += kChunk) P[q] = params[q];
  const long long pi = (long long)blockIdx.x * kChunk + t;
  const bool valid = pi < n;
  const long long src = valid ? (idx ? (long long)idx[pi] : pi) : 0;
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) {
    x[k] = valid ? (X[src * kMlpIn + k] - s.mean[k]) * s.istd[k] : 0.f;
    XS[t * kMlpIn + k] = x[k];
  }
  const float b = valid ? base[src] : 0.f;
  const float tv = valid ? target[src] : 0.f;
  __syncthreads();
  // forward, keeping h1 and h2 for the backward pass
  {
    float h1[kMlpH];
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
      float a = P[kMlpB1 + j];
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) a = fmaf(P[kMlpW1 + j * kMlpIn + k], x[k], a);
      h1[j] = fmaxf(a, 0.f);
      H1[t * kHPad + j] = h1[j];
    }
    float y = P[kMlpB3];
#pragma unroll 2
    for (int j = 0; j < kMlpH; ++j) {
      const float4* w = reinterpret_cast<const float4*>(P + kMlpW2 + j * kMlpH);
      float a = P[kMlpB2 + j];
#pragma unroll
      for (int i = 0; i < kMlpH / 4; ++i) {
        const float4 q = w[i];
        a = fmaf(q.x, h1[4 * i], a);
        a = fmaf(q.y, h1[4 * i + 1], a);
        a = fmaf(q.z, h1[4 * i + 2], a);
        a = fmaf(q.w, h1[4 * i + 3], a);
      }
      const float h2 = fmaxf(a, 0.f);
      D2[t * kHPad + j] = h2;
      y = fmaf(P[kMlpW3 + j], h2, y);
    }
    const float r = s.cscale * y * b - tv;
    DY[t] = valid ? 2.f * r * b * s.cscale * scale_over_n : 0.f;
    RL[t] = valid ? r * r : 0.f;
  }
  __syncthreads();
  float* g = G + (long long)blockIdx.x * kGradStride;
  if (t < kMlpH) {
    float a = 0.f;
    for (int p = 0; p < kChunk; ++p) a = fmaf(DY[p], D2[p * kHPad + t], a);
    g[kMlpW3 + t] = a;
  } else if (t == kMlpH) {
    float a = 0.f;
    for (int p = 0; p < kChunk; ++p) a += DY[p];
    g[kMlpB3] = a;
  } else if (t == kMlpH + 1) {
    float a = 0.f;
    for (int p = 0; p < kChunk; ++p) a += RL[p];
    g[kMlpParams] = a;
  }
  __syncthreads();
  // dL/da2 in place of h2 (ReLU: h2 > 0 exactly where a2 > 0)
  {
    const float dy = DY[t];
#pragma unroll 8
    for (int j = 0; j < kMlpH; ++j) {
      const float h2 = D2[t * kHPad + j];
      D2[t * kHPad + j] = h2 > 0.f ? dy * P[kMlpW3 + j] : 0.f;
    }
  }
  __syncthreads();
  // dW2[j][i] = sum_p dA2[p][j] h1[p][i]: thread (i = t % 64, 32 rows j from
  // j0 = 32 (t / 64)); in a warp j0 is fixed, so dA2 reads are broadcasts and
  // h1 reads consecutive
  {
    const int i = t & (kMlpH - 1), j0 = (t >> 6) * 32;
    float acc[32];
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) acc[jj] = 0.f;
    for (int p = 0; p < kChunk; ++p) {
      const float h = H1[p * kHPad + i];
#pragma unroll
      for (int jj = 0; jj < 32; ++jj) acc[jj] = fmaf(D2[p * kHPad + j0 + jj], h, acc[jj]);
    }
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) g[kMlpW2 + (j0 + jj) * kMlpH + i] = acc[jj];
  }
  __syncthreads();
  // dL/da1[p][i] = (sum_j dA2[p][j] W2[j][i]) [h1 > 0], in place of h1
  {
    float d1[kMlpH];
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) d1[i] = 0.f;
#pragma unroll 2
    for (int j = 0; j < kMlpH; ++j) {
      const float d = D2[t * kHPad + j];
      const float4* w = reinterpret_cast<const float4*>(P + kMlpW2 + j * kMlpH);
#pragma unroll
      for (int i = 0; i < kMlpH / 4; ++i) {
        const float4 q = w[i];
        d1[4 * i] = fmaf(d, q.x, d1[4 * i]);
        d1[4 * i + 1] = fmaf(d, q.y, d1[4 * i + 1]);
        d1[4 * i + 2] = fmaf(d, q.z, d1[4 * i + 2]);
        d1[4 * i + 3] = fmaf(d, q.w, d1[4 * i + 3]);
      }
    }
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
      const float h1 = H1[t * kHPad + i];
      H1[t * kHPad + i] = h1 > 0.f ? d1[i] : 0.f;
    }
  }
  __syncthreads();
  if (t < kMlpH) {
    // dW1[i][k] = sum_p dA1[p][i] x[p][k], db1[i] = sum_p dA1[p][i]
    float acc[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, bacc = 0.f;
    for (int p = 0; p < kChunk; ++p) {
      const float d = H1[p * kHPad + t];
      bacc += d;
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) acc[k] = fmaf(d, XS[p * kMlpIn + k], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) g[kMlpW1 + t * kMlpIn + k] = acc[k];
    g[kMlpB1 + t] = bacc;
  } else {
    // db2[j] = sum_p dA2[p][j]
    const int j = t - kMlpH;
    float a = 0.f;
    for (int p = 0; p < kChunk; ++p) a += D2[p * kHPad + j];
    g[kMlpB2 + j] = a;
  }
}

struct AdamArgs {
  float lr, beta1, beta2, eps, bc1, bc2;  // bc = 1 - beta^t
};

__global__ void k_mlp_adam(const float* __restrict__ G, int nchunks, float* __restrict__ params,
                           float* __restrict__ m, float* __restrict__ v, AdamArgs a,
                           float* __restrict__ grad_out, float* __restrict__ loss_out, float loss_scale) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > kMlpParams) return;
  float s = 0.f;
  for (int c = 0; c < nchunks; ++c) s += G[(long long)c * kGradStride + q];
  if (q == kMlpParams) {
    if (loss_out) *loss_out = s * loss_scale;
    return;
  }
  if (grad_out) grad_out[q] = s;
  if (a.lr > 0.f) {
    const float mq = a.beta1 * m[q] + (1.f - a.beta1) * s;
    const float vq = a.beta2 * v[q] + (1.f - a.beta2) * s * s;
    m[q] = mq;
    v[q] = vq;
    params[q] -= a.lr * (mq / a.bc1) / (sqrtf(vq / a.bc2) + a.eps);
  }
}

__global__ void __launch_bounds__(128) k_mlp_predict(const float* __restrict__ params, MlpScaling s,
                                                     const float* __restrict__ X, long long n,
                                                     float* __restrict__ C) {
  extern __shared__ __align__(16) float sm[];
  for (int q = threadIdx.x; q < kMlpParams; q += blockDim.x) sm[q] = params[q];
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) x[k] = (X[p * kMlpIn + k] - s.mean[k]) * s.istd[k];
  C[p] = s.cscale * mlp_forward(sm, x);
}

// splitmix64: deterministic initial weights from a seed
static uint64_t splitmix(uint64_t& z) {
  z += 0x9E3779B97F4A7C15ull;
  uint64_t r = z;
  r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
  r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
  return r ^ (r >> 31);
}

}  // namespace mf

using namespace mf;

struct mf_mlp {
  DevBuf params, m, v, grad_table, grad, loss;
  MlpScaling s;
  float loss_scale = 1.f;
  long long step = 0;
};

namespace mf {
const float* mlp_device_params(const mf_mlp_t* mlp) { return mlp->params.as<float>(); }
const MlpScaling& mlp_scaling(const mf_mlp_t* mlp) { return mlp->s; }
}  // namespace mf

extern "C" {

int mf_mlp_create(unsigned long long seed, mf_mlp_t** out) {
  if (!out) return set_error(MF_ERR_ARG, "mf_mlp_create: null output");
  *out = nullptr;
  mf_mlp* mlp = new mf_mlp();
  for (int k = 0; k < kMlpIn; ++k) {
    mlp->s.mean[k] = 0.f;
    mlp->s.istd[k] = 1.f;
    mlp->s.lo[k] = -INFINITY;
    mlp->s.hi[k] = INFINITY;
  }
  mlp->s.cscale = 1.f;
  // He-uniform weights (limit sqrt(6 / fan_in)), zero biases, output bias 1
  // so that an untrained network starts near the constant coefficient cscale
  std::vector<float> p(kMlpParams, 0.f);
  uint64_t z = seed;
  auto uni = [&](float lim) { return lim * (float)((double)(splitmix(z) >> 11) * 0x1.0p-53 * 2.0 - 1.0); };
  for (int q = 0; q < kMlpH * kMlpIn; ++q) p[kMlpW1 + q] = uni(std::sqrt(6.f / kMlpIn));
  for (int q = 0; q < kMlpH * kMlpH; ++q) p[kMlpW2 + q] = uni(std::sqrt(6.f / kMlpH));
  for (int q = 0; q < kMlpH; ++q) p[kMlpW3 + q] = uni(std::sqrt(6.f / kMlpH)) * 0.1f;
  p[kMlpB3] = 1.f;
  int rc;
  if ((rc = mlp->params.ensure(sizeof(float) * kParamsPad)) || (rc = mlp->m.ensure(sizeof(float) * kParamsPad)) ||
      (rc = mlp->v.ensure(sizeof(float) * kParamsPad)) || (rc = mlp->grad.ensure(sizeof(float) * kParamsPad)) ||
      (rc = mlp->loss.ensure(sizeof(float) * 4))) {
    mf_mlp_destroy(mlp);
    return rc;
  }
  if (cudaMemcpy(mlp->params.ptr, p.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(mlp->m.ptr, 0, sizeof(float) * kParamsPad) != cudaSuccess ||
      cudaMemset(mlp->v.ptr, 0, sizeof(float) * kParamsPad) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess) {
    mf_mlp_destroy(mlp);
    return set_error(MF_ERR_CUDA, "mf_mlp_create: upload failed");
  }
  *out = mlp;
  return MF_OK;
}

int mf_mlp_destroy(mf_mlp_t* mlp) {
  if (!mlp) return MF_OK;
  for (DevBuf* b : {&mlp->params, &mlp->m, &mlp->v, &mlp->grad_table, &mlp->grad, &mlp->loss}) b->release();
  delete mlp;
  return MF_OK;
}

int mf_mlp_num_params(void) { return kMlpParams; }

int mf_mlp_get_params(const mf_mlp_t* mlp, float* host) {
  if (!mlp || !host) return set_error(MF_ERR_ARG, "mf_mlp_get_params: bad arguments");
  MF_CUDA(cudaMemcpy(host, mlp->params.ptr, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  return MF_OK;
}

int mf_mlp_set_params(mf_mlp_t* mlp, const float* host) {
  if (!mlp || !host) return set_error(MF_ERR_ARG, "mf_mlp_set_params: bad arguments");
  MF_CUDA(cudaMemcpy(mlp->params.ptr, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  MF_CUDA(cudaMemset(mlp->m.ptr, 0, sizeof(float) * kParamsPad));
  MF_CUDA(cudaMemset(mlp->v.ptr, 0, sizeof(float) * kParamsPad));
  MF_CUDA(cudaDeviceSynchronize());  // ordered before work on any stream
  mlp->step = 0;
  return MF_OK;
}

int mf_mlp_set_scaling(mf_mlp_t* mlp, const float* mean, const float* istd, const float* lo, const float* hi,
                       float cscale, float loss_scale) {
  if (!mlp || !mean || !istd || !lo || !hi || !(cscale > 0.f) || !(loss_scale > 0.f))
    return set_error(MF_ERR_ARG, "mf_mlp_set_scaling: bad arguments");
  for (int k = 0; k < kMlpIn; ++k) {
    mlp->s.mean[k] = mean[k];
    mlp->s.istd[k] = istd[k];
    mlp->s.lo[k] = lo[k];
    mlp->s.hi[k] = hi[k];
  }
  mlp->s.cscale = cscale;
  mlp->loss_scale = loss_scale;
  return MF_OK;
}

int mf_mlp_train_step(mf_mlp_t* mlp, const float* X, const float* base, const float* target, const int* idx,
                      long long n, float lr, float* grad_host, float* loss_host, void* stream) {
  if (!mlp || !X || !base || !target || n <= 0 || !(lr >= 0.f))
    return set_error(MF_ERR_ARG, "mf_mlp_train_step: bad arguments");
  if (!is_device_ptr(X) || !is_device_ptr(base) || !is_device_ptr(target) || (idx && !is_device_ptr(idx)))
    return set_error(MF_ERR_ARG, "mf_mlp_train_step: device arrays required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long nchunks = (n + kChunk - 1) / kChunk;
  if (nchunks > (1LL << 24)) return set_error(MF_ERR_ARG, "mf_mlp_train_step: batch too large");
  int rc = mlp->grad_table.ensure(sizeof(float) * kGradStride * (size_t)nchunks);
  if (rc) return rc;
  MF_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem));
  k_mlp_grad<<<(unsigned)nchunks, kChunk, kGradSmem, st>>>(mlp->params.as<float>(), mlp->s,
                                                           mlp->loss_scale / (float)n, X, base, target, idx, n,
                                                           mlp->grad_table.as<float>());
  MF_CUDA(cudaGetLastError());
  AdamArgs a{lr, 0.9f, 0.999f, 1e-8f, 1.f, 1.f};
  if (lr > 0.f) {
    mlp->step += 1;
    a.bc1 = (float)(1.0 - std::pow(0.9, (double)mlp->step));
    a.bc2 = (float)(1.0 - std::pow(0.999, (double)mlp->step));
  }
  k_mlp_adam<<<(kMlpParams + 1 + 255) / 256, 256, 0, st>>>(
      mlp->grad_table.as<float>(), (int)nchunks, mlp->params.as<float>(), mlp->m.as<float>(), mlp->v.as<float>(), a,
      mlp->grad.as<float>(), mlp->loss.as<float>(), mlp->loss_scale / (float)n);
  MF_CUDA(cudaGetLastError());
  if (grad_host) {
    MF_CUDA(cudaMemcpyAsync(grad_host, mlp->grad.ptr, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st));
  }
  if (loss_host) {
    MF_CUDA(cudaMemcpyAsync(loss_host, mlp->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  if (grad_host || loss_host) MF_CUDA(cudaStreamSynchronize(st));
  return MF_OK;
}

int mf_mlp_predict(const mf_mlp_t* mlp, const float* X, long long n, float* C, void* stream) {
  if (!mlp || !X || !C || n < 0) return set_error(MF_ERR_ARG, "mf_mlp_predict: bad arguments");
  if (n == 0) return MF_OK;
  if (!is_device_ptr(X) || !is_device_ptr(C)) return set_error(MF_ERR_ARG, "mf_mlp_predict: device arrays required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_mlp_predict<<<(unsigned)((n + 127) / 128), 128, sizeof(float) * kParamsPad, st>>>(mlp->params.as<float>(), mlp->s,
                                                                                       X, n, C);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

}  // extern "C"
