// Learned LES coefficient: shared device pieces.
//
// A 6-64-64-1 ReLU network maps six dimensionless invariants of the resolved
// velocity gradient g = grad(u) to the coefficient C(x) of the Smagorinsky
// form nu_t = C(x) Delta^2 sqrt(2 S:S) (the plain model is C = const,
// navier_LES type 1, class_navier_3D.f90:1225-1455).  There is no reference
// counterpart: the reference has only the plain models, which here act as
// the per-point fallback outside the training range.
//
// Features (G2 = g:g, S and W the symmetric and antisymmetric parts of g):
//   f0 = S:S / G2            f1 = tr(S^3) / G2^1.5    f2 = tr(W^2 S) / G2^1.5
//   f3 = tr(W^2 S^2) / G2^2  f4 = det(g) / G2^1.5     f5 = tr(g) / G2^0.5
// all invariant under rotations and under scaling of g, and bounded in
// magnitude by 1 (f5 by sqrt(3)).  Features and network run in FP32.
#pragma once
#include <cuda_runtime.h>

#include "mf_line.cuh"
#include "mflops_gb300.h"

namespace mf {

constexpr int kMlpIn = 6, kMlpH = 64;
// parameter layout (FP32): W1[H][In], b1[H], W2[H][H] (row j = output j),
// b2[H], w3[H], b3
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpH * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpH;
constexpr int kMlpB2 = kMlpW2 + kMlpH * kMlpH;
constexpr int kMlpW3 = kMlpB2 + kMlpH;
constexpr int kMlpB3 = kMlpW3 + kMlpH;
constexpr int kMlpParams = kMlpB3 + 1;  // 4673

// Input standardisation and training range of a trained network.
struct MlpScaling {
  float mean[kMlpIn], istd[kMlpIn];  // x_net = (f - mean) * istd
  float lo[kMlpIn], hi[kMlpIn];      // training range of the raw features
  float cscale;                      // C = cscale * network output
};

// FP32 rounding of an FP64 gradient tensor on the integer pipe (narrow():
// GB300's conversion unit runs at the narrow FP64 rate).
__device__ __forceinline__ void narrow_grad(const double gd[3][3], float g[3][3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) g[a][b] = narrow(gd[a][b]);
}

// Invariant features of one gradient tensor (FP32 arithmetic: the features
// only feed the FP32 network, and FP64 would cost about 240 operations per
// point on the narrow FP64 pipe); *ssf receives S:S in FP32.  False when g:g
// lies outside (1e-30, 1e30), where the point falls back.
__device__ __forceinline__ bool grad_features(const float g[3][3], float f[kMlpIn], float* ssf) {
  float g2 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) g2 = fmaf(g[a][b], g[a][b], g2);
  if (!(g2 > 1e-30f) || !(g2 < 1e30f)) return false;
  float S[3][3], W[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      S[a][b] = 0.5f * (g[a][b] + g[b][a]);
      W[a][b] = 0.5f * (g[a][b] - g[b][a]);
    }
  float S2[3][3], W2[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      S2[a][b] = S[a][0] * S[0][b] + S[a][1] * S[1][b] + S[a][2] * S[2][b];
      W2[a][b] = W[a][0] * W[0][b] + W[a][1] * W[1][b] + W[a][2] * W[2][b];
    }
  float ss = 0.f, s3 = 0.f, w2s = 0.f, w2s2 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      ss = fmaf(S[a][b], S[a][b], ss);
      s3 = fmaf(S2[a][b], S[b][a], s3);
      w2s = fmaf(W2[a][b], S[b][a], w2s);
      w2s2 = fmaf(W2[a][b], S2[b][a], w2s2);
    }
  const float det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[2][1]) -
                    g[0][1] * (g[1][0] * g[2][2] - g[1][2] * g[2][0]) +
                    g[0][2] * (g[1][0] * g[2][1] - g[1][1] * g[2][0]);
  *ssf = ss;
  const float ig2 = 1.f / g2, ir = rsqrtf(g2), ir3 = ig2 * ir;
  f[0] = ss * ig2;
  f[1] = s3 * ir3;
  f[2] = w2s * ir3;
  f[3] = w2s2 * ig2 * ig2;
  f[4] = det * ir3;
  f[5] = (g[0][0] + g[1][1] + g[2][2]) * ir;
  return true;
}

// Network output for standardised inputs x; P points to the parameters
// (shared memory in every caller, read as warp-wide broadcasts).
__device__ __forceinline__ float mlp_forward(const float* __restrict__ P, const float x[kMlpIn]) {
  float h1[kMlpH];
#pragma unroll
  for (int j = 0; j < kMlpH; ++j) {
    float a = P[kMlpB1 + j];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) a = fmaf(P[kMlpW1 + j * kMlpIn + k], x[k], a);
    h1[j] = fmaxf(a, 0.f);
  }
  float y = P[kMlpB3];
#pragma unroll 4
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
    y = fmaf(P[kMlpW3 + j], fmaxf(a, 0.f), y);
  }
  return y;
}

// Standardised network input from raw features; false outside the range.
__device__ __forceinline__ bool mlp_input(const MlpScaling& s, const float f[kMlpIn], float x[kMlpIn]) {
  bool in = true;
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) {
    const float v = f[k];
    in = in && (v >= s.lo[k]) && (v <= s.hi[k]);
    x[k] = (v - s.mean[k]) * s.istd[k];
  }
  return in;
}

// Device parameters and scaling of a network handle (host functions).
const float* mlp_device_params(const mf_mlp_t* mlp);
const MlpScaling& mlp_scaling(const mf_mlp_t* mlp);

}  // namespace mf
