// Internal interface between the solver orchestration (mf_solver.cu) and
// the tcgen05 split-precision transform (mf_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "mf_internal.h"

namespace mf {

// One axis transform  Y[n][m] = sum_k B[n][k] * X[m][k]  on the tensor cores,
// with three products hi*hi + hi*lo + lo*hi accumulated in FP32, the
// operands given either as split-BF16 (hi, lo) planes or (3xTF32) as FP32 X
// and two TF32-rounded FP32 planes of B.  X rows have pitch K, Y rows pitch
// M.  M is a multiple of 128, K = N is a multiple of 64 and <= 256.
struct TcEpilogue {
  int kind = 0;                  // 0 store, 1 eigen divide + store, 2 FP32 store/add
  __nv_bfloat16* y_hi = nullptr; // kinds 0,1, BF16 format: [N][M]
  __nv_bfloat16* y_lo = nullptr;
  float* y32 = nullptr;          // kinds 0,1, TF32 format: [N][M]
  // kind 1: m = i + P1*j, n = k
  const float* lam_x = nullptr;  // [P1], [P2], [P3] eigenvalues, 0 past n
  const float* lam_y = nullptr;
  const float* lam_z = nullptr;
  const uint8_t* null_x = nullptr;  // 1 where |lambda| < 1e-11 (FP64 test at set-up)
  const uint8_t* null_y = nullptr;
  const uint8_t* null_z = nullptr;
  float sigma = 0.f;
  int sigma_null = 0;            // |sigma| < 1e-11
  // kind 2: out[i + n1*(j + n2*k)] (+)= y  (interior layout, FP32)
  float* out = nullptr;
  int accumulate = 0;
  int n1 = 0, n2 = 0, n3 = 0, P1 = 0, P2 = 0;
};

struct TcPlan;  // opaque: tensor maps for one transform

// Creates tensor maps for X (rows=M, cols=K) and the matrix planes (N x K):
// BF16 planes, or with tf32 FP32 X (x_lo unused) and FP32 planes.
int tc_plan_create(TcPlan** plan, bool tf32, const void* x_hi, const void* x_lo, const void* b_hi,
                   const void* b_lo, int M, int N, int K);
void tc_plan_destroy(TcPlan* plan);
// plan: 0 the process default (tc_set_tf32_plan), 1 / 2 as below.
int tc_transform(const TcPlan* plan, const TcEpilogue& epi, int* dev_err, cudaStream_t st,
                 int tf32_plan = 0);
// The 128-column 3xTF32 plan exists for this transform (N % 128 == 0).
bool tc_has_wide(const TcPlan* plan);
// 3xTF32 plan: 0 default, 1 64-column slices (B resident), 2 128-column
// slices (B streamed) where N % 128 == 0.  Process-wide.
void tc_set_tf32_plan(int plan);
int tc_get_tf32_plan();

}  // namespace mf
