// Split-precision eigenvector transform on the 5th-generation tensor cores.
//
//   Y[n][m] = sum_k B[n][k] X[m][k],   X = Xh + Xl,  B = Bh + Bl  (BF16 pairs)
//   D = Xh*Bh + Xh*Bl + Xl*Bh           (three tcgen05.mma, FP32 in TMEM)
//
// One CTA owns a 128-row tile of X and the whole N (<= 256) extent of B, so
// the accumulator is a 128-lane x N-column block of tensor memory.  Warp 0
// (one elected thread) streams 64-wide K chunks of Xh, Xl, Bh, Bl with TMA
// into 128-byte-swizzled shared memory (two stages); warp 1 allocates TMEM
// and one of its threads issues the MMAs and commits each stage back to the
// producer.  After the last commit all four warps drain TMEM with
// tcgen05.ld (warp w owns lanes 32w..32w+31) and run the fused epilogue:
//   kind 0: split the FP32 result into BF16 planes Y[n][m] (coalesced in m);
//   kind 1: same, after the eigenvalue divide 1/(lx_i+ly_j+lz_k+sigma);
//   kind 2: add (or store) the result into the FP64 solution u.
// Every mbarrier wait is bounded (about two seconds of clock); on expiry the
// kernel raises *err, skips the remaining work and still releases TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "mf_solver.h"

namespace mf {

struct TcPlan {
  CUtensorMap x_hi, x_lo, b_hi, b_lo;
  int M = 0, N = 0, K = 0;
};

namespace {

constexpr int kBlockM = 128;
constexpr int kChunkK = 64;  // bf16 elements per 128-byte swizzle row
constexpr int kStages = 2;
constexpr long long kWaitCycles = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and *err raised) once the clock budget is spent.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(err, 1);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), sm_100 descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version
  d |= (uint64_t)2 << 61;                   // SWIZZLE_128B
  return d;
}

// Instruction descriptor: kind::f16 with BF16 A/B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_load32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void store_split(__nv_bfloat16* hi, __nv_bfloat16* lo, long long idx,
                                            float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[idx] = h;
  lo[idx] = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void __launch_bounds__(128, 1)
    k_tc_transform(const __grid_constant__ CUtensorMap tx_hi, const __grid_constant__ CUtensorMap tx_lo,
                   const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                   int M, int N, int K, TcEpilogue e, int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
  __shared__ uint32_t tmem_slot;
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const uint32_t a_bytes = kBlockM * 128;        // one 128 x 64 BF16 tile
  const uint32_t b_bytes = (uint32_t)N * 128;    // one N x 64 BF16 tile
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBlockM;
  const int nk = K / kChunkK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // TMEM columns: power of two >= 32 covering N
  const uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (threadIdx.x == 0) {
    // producer
    for (int c = 0; c < nk; ++c) {
      const int s = c % kStages;
      if (c >= kStages && !mbar_wait(&empty_bar[s], ((c / kStages) - 1) & 1, err)) break;
      uint8_t* st = smem + s * stage_bytes;
      mbar_expect_tx(&full_bar[s], stage_bytes);
      tma_load_2d(st, &tx_hi, &full_bar[s], c * kChunkK, m0);
      tma_load_2d(st + a_bytes, &tx_lo, &full_bar[s], c * kChunkK, m0);
      tma_load_2d(st + 2 * a_bytes, &tb_hi, &full_bar[s], c * kChunkK, 0);
      tma_load_2d(st + 2 * a_bytes + b_bytes, &tb_lo, &full_bar[s], c * kChunkK, 0);
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer
    const uint32_t idesc = instr_desc_bf16(kBlockM, N);
    bool ok = true;
    for (int c = 0; c < nk && ok; ++c) {
      const int s = c % kStages;
      ok = mbar_wait(&full_bar[s], (c / kStages) & 1, err);
      if (!ok) break;
      fence_after();
      const uint32_t base = smem_u32(smem + s * stage_bytes);
#pragma unroll
      for (int kk = 0; kk < kChunkK / 16; ++kk) {
        const uint64_t ah = smem_desc(base + kk * 32);
        const uint64_t al = smem_desc(base + a_bytes + kk * 32);
        const uint64_t bh = smem_desc(base + 2 * a_bytes + kk * 32);
        const uint64_t bl = smem_desc(base + 2 * a_bytes + b_bytes + kk * 32);
        mma_bf16(tmem, al, bh, idesc, (c | kk) != 0 ? 1u : 0u);
        mma_bf16(tmem, ah, bl, idesc, 1u);
        mma_bf16(tmem, ah, bh, idesc, 1u);
      }
      mma_commit(&empty_bar[s]);
    }
    if (ok) mma_commit(&done_bar);
  }
  __syncwarp();

  // epilogue: all 128 threads, lane row = warp*32 + lane
  const bool ready = mbar_wait(&done_bar, 0, err);
  fence_after();
  if (ready) {
    const long long m = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    float v[32];
    if (e.kind == 0) {
      for (int cc = 0; cc < N / 32; ++cc) {
        tmem_load32(trow + cc * 32, v);
#pragma unroll
        for (int q = 0; q < 32; ++q) store_split(e.y_hi, e.y_lo, (long long)(cc * 32 + q) * M + m, v[q]);
      }
    } else if (e.kind == 1) {
      const int i = (int)(m % e.P1), j = (int)(m / e.P1);
      const bool valid = (i < e.n1) && (j < e.n2);
      const float lxy = valid ? e.lam_x[i] + e.lam_y[j] : 0.f;
      const bool nxy = valid && e.sigma_null && e.null_x[i] && e.null_y[j];
      for (int cc = 0; cc < N / 32; ++cc) {
        tmem_load32(trow + cc * 32, v);
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int k = cc * 32 + q;
          float r = 0.f;
          if (valid && k < e.n3 && !(nxy && e.null_z[k])) r = v[q] / ((lxy + e.lam_z[k]) + e.sigma);
          store_split(e.y_hi, e.y_lo, (long long)k * M + m, r);
        }
      }
    } else {
      const int i = (int)(m % e.P1), j = (int)(m / e.P1);
      const bool valid = (i < e.n1) && (j < e.n2);
      for (int cc = 0; cc < N / 32; ++cc) {
        tmem_load32(trow + cc * 32, v);
        if (!valid) continue;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int k = cc * 32 + q;
          if (k >= e.n3) continue;
          const long long idx = i + (long long)e.n1 * (j + (long long)e.n2 * k);
          e.u[idx] = e.accumulate ? e.u[idx] + (double)v[q] : (double)v[q];
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encode() {
  if (g_encode) return MF_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
    return set_error(MF_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return MF_OK;
}

int make_map(CUtensorMap* map, const __nv_bfloat16* ptr, int rows, int cols, int box_rows) {
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(ptr),
                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(MF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return MF_OK;
}

}  // namespace

int tc_plan_create(TcPlan** out, const __nv_bfloat16* x_hi, const __nv_bfloat16* x_lo,
                   const __nv_bfloat16* b_hi, const __nv_bfloat16* b_lo, int M, int N, int K) {
  *out = nullptr;
  if (M % kBlockM || K % kChunkK || N != K || N < 64 || N > 256 || N % 32)
    return set_error(MF_ERR_UNSUPPORTED, "tensor-core transform: unsupported shape M=%d N=%d K=%d", M,
                     N, K);
  for (const void* p : {(const void*)x_hi, (const void*)x_lo, (const void*)b_hi, (const void*)b_lo})
    if (reinterpret_cast<uintptr_t>(p) % 16)
      return set_error(MF_ERR_ARG, "tensor-core transform: operands must be 16-byte aligned");
  int rc = get_encode();
  if (rc) return rc;
  TcPlan* p = new TcPlan();
  p->M = M;
  p->N = N;
  p->K = K;
  if ((rc = make_map(&p->x_hi, x_hi, M, K, kBlockM)) || (rc = make_map(&p->x_lo, x_lo, M, K, kBlockM)) ||
      (rc = make_map(&p->b_hi, b_hi, N, K, N)) || (rc = make_map(&p->b_lo, b_lo, N, K, N))) {
    delete p;
    return rc;
  }
  *out = p;
  return MF_OK;
}

void tc_plan_destroy(TcPlan* p) { delete p; }

int tc_transform(const TcPlan* p, const TcEpilogue& e, int* dev_err, cudaStream_t st) {
  const size_t stage = 2 * (size_t)kBlockM * 128 + 2 * (size_t)p->N * 128;
  const size_t smem = kStages * stage + 1024;
  static bool attr = false;
  if (!attr) {
    MF_CUDA(cudaFuncSetAttribute(k_tc_transform, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kStages * (2 * kBlockM * 128 + 2 * 256 * 128) + 1024)));
    attr = true;
  }
  k_tc_transform<<<p->M / kBlockM, 128, smem, st>>>(p->x_hi, p->x_lo, p->b_hi, p->b_lo, p->M, p->N,
                                                    p->K, e, dev_err);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

}  // namespace mf
