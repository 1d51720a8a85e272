// Split-precision eigenvector transform on the 5th-generation tensor cores.
//
//   Y[n][m] = sum_k B[n][k] X[m][k],   X = Xh + Xl,  B = Bh + Bl
//   D = Xh*Bh + Xh*Bl + Xl*Bh           (three tcgen05.mma, FP32 in TMEM)
//
// Two operand formats:
//  * split-BF16 (kind::f16): X is stored as two BF16 planes, B likewise;
//  * 3xTF32 (kind::tf32): X is stored as FP32.  The tensor core reads an FP32
//    operand as TF32 by ignoring its 13 low mantissa bits, so the landed
//    tile itself is the hi part, trunc(x); converter warps copy it and the
//    lo part rna_tf32(x - trunc(x)) into TMEM, where all three MMAs read
//    their A operand, so that shared memory serves only B and the landed
//    tiles (an MMA reading both operands from shared memory is bound by
//    its 128 bytes per cycle).  B is stored as two TF32-rounded FP32
//    planes.  Each 128-byte swizzle row holds 32 K values instead of 64, and
//    the split keeps ~21 bits of every operand instead of ~16, which lets
//    one refinement step reach 1e-10.
//
// Persistent, warp-specialised kernel (one CTA per SM):
//  * the N extent is cut into NS slices of NW = N/NS columns; a CTA owns one
//    slice and keeps both BF16 planes of that slice of B resident in shared
//    memory (K x NW x 2 planes, <= 128 KB), loaded once by TMA;
//  * warp 0 (one lane) streams 128 x 64 chunks of Xh and Xl through a ring
//    of TMA stages (128-byte swizzle);
//  * warp 1 allocates TMEM and one lane issues the three tcgen05.mma per
//    32-byte K step into one of two accumulator sets, so the MMAs of tile
//    t+1 overlap the epilogue of tile t.  BF16: one FP32 accumulator per set
//    (NW columns).  TF32: three per set, because every MMA rounds its
//    running sum and the error grows with the number of MMAs accumulated
//    into one sum: the small products hi*lo + lo*hi, and hi*hi over the
//    first and over the second half of K, are summed by the epilogue;
//  * (3xTF32 only) 4 converter warps copy each landed FP32 stage (hi and lo
//    parts) into one of kOpSlots TMEM operand slots and release the ring
//    stage; the MMA thread issues up to kOpSlots converted stages per
//    barrier test;
//  * the epilogue warps (8 for BF16, 4 for TF32) drain the accumulator with
//    tcgen05.ld (warp w owns TMEM lanes 32*(w%4)..+31) and run the fused
//    epilogue:
//      kind 0: store the result Y[n][m] (coalesced in m) in the operand format
//              of the next transform (BF16 planes or FP32);
//      kind 1: same, after the eigenvalue divide 1/(lx_i+ly_j+lz_k+sigma);
//      kind 2: add (or store) the result into the FP32 solution array.
// The two CTAs that own the two slices of the same M tile run in step, so
// the second read of each X tile is served by L2.
// Every mbarrier wait is bounded (about two seconds of clock); on expiry the
// kernel raises *err, skips the remaining work and still releases TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "mf_solver.h"
#include "mf_tcgen05.cuh"

namespace mf {

struct TcPlan {
  CUtensorMap x_hi, x_lo, b_hi, b_lo;  // x_lo unused for 3xTF32
  CUtensorMap b_hi_w, b_lo_w;          // 3xTF32 with N % 128 == 0: 128-row boxes of B
  int M = 0, N = 0, K = 0;
  bool tf32 = false;
  bool wide = false;                   // the 128-column plan is available
};

// 3xTF32 plan choice: 0 = default (128-column slices where N % 128 == 0),
// 1 = 64-column slices with B resident, 2 = 128-column slices when possible.
static int g_tf32_plan = 0;
void tc_set_tf32_plan(int plan) { g_tf32_plan = plan; }
int tc_get_tf32_plan() { return g_tf32_plan; }

namespace {

constexpr int kBlockM = 128;

// Per-format constants.  Warp roles: 0 TMA, 1 MMA, then the epilogue warps,
// then (TF32) the converter warps.
template <bool kTf32>
struct Cfg {
  static constexpr int kChunkK = kTf32 ? 32 : 64;  // K values per 128-byte swizzle row
  static constexpr int kEpiWarps = kTf32 ? 4 : 8;  // one or two per TMEM lane quarter
  static constexpr int kCvtWarps = kTf32 ? 4 : 0;
  static constexpr int kEpiThreads = 32 * kEpiWarps;
  static constexpr int kCvtThreads = 32 * kCvtWarps;
  static constexpr int kThreads = 64 + kEpiThreads + kCvtThreads;
};

using namespace mf::tcg;

__device__ __forceinline__ void store_split(__nv_bfloat16* hi, __nv_bfloat16* lo, int idx,
                                            float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[idx] = h;
  lo[idx] = __float2bfloat16_rn(v - __bfloat162float(h));
}


constexpr int kMaxStages = 8;
// 3xTF32: the A operand (hi and lo parts) lives in TMEM, where the tensor
// core reads it without using shared-memory bandwidth; operand slots of
// 64 columns (hi at +0, lo at +32) follow the two accumulator sets
// (2 x 3 x 64 = 384 columns).  Shared memory then carries only the landed
// tiles and B: an MMA that reads A and B from shared memory is bound by
// its 128 bytes per cycle.
constexpr int kOpSlots = 2;
constexpr uint32_t kOpCol = 384;
// Stages whose A boxes are prefetched into L2 ahead of their shared-memory
// load.  A load that misses L2 takes ~2 us on a busy GB300, several times
// the time the tensor cores need for the stages that fit in the ring.
constexpr int kPrefetchAhead = 8;

// Shared-memory plan of one launch (host and device agree on it).  A BF16
// stage holds two 128 x 128-byte tiles (the hi and lo planes), a 3xTF32
// stage one (the FP32 tile; its lo part goes to TMEM).
struct TcShape {
  int NS, NW, nk, stages, tiles;  // tiles: 128 x 128-byte tiles per stage
  __host__ __device__ uint32_t b_chunk() const { return (uint32_t)NW * 128; }
  __host__ __device__ uint32_t b_bytes() const { return 2u * nk * b_chunk(); }
  __host__ __device__ uint32_t a_stage() const { return (uint32_t)tiles * kBlockM * 128; }
  __host__ __device__ uint32_t smem() const { return b_bytes() + stages * a_stage() + 1024; }
};

// Epilogue of 32 accumulator columns n0..n0+31 of row m (all indices fit in
// 32 bits: M*N and n1*n2*n3 are below 2^31 for every supported shape).
// (i, j) = (m % P1, m / P1) for kinds 1 and 2, computed once per tile.
template <bool kTf32>
__device__ __forceinline__ void store_y(const TcEpilogue& e, int idx, float v) {
  if constexpr (kTf32)
    e.y32[idx] = v;
  else
    store_split(e.y_hi, e.y_lo, idx, v);
}

template <bool kTf32>
__device__ __forceinline__ void epilogue_cols(const TcEpilogue& e, const float* v, int M, int m,
                                              int n0, int i, int j, bool valid, float lxy, bool nxy,
                                              const float* s_lz, const uint8_t* s_nz) {
  if (e.kind == 0) {
    int idx = n0 * M + m;
#pragma unroll
    for (int q = 0; q < 32; ++q, idx += M) store_y<kTf32>(e, idx, v[q]);
  } else if (e.kind == 1) {
    // s_lz holds lam_z(k) + sigma
    int idx = n0 * M + m;
    if (valid && !nxy && n0 + 32 <= e.n3) {
#pragma unroll
      for (int q = 0; q < 32; ++q, idx += M)
        store_y<kTf32>(e, idx, __fdividef(v[q], lxy + s_lz[n0 + q]));
    } else {
#pragma unroll
      for (int q = 0; q < 32; ++q, idx += M) {
        const int k = n0 + q;
        float r = 0.f;
        if (valid && k < e.n3 && !(nxy && s_nz[k])) r = __fdividef(v[q], lxy + s_lz[k]);
        store_y<kTf32>(e, idx, r);
      }
    }
  } else {
    if (!valid) return;
    const int plane = e.n1 * e.n2;
    const int base = i + e.n1 * j + n0 * plane;
    const int cols = min(32, e.n3 - n0);
    float old[32];
    // all loads first: the stores below may alias them as far as the
    // compiler knows, which would otherwise serialise load -> add -> store
#pragma unroll
    for (int q = 0; q < 32; ++q) old[q] = (e.accumulate && q < cols) ? e.out[base + q * plane] : 0.f;
#pragma unroll
    for (int q = 0; q < 32; ++q)
      if (q < cols) e.out[base + q * plane] = old[q] + v[q];
  }
}

template <bool kTf32>
__global__ void __launch_bounds__(Cfg<kTf32>::kThreads, 1)
    k_tc_transform(const __grid_constant__ CUtensorMap tx_hi, const __grid_constant__ CUtensorMap tx_lo,
                   const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                   int M, TcShape sh, TcEpilogue e, int* err) {
  using C = Cfg<kTf32>;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar_b, full_bar[kMaxStages], empty_bar[kMaxStages], acc_full[2], acc_empty[2];
  __shared__ uint64_t cvt_bar[kOpSlots], op_free[kOpSlots];  // 3xTF32 operand slots in TMEM
  __shared__ uint32_t tmem_slot;
  __shared__ float s_lz[256];     // z eigenvalues (divide epilogue)
  __shared__ uint8_t s_nz[256];   // z null-mode flags
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (e.kind == 1)
    for (int k = threadIdx.x; k < 256; k += blockDim.x) {
      s_lz[k] = k < e.n3 ? e.lam_z[k] + e.sigma : 0.f;
      s_nz[k] = k < e.n3 ? e.null_z[k] : 0;
    }
  const int NW = sh.NW, nk = sh.nk, S = sh.stages;
  const int slice = blockIdx.x % sh.NS;
  const int cta_rank = blockIdx.x / sh.NS, cta_count = gridDim.x / sh.NS;
  const int mtiles = M / kBlockM;
  const uint32_t bchunk = sh.b_chunk();
  uint8_t* b_hi = smem;
  uint8_t* b_lo = smem + (size_t)nk * bchunk;
  uint8_t* a_base = smem + sh.b_bytes();
  constexpr uint32_t kTile = kBlockM * 128;  // one 128-row x 128-byte tile

  if (threadIdx.x == 0) {
    mbar_init(&bar_b, 1);
    for (int s = 0; s < S; ++s) {
      mbar_init(&full_bar[s], 1);
      // released by the MMA commit (BF16) or by the converters once they
      // have read the stage (3xTF32)
      mbar_init(&empty_bar[s], kTf32 ? C::kCvtThreads : 1);
    }
    for (int o = 0; o < kOpSlots; ++o) {
      mbar_init(&cvt_bar[o], C::kCvtThreads > 0 ? C::kCvtThreads : 1);
      mbar_init(&op_free[o], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], C::kEpiThreads);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int set_cols = kTf32 ? 3 * NW : NW;  // TMEM columns of one accumulator set
  const uint32_t ncols = 2 * set_cols <= 32    ? 32
                         : 2 * set_cols <= 64  ? 64
                         : 2 * set_cols <= 128 ? 128
                         : 2 * set_cols <= 256 ? 256
                                               : 512;
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

  if (warp == 0) {
    if (lane == 0) {
      // resident slice of B
      mbar_expect_tx(&bar_b, sh.b_bytes());
      for (int c = 0; c < nk; ++c) {
        tma_load_2d(b_hi + (size_t)c * bchunk, &tb_hi, &bar_b, c * C::kChunkK, slice * NW);
        tma_load_2d(b_lo + (size_t)c * bchunk, &tb_lo, &bar_b, c * C::kChunkK, slice * NW);
      }
      int it = 0, s = 0;
      uint32_t ph = 0;  // phase of the current use of stage s
      bool ok = true;
      // prefetch cursor: (pt, pc) runs kPrefetchAhead stages ahead of (t, c)
      int pt = cta_rank, pc = 0;
      auto prefetch_next = [&]() {
        if (pt >= mtiles) return;
        tma_prefetch_2d(&tx_hi, pc * C::kChunkK, pt * kBlockM);
        if constexpr (!kTf32) tma_prefetch_2d(&tx_lo, pc * C::kChunkK, pt * kBlockM);
        if (++pc == nk) {
          pc = 0;
          pt += cta_count;
        }
      };
      for (int q = 0; q < kPrefetchAhead; ++q) prefetch_next();
      for (int t = cta_rank; t < mtiles && ok; t += cta_count) {
        for (int c = 0; c < nk; ++c) {
          prefetch_next();
          if (it >= S && !(ok = mbar_wait(&empty_bar[s], ph ^ 1u, err))) break;
          uint8_t* st = a_base + (size_t)s * sh.a_stage();
          if constexpr (kTf32) {
            mbar_expect_tx(&full_bar[s], kTile);
            tma_load_2d(st, &tx_hi, &full_bar[s], c * C::kChunkK, t * kBlockM);
          } else {
            mbar_expect_tx(&full_bar[s], 2 * kTile);
            tma_load_2d(st, &tx_hi, &full_bar[s], c * C::kChunkK, t * kBlockM);
            tma_load_2d(st + kTile, &tx_lo, &full_bar[s], c * C::kChunkK, t * kBlockM);
          }
          ++it;
          if (++s == S) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // This single thread paces the whole CTA, so its loop is kept short:
      // descriptors are formed once and advanced by adding the byte offset
      // / 16 to their start-address field, stage and phase are counters.
      const uint32_t idesc = instr_desc(kBlockM, NW, kTf32);
      bool ok = mbar_wait(&bar_b, 0, err);
      const uint64_t a0 = smem_desc(smem_u32(a_base));
      const uint64_t bh0 = smem_desc(smem_u32(b_hi)), bl0 = smem_desc(smem_u32(b_lo));
      const uint32_t a_step = sh.a_stage() >> 4, b_step = bchunk >> 4, lo_off = kTile >> 4;
      int s = 0, o = 0, tc = 0;
      uint32_t ph = 0, pho = 0;  // phases of ring stage s (BF16) and TMEM operand slot o (TF32)
      for (int t = cta_rank; t < mtiles && ok; t += cta_count, ++tc) {
        const int b = tc & 1, u = tc >> 1;
        if (u > 0 && !(ok = mbar_wait(&acc_empty[b], (u - 1) & 1, err))) break;
        fence_after();
        const uint32_t d = tmem + (uint32_t)(b * set_cols);
        if constexpr (kTf32) {
          // Up to kOpSlots converted stages per barrier test: the converters
          // finish stages in order, so a converted later stage implies the
          // earlier one, and the tensor pipe (idle while this thread tests
          // a barrier) gets the MMAs of both in a row.
          for (int c = 0; c < nk && ok;) {
            int m = min(kOpSlots, nk - c);
            if (m == 2 && !mbar_test(&cvt_bar[o ^ 1], pho ^ (o == 1 ? 1u : 0u))) m = 1;
            if (m == 1 && !(ok = mbar_wait(&cvt_bar[o], pho, err))) break;
            fence_after();
            for (int q = 0; q < m; ++q, ++c) {
              const uint64_t bh = bh0 + (uint64_t)(c * b_step), bl = bl0 + (uint64_t)(c * b_step);
              const uint32_t ahi = tmem + kOpCol + (uint32_t)(64 * o), alo = ahi + 32;
              // hi*hi of the first / second half of K into its own sum; hi*lo
              // and lo*hi into the small-product sum
              const uint32_t dh = d + (uint32_t)((c < nk / 2 ? 1 : 2) * NW);
              const uint32_t acc_h = (c == 0 || c == nk / 2) ? 0u : 1u, acc_l = c == 0 ? 0u : 1u;
              // the small-product sum takes the four hi*lo products of the
              // stage, then its four lo*hi products (the order of the wide
              // form, which issues the hi products before the lo operand is
              // converted)
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                mma_tf32_ta(dh, ahi + 8 * kk, bh + 2 * kk, idesc, kk ? 1u : acc_h);
                mma_tf32_ta(d, ahi + 8 * kk, bl + 2 * kk, idesc, kk ? 1u : acc_l);
              }
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) mma_tf32_ta(d, alo + 8 * kk, bh + 2 * kk, idesc, 1u);
              mma_commit(&op_free[o]);
              if (++o == kOpSlots) {
                o = 0;
                pho ^= 1u;
              }
            }
          }
        } else {
          uint64_t bh = bh0, bl = bl0;
          for (int c = 0; c < nk; ++c) {
            if (!(ok = mbar_wait(&full_bar[s], ph, err))) break;
            fence_after();
            const uint64_t ah = a0 + (uint64_t)(s * a_step), al = ah + lo_off;
            // four 32-byte K steps (16 BF16 values) per 128-byte row
            const uint32_t acc0 = c == 0 ? 0u : 1u;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              mma<false>(d, al + 2 * kk, bh + 2 * kk, idesc, kk ? 1u : acc0);
              mma<false>(d, ah + 2 * kk, bl + 2 * kk, idesc, 1u);
              mma<false>(d, ah + 2 * kk, bh + 2 * kk, idesc, 1u);
            }
            mma_commit(&empty_bar[s]);
            bh += b_step;
            bl += b_step;
            if (++s == S) {
              s = 0;
              ph ^= 1u;
            }
          }
        }
        if (ok) mma_commit(&acc_full[b]);
      }
    }
  } else if (warp < 2 + C::kEpiWarps) {
    const int q = warp & 3;                 // TMEM lane quarter this warp may access
    const int part = (warp - 2) >> 2;       // which share of the NW columns
    constexpr int parts = C::kEpiWarps / 4;
    const int row = q * 32 + lane;
    const int chunks = NW / 32, per = (chunks + parts - 1) / parts;  // split on 32-column chunks
    const int c_lo = part * per * 32, c_hi = min(NW, (part + 1) * per * 32);
    int tc = 0;
    for (int t = cta_rank; t < mtiles; t += cta_count, ++tc) {
      const int b = tc & 1;
      if (!mbar_wait(&acc_full[b], (tc >> 1) & 1, err, 128)) break;
      __syncwarp();
      fence_after();
      const int m = t * kBlockM + row;
      int i = 0, j = 0;
      bool valid = false, nxy = false;
      float lxy = 0.f;
      if (e.kind != 0) {
        i = m % e.P1;
        j = m / e.P1;
        valid = (i < e.n1) && (j < e.n2);
        if (e.kind == 1 && valid) {
          lxy = e.lam_x[i] + e.lam_y[j];
          nxy = e.sigma_null && e.null_x[i] && e.null_y[j];
        }
      }
      const uint32_t trow = tmem + (static_cast<uint32_t>(q * 32) << 16) + (uint32_t)(b * set_cols);
      float v[32];
      for (int cc = c_lo; cc < c_hi; cc += 32) {
        tmem_load32(trow + cc, v);
        if constexpr (kTf32) {
          // (s + h1) + h2: h1 = hi*hi over the first half of K at +NW, h2
          // over the second half at +2NW
          float w[32];
          tmem_load32(trow + NW + cc, w);
#pragma unroll
          for (int x = 0; x < 32; ++x) v[x] += w[x];
          tmem_load32(trow + 2 * NW + cc, w);
#pragma unroll
          for (int x = 0; x < 32; ++x) v[x] += w[x];
        }
        epilogue_cols<kTf32>(e, v, M, m, slice * NW + cc, i, j, valid, lxy, nxy, s_lz, s_nz);
      }
      fence_before();
      mbar_arrive(&acc_empty[b]);
    }
  } else if constexpr (kTf32) {
    // Converter warps: every landed FP32 stage goes to a TMEM operand slot,
    // one tile row per thread: hi = the FP32 bits (read as TF32, i.e.
    // truncated, by the tensor core) and lo = rna_tf32(x - trunc(x)).  A
    // warp reaches only its TMEM lane quarter, so warp w converts rows
    // 32*(w%4)..+31.  The tile has the 128-byte swizzle: 16-byte chunk j of
    // row r sits at chunk position j ^ (r % 8).  The ring stage is released
    // as soon as it has been read.
    const int row = 32 * (warp & 3) + lane;
    const uint32_t lane_base = static_cast<uint32_t>(32 * (warp & 3)) << 16;
    int s = 0, o = 0, it = 0;
    uint32_t ph = 0, pho = 0;
    bool ok = true;
    for (int t = cta_rank; t < mtiles && ok; t += cta_count) {
      for (int c = 0; c < nk; ++c, ++it) {
        if (!(ok = mbar_wait(&full_bar[s], ph, err, 32))) break;
        const float4* rowp =
            reinterpret_cast<const float4*>(a_base + (size_t)s * sh.a_stage() + (size_t)row * 128);
        float hi[32], lo[32];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 x = rowp[j ^ (row & 7)];
          hi[4 * j + 0] = x.x;
          hi[4 * j + 1] = x.y;
          hi[4 * j + 2] = x.z;
          hi[4 * j + 3] = x.w;
        }
        // reads done: the ring stage may be refilled by TMA
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&empty_bar[s]);
#pragma unroll
        for (int q = 0; q < 32; ++q) lo[q] = tf32_lo(hi[q]);
        // the operand slot is free once the MMAs of its previous stage completed
        if (it >= kOpSlots && !(ok = mbar_wait(&op_free[o], pho ^ 1u, err, 32))) break;
        const uint32_t slot = tmem + lane_base + kOpCol + (uint32_t)(64 * o);
        tmem_store32(slot, hi);
        tmem_store32(slot + 32, lo);
        fence_before();
        mbar_arrive(&cvt_bar[o]);
        if (++s == S) {
          s = 0;
          ph ^= 1u;
        }
        if (++o == kOpSlots) {
          o = 0;
          pho ^= 1u;
        }
      }
    }
  }
  __syncwarp();
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

// ---------------------------------------------------------------------------
// 3xTF32 with 128-column N slices ("wide" plan).
//
// Same products and the same three accumulators per output as above, but a
// CTA owns 128 columns of N (two slices for N = 256), so every tcgen05.mma
// is M128 N128 K8: twice the work per instruction of the N64 form, whose
// rate in the kernel is bound by the single issuing thread.  The slice of B
// (hi and lo planes, 256 KB for K = 256) no longer fits in shared memory
// beside the ring, so it streams with the X tiles: a ring stage holds the
// FP32 X tile (16 KB) and both B planes of the same 32 K values (2 x 16 KB);
// B is 512 KB in all and stays in L2.  TMEM: the three accumulators of one
// tile (h1 = hi*hi over the first half of K, h2 = over the second half,
// s = hi*lo + lo*hi; 3 x 128 columns) and four slots for the lo part of
// the A operand (4 x 32 columns, one stage each).  The hi part is the landed FP32 tile
// itself (the tensor core reads FP32 as TF32 by ignoring the low mantissa
// bits), so the hi*hi and hi*lo MMAs take A from shared memory and the
// converter warps only form and store lo.  The accumulators are
// single-buffered: the next tile's first MMAs wait until the epilogue warps
// have read s and h1, its second half until they have read h2; the stores
// follow.  Each output sums the same products in the same accumulators as
// the narrow form and the epilogue adds (s + h1) + h2 in the same order,
// so both forms give identical results.
constexpr int kWideNW = 128;
constexpr int kWideStages = 4;
constexpr int kWideEpiWarps = 8;
constexpr int kWideCvtWarps = 4;
constexpr int kWideThreads = 64 + 32 * (kWideEpiWarps + kWideCvtWarps);
constexpr uint32_t kWideTile = kBlockM * 128;          // 16 KB: 128 rows x 32 FP32
constexpr uint32_t kWideStage = 3 * kWideTile;          // X tile + B hi + B lo
constexpr uint32_t kWideSmem = kWideStages * kWideStage + 1024;
constexpr uint32_t kWideH1 = 0, kWideH2 = 128, kWideS = 256, kWideSlot = 384;
// one operand slot per ring stage, each the lo part of that stage's 32 K
// values.  A slot needs no barrier of its own: the converters write slot s
// only after stage s has landed again, which the producer issued only after
// the stage's previous use was released, and that release (empty_bar) waits
// for the commit that follows the MMAs which read the slot
constexpr int kWideSlots = kWideStages;
constexpr uint32_t kWideSlotCols = 32;

__global__ void __launch_bounds__(kWideThreads, 1)
    k_tc_tf32_wide(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tb_hi,
                   const __grid_constant__ CUtensorMap tb_lo, int M, int N, int K, TcEpilogue e,
                   int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[kWideStages], empty_bar[kWideStages];
  __shared__ uint64_t cvt_bar[kWideSlots];
  __shared__ uint64_t acc_full, acc_free, h2_free;
  __shared__ uint32_t tmem_slot;
  __shared__ float s_lz[256];
  __shared__ uint8_t s_nz[256];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kCvtThreads = 32 * kWideCvtWarps, kEpiThreads = 32 * kWideEpiWarps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (e.kind == 1)
    for (int k = threadIdx.x; k < 256; k += blockDim.x) {
      s_lz[k] = k < e.n3 ? e.lam_z[k] + e.sigma : 0.f;
      s_nz[k] = k < e.n3 ? e.null_z[k] : 0;
    }
  const int NS = N / kWideNW, nk = K / 32, half = nk / 2;
  const int slice = blockIdx.x % NS;
  const int cta_rank = blockIdx.x / NS, cta_count = gridDim.x / NS;
  const int mtiles = M / kBlockM;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kWideStages; ++s) {
      mbar_init(&full_bar[s], 1);
      // the converters read the X tile, the MMAs the B planes
      mbar_init(&empty_bar[s], kCvtThreads + 1);
    }
    for (int o = 0; o < kWideSlots; ++o) mbar_init(&cvt_bar[o], kCvtThreads);
    mbar_init(&acc_full, 1);
    mbar_init(&acc_free, kEpiThreads);  // s and h1 read
    mbar_init(&h2_free, kEpiThreads);   // h2 read
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0, s = 0;
      uint32_t ph = 0;
      bool ok = true;
      int pt = cta_rank, pc = 0;
      auto prefetch_next = [&]() {
        if (pt >= mtiles) return;
        tma_prefetch_2d(&tx, pc * 32, pt * kBlockM);
        if (++pc == nk) {
          pc = 0;
          pt += cta_count;
        }
      };
      for (int q = 0; q < kPrefetchAhead; ++q) prefetch_next();
      for (int t = cta_rank; t < mtiles && ok; t += cta_count) {
        for (int c = 0; c < nk; ++c) {
          prefetch_next();
          if (it >= kWideStages && !(ok = mbar_wait(&empty_bar[s], ph ^ 1u, err))) break;
          uint8_t* st = smem + (size_t)s * kWideStage;
          mbar_expect_tx(&full_bar[s], kWideStage);
          tma_load_2d(st, &tx, &full_bar[s], c * 32, t * kBlockM);
          tma_load_2d(st + kWideTile, &tb_hi, &full_bar[s], c * 32, slice * kWideNW);
          tma_load_2d(st + 2 * kWideTile, &tb_lo, &full_bar[s], c * 32, slice * kWideNW);
          ++it;
          if (++s == kWideStages) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = instr_desc(kBlockM, kWideNW, true);
      const uint64_t a0 = smem_desc(smem_u32(smem));
      const uint64_t b0 = smem_desc(smem_u32(smem + kWideTile));
      const uint32_t stage_step = kWideStage >> 4, lo_off = kWideTile >> 4;
      int s = 0, tc = 0;  // ring stage = operand slot
      uint32_t ph = 0;
      bool ok = true;
      for (int t = cta_rank; t < mtiles && ok; t += cta_count, ++tc) {
        const uint32_t prev = (uint32_t)(tc - 1) & 1u;
        if (tc > 0 && !(ok = mbar_wait(&acc_free, prev, err))) break;
        fence_after();
        for (int c = 0; c < nk && ok; ++c) {
          // h2 of the previous tile is read while the first half of K runs
          if (c == half && tc > 0) {
            if (!(ok = mbar_wait(&h2_free, prev, err))) break;
            fence_after();
          }
          if (!(ok = mbar_wait(&full_bar[s], ph, err))) break;
          fence_after();
          const uint64_t bh = b0 + (uint64_t)(s * stage_step), bl = bh + lo_off;
          const uint64_t ah = a0 + (uint64_t)(s * stage_step);
          const uint32_t dh = tmem + (c < half ? kWideH1 : kWideH2), ds = tmem + kWideS;
          const uint32_t acc_h = (c == 0 || c == half) ? 0u : 1u, acc_s = c == 0 ? 0u : 1u;
          // the hi*hi and hi*lo products of the stage need only the landed
          // tile (hi: the FP32 tile itself, read as TF32 by the tensor core),
          // so they go first and keep the tensor pipe busy while the
          // converters form the lo operand
#pragma unroll
          for (int k8 = 0; k8 < 4; ++k8) {
            mma<true>(dh, ah + 2 * k8, bh + 2 * k8, idesc, k8 ? 1u : acc_h);
            mma<true>(ds, ah + 2 * k8, bl + 2 * k8, idesc, k8 ? 1u : acc_s);
          }
          // then lo*hi, from the stage's operand slot once converted
          if (!(ok = mbar_wait(&cvt_bar[s], ph, err))) break;
          fence_after();
          {
            const uint32_t alo = tmem + kWideSlot + (uint32_t)(kWideSlotCols * s);
#pragma unroll
            for (int k8 = 0; k8 < 4; ++k8) mma_tf32_ta(ds, alo + 8 * k8, bh + 2 * k8, idesc, 1u);
          }
          mma_commit(&empty_bar[s]);
          if (++s == kWideStages) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (ok) mma_commit(&acc_full);
      }
    }
  } else if (warp < 2 + kWideEpiWarps) {
    const int q = warp & 3;             // TMEM lane quarter of this warp
    const int part = (warp - 2) >> 2;   // which 64 of the 128 columns
    const int row = q * 32 + lane;
    const uint32_t lanes = static_cast<uint32_t>(q * 32) << 16;
    const int c0 = 64 * part;
    int tc = 0;
    for (int t = cta_rank; t < mtiles; t += cta_count, ++tc) {
      if (!mbar_wait(&acc_full, (uint32_t)tc & 1u, err, 128)) break;
      __syncwarp();
      fence_after();
      const int m = t * kBlockM + row;
      int i = 0, j = 0;
      bool valid = false, nxy = false;
      float lxy = 0.f;
      if (e.kind != 0) {
        i = m % e.P1;
        j = m / e.P1;
        valid = (i < e.n1) && (j < e.n2);
        if (e.kind == 1 && valid) {
          lxy = e.lam_x[i] + e.lam_y[j];
          nxy = e.sigma_null && e.null_x[i] && e.null_y[j];
        }
      }
      // v = (s + h1) + h2, the order of the narrow form.  s and h1 are
      // released first (the next tile writes them from its first K step),
      // h2 after its read (the next tile writes it from the second half)
      float v[64], w[32];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        tmem_load32(tmem + lanes + c0 + 32 * hh + kWideS, v + 32 * hh);
        tmem_load32(tmem + lanes + c0 + 32 * hh + kWideH1, w);
#pragma unroll
        for (int x = 0; x < 32; ++x) v[32 * hh + x] += w[x];
      }
      fence_before();
      mbar_arrive(&acc_free);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        tmem_load32(tmem + lanes + c0 + 32 * hh + kWideH2, w);
#pragma unroll
        for (int x = 0; x < 32; ++x) v[32 * hh + x] += w[x];
      }
      fence_before();
      mbar_arrive(&h2_free);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh)
        epilogue_cols<true>(e, v + 32 * hh, M, m, slice * kWideNW + c0 + 32 * hh, i, j, valid, lxy, nxy,
                            s_lz, s_nz);
    }
  } else {
    // converter warps: as in k_tc_transform<true>, with the X tile at the
    // start of each (wider) ring stage
    const int row = 32 * (warp & 3) + lane;
    const uint32_t lane_base = static_cast<uint32_t>(32 * (warp & 3)) << 16;
    int s = 0;  // ring stage = operand slot
    uint32_t ph = 0;
    bool ok = true;
    for (int t = cta_rank; t < mtiles && ok; t += cta_count) {
      for (int c = 0; c < nk; ++c) {
        if (!(ok = mbar_wait(&full_bar[s], ph, err, 32))) break;
        const float4* rowp =
            reinterpret_cast<const float4*>(smem + (size_t)s * kWideStage + (size_t)row * 128);
        float hi[32], lo[32];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 x = rowp[j ^ (row & 7)];
          hi[4 * j + 0] = x.x;
          hi[4 * j + 1] = x.y;
          hi[4 * j + 2] = x.z;
          hi[4 * j + 3] = x.w;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&empty_bar[s]);
#pragma unroll
        for (int x = 0; x < 32; ++x) lo[x] = tf32_lo(hi[x]);
        // into this stage's operand slot (free: see kWideSlots)
        fence_after();
        tmem_store32(tmem + lane_base + kWideSlot + (uint32_t)(kWideSlotCols * s), lo);
        fence_before();
        mbar_arrive(&cvt_bar[s]);
        if (++s == kWideStages) {
          s = 0;
          ph ^= 1u;
        }
      }
    }
  }
  __syncwarp();
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
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

// 2D map over a row-major rows x cols array of BF16 or FP32, box = one
// 128-byte swizzle row of K values by box_rows rows.
int make_map(CUtensorMap* map, const void* ptr, bool f32, int rows, int cols, int box_rows) {
  const int esz = f32 ? 4 : 2;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * esz};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                        2, const_cast<void*>(ptr), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(MF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return MF_OK;
}

}  // namespace

// BF16: NS = 2 slices from N = 128 (resident B <= 128 KB).  TF32 holds half
// as many K values per byte and three accumulators per set, so it always
// uses 64-column slices (2 x 3 x 64 TMEM columns).
static TcShape shape_for(int N, int K, bool tf32) {
  TcShape sh;
  if (tf32)
    sh.NS = N / 64;
  else
    sh.NS = N >= 128 ? 2 : 1;
  sh.NW = N / sh.NS;
  sh.nk = K / (tf32 ? 32 : 64);
  sh.tiles = tf32 ? 1 : 2;
  const uint32_t budget = 224 * 1024;
  const uint32_t left = sh.b_bytes() < budget ? budget - sh.b_bytes() : 0;
  sh.stages = (int)std::min<uint32_t>(kMaxStages, left / sh.a_stage());
  return sh;
}

int tc_plan_create(TcPlan** out, bool tf32, const void* x_hi, const void* x_lo, const void* b_hi,
                   const void* b_lo, int M, int N, int K) {
  *out = nullptr;
  const int chunk = tf32 ? 32 : 64;
  if (M % kBlockM || K % chunk || N != K || N < 64 || N > 256 || N % 32 ||
      (long long)M * N >= (1LL << 31))
    return set_error(MF_ERR_UNSUPPORTED, "tensor-core transform: unsupported shape M=%d N=%d K=%d", M,
                     N, K);
  if (!tf32 && !x_lo) return set_error(MF_ERR_ARG, "tensor-core transform: missing lo plane");
  for (const void* p : {x_hi, tf32 ? x_hi : x_lo, b_hi, b_lo})
    if (!p || reinterpret_cast<uintptr_t>(p) % 16)
      return set_error(MF_ERR_ARG, "tensor-core transform: operands must be 16-byte aligned");
  int rc = get_encode();
  if (rc) return rc;
  const TcShape sh = shape_for(N, K, tf32);
  if (sh.stages < 2 || sh.NW % 32)
    return set_error(MF_ERR_UNSUPPORTED, "tensor-core transform: no shared-memory plan for N=%d", N);
  TcPlan* p = new TcPlan();
  p->M = M;
  p->N = N;
  p->K = K;
  p->tf32 = tf32;
  if ((rc = make_map(&p->x_hi, x_hi, tf32, M, K, kBlockM)) ||
      (rc = make_map(&p->x_lo, tf32 ? x_hi : x_lo, tf32, M, K, kBlockM)) ||
      (rc = make_map(&p->b_hi, b_hi, tf32, N, K, sh.NW)) ||
      (rc = make_map(&p->b_lo, b_lo, tf32, N, K, sh.NW))) {
    delete p;
    return rc;
  }
  if (tf32 && N % kWideNW == 0) {
    if ((rc = make_map(&p->b_hi_w, b_hi, true, N, K, kWideNW)) ||
        (rc = make_map(&p->b_lo_w, b_lo, true, N, K, kWideNW))) {
      delete p;
      return rc;
    }
    p->wide = true;
  }
  *out = p;
  return MF_OK;
}

void tc_plan_destroy(TcPlan* p) { delete p; }

template <bool kTf32>
static int launch(const TcPlan* p, const TcEpilogue& e, int* dev_err, cudaStream_t st) {
  const TcShape sh = shape_for(p->N, p->K, kTf32);
  static int num_sms = 0;
  if (!num_sms) {
    int dev = 0;
    MF_CUDA(cudaGetDevice(&dev));
    MF_CUDA(cudaFuncSetAttribute(k_tc_transform<kTf32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 224 * 1024 + 1024));
    int sms = 0;
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    num_sms = sms;
  }
  const int mtiles = p->M / kBlockM;
  const int grid = std::min(num_sms / sh.NS, mtiles) * sh.NS;
  k_tc_transform<kTf32><<<grid, Cfg<kTf32>::kThreads, sh.smem(), st>>>(
      p->x_hi, p->x_lo, p->b_hi, p->b_lo, p->M, sh, e, dev_err);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static int launch_wide(const TcPlan* p, const TcEpilogue& e, int* dev_err, cudaStream_t st) {
  static int num_sms = 0;
  if (!num_sms) {
    int dev = 0;
    MF_CUDA(cudaGetDevice(&dev));
    MF_CUDA(cudaFuncSetAttribute(k_tc_tf32_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWideSmem));
    int sms = 0;
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    num_sms = sms;
  }
  const int NS = p->N / kWideNW;
  const int mtiles = p->M / kBlockM;
  const int grid = std::min(num_sms / NS, mtiles) * NS;
  k_tc_tf32_wide<<<grid, kWideThreads, kWideSmem, st>>>(p->x_hi, p->b_hi_w, p->b_lo_w, p->M, p->N,
                                                         p->K, e, dev_err);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

bool tc_has_wide(const TcPlan* p) { return p->tf32 && p->wide; }

int tc_transform(const TcPlan* p, const TcEpilogue& e, int* dev_err, cudaStream_t st, int plan) {
  if (p->tf32 ? !e.y32 && e.kind != 2 : (!e.y_hi || !e.y_lo) && e.kind != 2)
    return set_error(MF_ERR_ARG, "tensor-core transform: output does not match the operand format");
  if (plan == 0) plan = g_tf32_plan;
  if (p->tf32 && p->wide && plan != 1) return launch_wide(p, e, dev_err, st);
  return p->tf32 ? launch<true>(p, e, dev_err, st) : launch<false>(p, e, dev_err, st);
}

}  // namespace mf

extern "C" {

int mf_tc_tf32_plan_set(int plan) {
  if (plan < 0 || plan > 2) return mf::set_error(MF_ERR_ARG, "mf_tc_tf32_plan_set: plan must be 0, 1 or 2");
  mf::tc_set_tf32_plan(plan);
  return MF_OK;
}

int mf_tc_tf32_plan_get(void) { return mf::tc_get_tf32_plan(); }

}  // extern "C"
