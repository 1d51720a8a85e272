// Matrix-diagonalisation Poisson/Helmholtz solver on GB300.
//
// Reference path: solver_3d (class_field.f90:1072-1109) -> solve_3d
// (class_solver_3d.f90:83-299): boundary fold, three forward eigenvector
// transforms (dgx/dgy/dgz with V^-1), eigenvalue divide, three inverse
// transforms (with V), interior copy and boundary insertion / Neumann
// extrapolation.
//
// Layout.  Each transform contracts the axis that is contiguous in memory
// and writes its output with the axes rotated, Y[n][m] with m contiguous,
// so that the next axis to contract is contiguous again:
//   (i,j,k) -x-> (j,k,i') -y-> (k,i',j') -z-> (i',j',k')
// After three transforms the array is back in the reference's x-fastest
// order, every transform is a plain "X[m][k] times B^T" product with both
// operands K-major, and every store is coalesced along m.
//
// Plain path (MF_PREC_FP64): FP64 DFMA tiles; GB300's FP64 pipe bounds it.
// Mixed path: the six transforms run on tcgen05 (mf_tc.cu) as split-BF16
// three-product GEMMs into FP32 TMEM accumulators, with the eigenvalue
// divide fused into the third transform's epilogue and the solution update
// into the sixth's; iterative refinement recomputes the residual in FP64
// with the solver's own compact operator (pentalu factors of ddl and the
// 8-wide ddr), so the refined result converges to the FP64 solution.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "mf_line.cuh"
#include "mf_setup.h"
#include "mf_solver.h"

namespace mf {

// Null-mode threshold of the eigen divide: the reference compares with the
// default-kind literal 1e-11 (class_solver_3d.f90:207-208).
static const double kNullThresh = (double)1e-11f;

struct AxisDev {
  int n = 0, P = 0;
  int bc[2] = {1, 1};
  double bcc[4] = {0, 0, 0, 0};  // ddr(1,1), ddr(2,1), ddr(n-1,8), ddr(n,7)
  double neum[14] = {0};
  DevBuf V, Vinv, eig, invl4, rows;           // FP64
  DevBuf Vh, Vl, Vih, Vil, eigf, nullf;       // mixed path (padded P x P)
  DevBuf Vh32, Vl32, Vih32, Vil32;             // 3xTF32 planes (FP32, padded P x P)
  DevBuf invl4f;                               // FP32 copy of invl4
  DevBuf rowsf;                                // FP32 copy of rows
  DevBuf tri;                                  // TriRow[n] when the lhs is tridiagonal
  DevBuf trib;                                 // bottom table of the two-sided sweeps (TriRow[n-1-(n-1)/2])
  bool tri_ok = false;
  // Null mode (the one eigenvalue below the threshold, when there is exactly
  // one; -1 otherwise): row null_idx of V^-1 and column null_idx of V (FP64)
  int null_idx = -1;
  DevBuf null_row, null_col;
};

}  // namespace mf

using namespace mf;

// Staging slots of mf_solve_3d_mixed_many: with three, the upload of a
// problem need not wait for the download of the one two places before it
// (the host link carries both directions at once).
constexpr int kPipeSlots = 3;

struct mf_solver3d {
  AxisDev ax[3];
  int n[3] = {0, 0, 0};
  int P[3] = {0, 0, 0};
  DevBuf w0, w1;                               // FP64 work arrays (plain path)
  DevBuf st_rhs, st_solf, st_bc[3];            // host staging
  // mf_solve_3d_mixed_many: kPipeSlots staging slots, copy-in/out streams, events
  DevBuf pipe_rhs[kPipeSlots], pipe_solf[kPipeSlots], pipe_bc[kPipeSlots][3];
  cudaStream_t cin = nullptr, cout = nullptr;
  cudaEvent_t in_ready[kPipeSlots] = {}, solved[kPipeSlots] = {}, out_done[kPipeSlots] = {};
  // ... and per slot a CUDA graph of the mixed solve on that slot's buffers,
  // with the settings it was captured under
  struct PipeGraph {
    cudaGraphExec_t exec = nullptr;
    double sigma = 0.0;
    int precision = -1, refine = -1, plan = -1, tune = -1, resid = -1;
  } pipe_graph[kPipeSlots];
  cudaStream_t gcap = nullptr;  // capture stream of those graphs
  DevBuf R, R2;                                // FP64 scratch of the residual
  DevBuf nullpart;                             // null-mode projection: partial sums, coefficient
  DevBuf R1d;                                  // closed operators: FP64 r1 of the refinement
  DevBuf U32, C32, R1f;                        // mixed path: u1, correction, r1 (FP32)
  DevBuf Xa_hi, Xa_lo, Xb_hi, Xb_lo;           // split-BF16 planes
  DevBuf Xa32, Xb32;                           // 3xTF32 operands (FP32)
  DevBuf err;                                  // device error flag (int)
  DevBuf foldf;                                // FP32 c*bc face products (mixed path)
  TcPlan* plan[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  TcPlan* plan32[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  bool mixed_ready = false, mixed32_ready = false;
  int resid_mode = MF_RESID_FP64;             // residual arithmetic of the mixed path
  StageProfiler prof;
};

namespace mf {

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// rhs minus the boundary folds inv_lhs(:,{1,2,n-1,n}) * (ddr_bc * bc)
// (class_solver_3d.f90:104-175), x then y then z like the reference.
struct FoldArgs {
  const double* ix[4];
  const double* iy[4];
  const double* iz[4];
  double cx[4], cy[4], cz[4];
};

// Batched solves: problem blockIdx.y at the given element strides (0 = shared).
struct FoldBatch {
  long long rhs = 0, out = 0, bc[3] = {0, 0, 0};
};

__global__ void k_fold(const double* __restrict__ rhs, double* __restrict__ out,
                       const double* __restrict__ bcx, const double* __restrict__ bcy,
                       const double* __restrict__ bcz, FoldArgs a, int n1, int n2, int n3,
                       FoldBatch fb = FoldBatch()) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)n1 * n2 * n3;
  if (idx >= tot) return;
  rhs += blockIdx.y * fb.rhs;
  out += blockIdx.y * fb.out;
  bcx += blockIdx.y * fb.bc[0];
  bcy += blockIdx.y * fb.bc[1];
  bcz += blockIdx.y * fb.bc[2];
  const int i = (int)(idx % n1);
  const long long jk = idx / n1;
  const int j = (int)(jk % n2), k = (int)(jk / n2);
  double r = rhs[idx];
  {
    const double bl = bcx[j + (long long)n2 * k], bh = bcx[j + (long long)n2 * k + (long long)n2 * n3];
    r = r - a.ix[0][i] * (a.cx[0] * bl) - a.ix[1][i] * (a.cx[1] * bl) - a.ix[2][i] * (a.cx[2] * bh) -
        a.ix[3][i] * (a.cx[3] * bh);
  }
  {
    const double bl = bcy[i + (long long)n1 * k], bh = bcy[i + (long long)n1 * k + (long long)n1 * n3];
    r = r - a.iy[0][j] * (a.cy[0] * bl) - a.iy[1][j] * (a.cy[1] * bl) - a.iy[2][j] * (a.cy[2] * bh) -
        a.iy[3][j] * (a.cy[3] * bh);
  }
  {
    const double bl = bcz[i + (long long)n1 * j], bh = bcz[i + (long long)n1 * j + (long long)n1 * n2];
    r = r - a.iz[0][k] * (a.cz[0] * bl) - a.iz[1][k] * (a.cz[1] * bl) - a.iz[2][k] * (a.cz[2] * bh) -
        a.iz[3][k] * (a.cz[3] * bh);
  }
  out[idx] = r;
}

// FP64 transform Y[n][m] = sum_k A[n][k] X[m][k]  (A row-major N x K).
// Epilogues: 0 plain store; 1 eigenvalue divide (m = i + n1*j, n = k);
// 2 store into the interior of solf(0:n1+1,0:n2+1,0:n3+1).
struct GemmEpi {
  int kind = 0;
  const double* lx = nullptr;
  const double* ly = nullptr;
  const double* lz = nullptr;
  double sigma = 0.0, thresh = 0.0;
  int n1 = 0, n2 = 0;
};

constexpr int GBK = 16;

// BT x BT output tile per 256-thread CTA, (BT/16)^2 outputs per thread.  The
// FP64 pipe (about two DFMA per clock per SM) bounds this kernel at every
// size, so the tile only decides how evenly the work spreads over the SMs:
// 64 for large transforms, 32 when 64-wide tiles would leave SMs idle.
template <int BT>
__global__ void __launch_bounds__(256) k_gemm_f64(const double* __restrict__ X, int M, int K,
                                                  const double* __restrict__ A, int N,
                                                  double* __restrict__ Y, GemmEpi e, long long xs = 0,
                                                  long long ys = 0) {
  // batched solves: problem blockIdx.z at X + z xs, Y + z ys
  X += blockIdx.z * xs;
  Y += blockIdx.z * ys;
  constexpr int R = BT / 16;
  __shared__ double Xs[GBK][BT + 1];
  __shared__ double As[GBK][BT + 1];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  const long long m0 = (long long)blockIdx.x * BT;
  const int n0 = blockIdx.y * BT;
  double acc[R][R];
#pragma unroll
  for (int b = 0; b < R; ++b)
#pragma unroll
    for (int a = 0; a < R; ++a) acc[b][a] = 0.0;
  for (int k0 = 0; k0 < K; k0 += GBK) {
#pragma unroll
    for (int r = 0; r < (BT * GBK) / 256; ++r) {
      const int id = t + 256 * r;
      const int row = id / GBK, kk = id % GBK;
      const long long m = m0 + row;
      const int k = k0 + kk;
      Xs[kk][row] = (m < M && k < K) ? X[m * K + k] : 0.0;
      const int nn = n0 + row;
      As[kk][row] = (nn < N && k < K) ? A[(long long)nn * K + k] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      double xa[R], ab[R];
#pragma unroll
      for (int a = 0; a < R; ++a) xa[a] = Xs[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < R; ++b) ab[b] = As[kk][ty + 16 * b];
#pragma unroll
      for (int b = 0; b < R; ++b)
#pragma unroll
        for (int a = 0; a < R; ++a) acc[b][a] = fma(ab[b], xa[a], acc[b][a]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < R; ++b) {
    const int n = n0 + ty + 16 * b;
    if (n >= N) continue;
#pragma unroll
    for (int a = 0; a < R; ++a) {
      const long long m = m0 + tx + 16 * a;
      if (m >= M) continue;
      double v = acc[b][a];
      if (e.kind == 0) {
        Y[(long long)n * M + m] = v;
      } else {
        const int i = (int)(m % e.n1), j = (int)(m / e.n1);
        if (e.kind == 1) {
          const double lx = e.lx[i], ly = e.ly[j], lz = e.lz[n];
          const double big = fmax(fmax(fmax(fabs(e.sigma), fabs(lx)), fabs(ly)), fabs(lz));
          Y[(long long)n * M + m] = (big < e.thresh) ? 0.0 : v / (((lx + ly) + lz) + e.sigma);
        } else {
          const long long p1 = e.n1 + 2, p2 = e.n2 + 2;
          Y[(i + 1) + p1 * ((j + 1) + p2 * (long long)(n + 1))] = v;
        }
      }
    }
  }
}

// Boundary faces of solf: Dirichlet copy or 7-point Neumann extrapolation
// (class_solver_3d.f90:263-297, extrapolation_neum_{x,y,z} :658-776).
struct FaceArgs {
  long long sA, sa, sb;  // strides along the axis and the two face directions
  int n, na, nb;         // interior count along the axis, face extents
  int bc0, bc1;
  double nl[7], nr[7];
};

__global__ void k_faces(double* solf, const double* __restrict__ bc, FaceArgs f, long long s_solf = 0,
                        long long s_bc = 0) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)f.na * f.nb) return;
  solf += blockIdx.y * s_solf;  // batched solves: problem blockIdx.y
  bc += blockIdx.y * s_bc;
  const int a = (int)(t % f.na), b = (int)(t / f.na);
  double* p = solf + (a + 1) * f.sa + (b + 1) * f.sb;  // ghost-left node of this line
  const double blo = bc[t], bhi = bc[t + (long long)f.na * f.nb];
  if (f.bc0 == 1) {
    p[0] = blo;
  } else {
    double acc = blo;
    for (int m = 1; m < 7; ++m) acc = acc - f.nl[m] * p[m * f.sA];
    p[0] = acc * (1.0 / f.nl[0]);
  }
  const long long last = (long long)(f.n + 1) * f.sA;
  if (f.bc1 == 1) {
    p[last] = bhi;
  } else {
    double acc = bhi;
    for (int m = 5; m >= 0; --m) acc = acc - f.nr[m] * p[(long long)(f.n - 5 + m) * f.sA];
    p[last] = acc * (1.0 / f.nr[6]);
  }
}

// ---- residuals of the iterative refinement
//
// r = rin - sigma*u - (Lx + Ly + Lz) u, boundary data included, in three
// passes with one thread per line; lines are numbered so that a warp covers
// 32 neighbouring lines.  For y and z every step of the recurrence is then a
// coalesced access; for x the 32 lines are 4-8*n1 bytes apart and each
// thread walks its own cache lines, which stay in L1 while it consumes them.
// Many resident warps hide the latency of the dependent chains.
// T is the arithmetic type (double: the residual of the first approximate
// solution u1; float: the residual update r1 - A*C of the accumulated
// correction C), In the storage type of the differentiated array.
// The forward-elimination values go to a scratch array; the final store:
//   mode 0 (first pass):  out = rin - sigma*u - L u
//   mode 1 (middle pass): out = rin - L u
//   mode 2 (last pass):   rin - L u in the padded (P1,P2,P3) layout of the
//                         tensor-core transforms: split-BF16 planes, or FP32
//                         (x32) for the 3xTF32 transforms
//   mode 3 (last pass):   mode 2, and rin - L u also stored as FP32 (r32).
template <class T, class In>
struct ResidFin {
  int mode;
  const T* rin;          // offset to the line
  const In* u;           // mode 0, offset to the line
  T sigma;
  T* out;                // modes 0,1: result array, offset to the line
  __nv_bfloat16* hi;     // modes 2,3: planes, offset to the line's padded base
  __nv_bfloat16* lo;
  float* x32;            // modes 2,3 (3xTF32): FP32 operand, same offsets
  long long pstride;     // modes 2,3: padded stride along the line
  float* r32;            // mode 3: offset to the line
  __device__ __forceinline__ void operator()(T*, int i, long long idx, T y) const {
    put(i, idx, y, rin[idx], mode == 0 ? load_as<T, In>(u, idx) : T(0));
  }
  // Final store of row i with the row's rin (and, mode 0, u) value given.
  __device__ __forceinline__ void put(int i, long long idx, T y, T r, T uv) const {
    if (mode == 0) {
      // at sigma = 0 the same value without the product (and u is not loaded)
      out[idx] = sigma != T(0) ? r - sigma * uv - y : r - y;
    } else if (mode == 1) {
      out[idx] = r - y;
    } else {
      float v;
      if constexpr (sizeof(T) == 8)
        v = narrow(r - y);
      else
        v = r - y;
      if (x32) {
        x32[i * pstride] = v;
      } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i * pstride] = h;
        lo[i * pstride] = __float2bfloat16_rn(v - __bfloat162float(h));
      }
      if (mode == 3) r32[idx] = v;
    }
  }
};

template <class T>
struct ResidPass {
  const T* rows;       // packed operator rows of this axis
  int n;               // line length
  int na, nb;          // line grid
  long long sa, sb, s; // strides of the line grid and along the line
  const double* bc;    // bc(na, nb, 2), or null for homogeneous data
  double4 bcc;
  int mode;
  T sigma;
  long long pa, pb, pstride;  // modes 2,3: padded strides of (a, b) and along the line
};

template <class T, class In>
__global__ void __launch_bounds__(128) k_resid_lines(ResidPass<T> p, const In* u, const T* rin,
                                                     T* scratch, T* rout, __nv_bfloat16* hi,
                                                     __nv_bfloat16* lo, float* x32, float* r32) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)p.na * p.nb) return;
  const int a = (int)(t % p.na), b = (int)(t / p.na);
  const long long base = a * p.sa + b * p.sb;
  LineBCT<T> lb;
  if (p.bc) {
    lb.lo = (T)p.bc[t];
    lb.hi = (T)p.bc[t + (long long)p.na * p.nb];
    lb.c0 = (T)p.bcc.x; lb.c1 = (T)p.bcc.y; lb.c2 = (T)p.bcc.z; lb.c3 = (T)p.bcc.w;
  }
  ResidFin<T, In> fin;
  fin.mode = p.mode;
  fin.rin = rin + base;
  fin.u = u + base;
  fin.sigma = p.sigma;
  fin.out = rout ? rout + base : nullptr;
  const long long pbase = a * p.pa + b * p.pb;
  fin.hi = hi ? hi + pbase : nullptr;
  fin.lo = lo ? lo + pbase : nullptr;
  fin.x32 = x32 ? x32 + pbase : nullptr;
  fin.pstride = p.pstride;
  fin.r32 = r32 ? r32 + base : nullptr;
  if constexpr (sizeof(T) == 4)
    solve_line_comp(p.rows, p.n, u + base, scratch + base, p.s, fin);
  else
    solve_line(p.rows, p.n, u + base, scratch + base, p.s, lb, fin);
}

// ---- residual of an FP32 iterate with a tridiagonal operator (moment form)
//
// The solver's second-derivative operator has a tridiagonal implicit part
// (p = e = alpha = beta = 0 in its factors) and a 5-point explicit stencil
// inside the line.  With 1/c_i folded into the rows,
//   x~_i = S_i - ft_i x~_{i-1},   y_i = x~_i - dt_i y_{i+1},
//   S_i  = sum_m (r_m/c_i) u_{j_m} + (cbc/c_i) bc,
// which costs one FP64 FMA per sweep.  S_i is where FP64 loses its digits:
// on smooth data its terms are ~1e5 times the result.  For an FP32 iterate
// u it is evaluated in the moment form
//   S_i = sum_m r~_m (u_{j_m} - u_i) + cbc~ (bc - u_i) + rho_i u_i,
//   rho_i = sum_m r~_m + cbc~   (exact sum of the FP64 coefficients),
// an identity of exact arithmetic.  The differences of FP32 values are
// exact as two floats, their products with the coefficients (hi + lo
// floats) are formed with FMA error terms and summed with TwoSum, so the
// remaining cancellation (~1e2) meets ~2^-48 relative rounding: the result
// is more accurate than the FP64 evaluation of the same sum, and only the
// two sweeps and the final combination use the FP64 pipe.
struct TriRow {
  float wh[7], wl[7];  // r_m / c_i as hi + lo floats, stencil order of the packed rows
  float rh, rl;        // rho_i as hi + lo floats
  double ft, dt;       // f_i c_{i-1} / c_i,  d_i / c_i
  double cbc;          // boundary coefficient / c_i (rows 0, 1, n-2, n-1)
  double tw;           // twist row of the two-sided sweeps: 1 / (1 - dt_m et_{m+1})
  float fth, ftl, dth, dtl, cbh, cbl;  // ft, dt, cbc as hi + lo floats
  float pad2[2];
};
static_assert(sizeof(TriRow) == 128, "TriRow layout");

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// ---- double-FP32 ("float-float") arithmetic: a value is h + l with
// |l| <= ulp(h)/2; sums by TwoSum, products by the FMA error term
// (Dekker, Knuth).  About 2^-48 relative rounding per operation.
struct FF {
  float h, l;
};

__device__ __forceinline__ FF ff_norm(float s, float e) {  // |s| >= |e|
  const float h = s + e;
  return {h, e - (h - s)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return ff_norm(s, e + (a.l + b.l));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.h, -a.l}; }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
  const float p = a.h * b;
  float e = fmaf(a.h, b, -p);
  e = fmaf(a.l, b, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ float ff_to_float(FF a) { return a.h + a.l; }

// 2^k as a float for -126 <= k <= 127 (0 below, infinity above).
__device__ __forceinline__ float pow2f(int k) {
  if (k < -126) return 0.f;
  if (k > 127) return __uint_as_float(0x7F800000u);
  return __uint_as_float((uint32_t)(k + 127) << 23);
}

// Exact split of a double into h + l with integer operations: h holds the
// leading 24 mantissa bits (rounded), l the signed remainder (rounded to
// 24 bits, so the pair carries ~48 bits).  Values outside the normal FP32
// range flush to zero.
__device__ __forceinline__ FF ff_from_double(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return {0.f, 0.f};
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const uint32_t hm = (uint32_t)((m + (1ull << 28)) >> 29);      // <= 2^24
  const long long rem = (long long)m - ((long long)hm << 29);    // |rem| <= 2^28
  const float sc = pow2f(e - 1075);                               // 2^(e - 1023 - 52)
  float h = __uint2float_rn(hm) * (sc * 536870912.f);             // 2^29
  float l = __int2float_rn((int)rem) * sc;
  if (b >> 63) {
    h = -h;
    l = -l;
  }
  return {h, l};
}



// sum_{m < W, m != skip} (wh + wl)_m (v_m - ref) + rho ref, as FP64.
template <int W>
__device__ __forceinline__ double moment_sum(const TriRow& r, const float (&v)[W], float ref,
                                             int skip) {
  float h = 0.f, l = 0.f;
#pragma unroll
  for (int m = 0; m < W; ++m) {
    if (m == skip) continue;
    float dh, dl;
    two_sum(v[m], -ref, dh, dl);
    const float ph = r.wh[m] * dh;
    float pl = fmaf(r.wh[m], dh, -ph);
    pl = fmaf(r.wh[m], dl, pl);
    pl = fmaf(r.wl[m], dh, pl);
    float sh, se;
    two_sum(h, ph, sh, se);
    h = sh;
    l += se + pl;
  }
  const float ph = r.rh * ref;
  float pl = fmaf(r.rh, ref, -ph);
  pl = fmaf(r.rl, ref, pl);
  float sh, se;
  two_sum(h, ph, sh, se);
  return widen(sh) + widen(l + se + pl);
}

// xs holds the forward values of this line at stride xq (s, or the number of
// lines when they are stored row-major across lines)
__device__ __forceinline__ void solve_line_tri(const TriRow* __restrict__ R, int n, const float* u,
                                               double* xs, long long s, long long xq, double lo,
                                               double hi, const ResidFin<double, float>& fin) {
  float f[7], g[7];
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    f[m] = u[(long long)m * s];
    g[m] = u[(long long)(n - 7 + m) * s];
  }
  // rows 0 and 1: 7-wide stencils on u_0..u_6, boundary value lo
  double x0 = moment_sum<7>(R[0], f, f[0], 0) + R[0].cbc * (lo - widen(f[0]));
  double x1 = moment_sum<7>(R[1], f, f[1], 1) + R[1].cbc * (lo - widen(f[1])) - R[1].ft * x0;
  xs[0] = x0;
  xs[xq] = x1;
  double xm = x1;
  float w[5] = {f[0], f[1], f[2], f[3], f[4]};
  // interior rows 2..n-3; pf[k] = u(i + 3 + k)
  float pf[kAhead];
#pragma unroll
  for (int k = 0; k < kAhead; ++k) pf[k] = (5 + k < n) ? u[(long long)(5 + k) * s] : 0.f;
  int i = 2;
  for (; i + kAhead <= n - 2; i += kAhead) {
    float nb[kAhead];
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const int j = i + 3 + kAhead + k;
      nb[k] = (j < n) ? u[(long long)j * s] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const TriRow& r = R[i + k];
      const double x = moment_sum<5>(r, w, w[2], 2) - r.ft * xm;
      xs[(long long)(i + k) * xq] = x;
      xm = x;
      w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4]; w[4] = pf[k];
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) pf[k] = nb[k];
  }
  for (; i < n - 2; ++i) {
    const TriRow& r = R[i];
    const double x = moment_sum<5>(r, w, w[2], 2) - r.ft * xm;
    xs[(long long)i * xq] = x;
    xm = x;
    w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
    if (i + 3 < n) w[4] = u[(long long)(i + 3) * s];
  }
  // rows n-2 and n-1: 7-wide stencils on u_{n-7}..u_{n-1}, boundary value hi
  const TriRow& rA = R[n - 2];
  const TriRow& rB = R[n - 1];
  const double xA = moment_sum<7>(rA, g, g[5], 5) + rA.cbc * (hi - widen(g[5])) - rA.ft * xm;
  const double xB = moment_sum<7>(rB, g, g[6], 6) + rB.cbc * (hi - widen(g[6])) - rB.ft * xA;
  // back substitution with the final combination of each row; the forward
  // value, rin and (first pass) u of row i - k are loaded kAhead rows ahead
  const bool need_u = fin.mode == 0 && fin.sigma != 0.0;  // u enters only through sigma u
  auto uval = [&](long long o) { return need_u ? widen(fin.u[o]) : 0.0; };
  double y1 = xB;
  fin.put(n - 1, (long long)(n - 1) * s, xB, fin.rin[(long long)(n - 1) * s], uval((long long)(n - 1) * s));
  double y = xA - rA.dt * y1;
  fin.put(n - 2, (long long)(n - 2) * s, y, fin.rin[(long long)(n - 2) * s], uval((long long)(n - 2) * s));
  y1 = y;
  i = n - 3;
  double rb[kAhead], rr[kAhead];
  float ru[kAhead];
#pragma unroll
  for (int k = 0; k < kAhead; ++k) {
    const bool in = i - k >= 0;
    const long long o = (long long)(i - k) * s;
    rb[k] = in ? xs[(long long)(i - k) * xq] : 0.0;
    rr[k] = in ? fin.rin[o] : 0.0;
    ru[k] = (in && need_u) ? fin.u[o] : 0.f;
  }
  for (; i - (kAhead - 1) >= 0; i -= kAhead) {
    double nb[kAhead], nr[kAhead];
    float nu[kAhead];
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const int j = i - kAhead - k;
      const long long o = (long long)j * s;
      nb[k] = (j >= 0) ? xs[(long long)j * xq] : 0.0;
      nr[k] = (j >= 0) ? fin.rin[o] : 0.0;
      nu[k] = (j >= 0 && need_u) ? fin.u[o] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const double yy = rb[k] - R[i - k].dt * y1;
      fin.put(i - k, (long long)(i - k) * s, yy, rr[k], widen(ru[k]));
      y1 = yy;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      rb[k] = nb[k];
      rr[k] = nr[k];
      ru[k] = nu[k];
    }
  }
  for (; i >= 0; --i) {
    const long long o = (long long)i * s;
    const double yy = xs[(long long)i * xq] - R[i].dt * y1;
    fin.put(i, o, yy, fin.rin[o], uval(o));
    y1 = yy;
  }
}

__global__ void __launch_bounds__(128) k_resid_tri(ResidPass<double> p, const TriRow* __restrict__ R,
                                                   const float* u, const double* rin, double* scratch,
                                                   long long xq, double* rout, __nv_bfloat16* hi,
                                                   __nv_bfloat16* lo, float* x32, float* r32) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)p.na * p.nb) return;
  const int a = (int)(t % p.na), b = (int)(t / p.na);
  const long long base = a * p.sa + b * p.sb;
  double blo = 0.0, bhi = 0.0;
  if (p.bc) {
    blo = p.bc[t];
    bhi = p.bc[t + (long long)p.na * p.nb];
  }
  ResidFin<double, float> fin;
  fin.mode = p.mode;
  fin.rin = rin + base;
  fin.u = u + base;
  fin.sigma = p.sigma;
  fin.out = rout ? rout + base : nullptr;
  const long long pbase = a * p.pa + b * p.pb;
  fin.hi = hi ? hi + pbase : nullptr;
  fin.lo = lo ? lo + pbase : nullptr;
  fin.x32 = x32 ? x32 + pbase : nullptr;
  fin.pstride = p.pstride;
  fin.r32 = r32 ? r32 + base : nullptr;
  // xq != 0: the forward values go to a separate scratch array, row i of
  // line t at i * xq + t, so a warp's 32 lines touch consecutive addresses
  if (xq)
    solve_line_tri(R, p.n, u + base, scratch + t, p.s, xq, blo, bhi, fin);
  else
    solve_line_tri(R, p.n, u + base, scratch + base, p.s, p.s, blo, bhi, fin);
}

// ---- the same residual with two lanes per line (twisted factorisation)
//
// With T = L U (L unit lower bidiagonal, sub ft; U unit upper bidiagonal,
// super dt) the sweeps solve T y = S.  One lane eliminates rows 0..m from
// the top as above (x_i = S_i - ft_i x_{i-1}); its partner eliminates rows
// n-1..m+1 from the bottom with the U L factors of the same T
// (z_i = S_i / q_i - gt_i z_{i+1}, pivots q_i, gt_i = T_{i,i+1} / q_i,
// et_i = T_{i,i-1} / q_i), each on half the line.  At the twist the two
// meet: y_m = tw (x_m - dt_m z_{m+1}), y_{m+1} = tw (z_{m+1} - et_{m+1} x_m),
// tw = 1 / (1 - dt_m et_{m+1}); then each lane substitutes back over its
// own half (y_i = x_i - dt_i y_{i+1} upwards, y_i = z_i - et_i y_{i-1}
// downwards).  The bottom lane reads the line mirrored (negative stride)
// with a table stored in that order (weights reversed and scaled by 1/q_i,
// gt in `ft`, et in `dt`), so both lanes of a warp run the same
// instructions: the dependent chain is half as long and the pass has twice
// the warps of one thread per line, for the same FP64 work.  A warp holds
// 16 lines: lanes 0-15 the top halves, lanes 16-31 the bottom halves.
constexpr int kTw = 4;   // rows loaded ahead in the forward elimination of the two-sided sweeps
constexpr int kTwB = 2;  // ... and in their back substitution

__device__ __forceinline__ void solve_line_twist(const TriRow* __restrict__ R, int n, int cnt,
                                                 const float* u, double* xs, long long s, long long xq,
                                                 double bcv, const ResidFin<double, float>& fin,
                                                 unsigned mask) {
  float f[7];
#pragma unroll
  for (int m = 0; m < 7; ++m) f[m] = u[(long long)m * s];
  // rows 0 and 1 of this side: 7-wide stencils on its first seven nodes
  double x0 = moment_sum<7>(R[0], f, f[0], 0) + R[0].cbc * (bcv - widen(f[0]));
  double x1 = moment_sum<7>(R[1], f, f[1], 1) + R[1].cbc * (bcv - widen(f[1])) - R[1].ft * x0;
  xs[0] = x0;
  xs[xq] = x1;
  double xm = x1;
  float w[5] = {f[0], f[1], f[2], f[3], f[4]};
  float pf[kTw];  // pf[k] = u(i + 3 + k)
#pragma unroll
  for (int k = 0; k < kTw; ++k) pf[k] = (5 + k < 7) ? f[5 + k] : (5 + k < n) ? u[(long long)(5 + k) * s] : 0.f;
  int i = 2;
  for (; i + kTw <= cnt; i += kTw) {
    float nb[kTw];
#pragma unroll
    for (int k = 0; k < kTw; ++k) {
      const int j = i + 3 + kTw + k;
      nb[k] = (j < n) ? u[(long long)j * s] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kTw; ++k) {
      const TriRow& r = R[i + k];
      const double x = moment_sum<5>(r, w, w[2], 2) - r.ft * xm;
      xs[(long long)(i + k) * xq] = x;
      xm = x;
      w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4]; w[4] = pf[k];
    }
#pragma unroll
    for (int k = 0; k < kTw; ++k) pf[k] = nb[k];
  }
  for (; i < cnt; ++i) {
    const TriRow& r = R[i];
    const double x = moment_sum<5>(r, w, w[2], 2) - r.ft * xm;
    xs[(long long)i * xq] = x;
    xm = x;
    w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
    if (i + 3 < n) w[4] = u[(long long)(i + 3) * s];
  }
  // the twist: this side's last eliminated value and the partner's
  const double other = __shfl_xor_sync(mask, xm, 16);
  const bool need_u = fin.mode == 0 && fin.sigma != 0.0;  // u enters only through sigma u
  auto uval = [&](long long o) { return need_u ? widen(fin.u[o]) : 0.0; };
  i = cnt - 1;
  const TriRow& rt = R[i];
  double y1 = rt.tw * (xm - rt.dt * other);
  fin.put(i, (long long)i * s, y1, fin.rin[(long long)i * s], uval((long long)i * s));
  // back substitution over this side's rows cnt-2..0, loads kTwB rows ahead
  i = cnt - 2;
  double rb[kTwB], rr[kTwB];
  float ru[kTwB];
#pragma unroll
  for (int k = 0; k < kTwB; ++k) {
    const bool in = i - k >= 0;
    const long long o = (long long)(i - k) * s;
    rb[k] = in ? xs[(long long)(i - k) * xq] : 0.0;
    rr[k] = in ? fin.rin[o] : 0.0;
    ru[k] = (in && need_u) ? fin.u[o] : 0.f;
  }
  for (; i - (kTwB - 1) >= 0; i -= kTwB) {
    double nb[kTwB], nr[kTwB];
    float nu[kTwB];
#pragma unroll
    for (int k = 0; k < kTwB; ++k) {
      const int j = i - kTwB - k;
      const long long o = (long long)j * s;
      nb[k] = (j >= 0) ? xs[(long long)j * xq] : 0.0;
      nr[k] = (j >= 0) ? fin.rin[o] : 0.0;
      nu[k] = (j >= 0 && need_u) ? fin.u[o] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kTwB; ++k) {
      const double yy = rb[k] - R[i - k].dt * y1;
      fin.put(i - k, (long long)(i - k) * s, yy, rr[k], widen(ru[k]));
      y1 = yy;
    }
#pragma unroll
    for (int k = 0; k < kTwB; ++k) {
      rb[k] = nb[k];
      rr[k] = nr[k];
      ru[k] = nu[k];
    }
  }
  for (; i >= 0; --i) {
    const long long o = (long long)i * s;
    const double yy = xs[(long long)i * xq] - R[i].dt * y1;
    fin.put(i, o, yy, fin.rin[o], uval(o));
    y1 = yy;
  }
}

// Rt: the top table (TriRow[n], rows 0..m used); Rb: the bottom table in
// mirrored order (TriRow[n - 1 - m], entry k = row n-1-k); m = (n-1)/2.
template <int MODE>
__global__ void __launch_bounds__(128) k_resid_twist(ResidPass<double> p, const TriRow* __restrict__ Rt,
                                                     const TriRow* __restrict__ Rb, const float* u,
                                                     const double* rin, double* scratch, long long xq,
                                                     double* rout, __nv_bfloat16* hi, __nv_bfloat16* lo,
                                                     float* x32, float* r32) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool top = lane < 16;
  const long long lines = (long long)p.na * p.nb;
  const long long t = (g >> 5) * 16 + (lane & 15);
  const bool valid = t < lines;
  const unsigned mask = __ballot_sync(0xffffffffu, valid);  // both lanes of a line agree
  if (!valid) return;
  const int a = (int)(t % p.na), b = (int)(t / p.na);
  const int m = (p.n - 1) >> 1;
  const int cnt = top ? m + 1 : p.n - 1 - m;
  const long long base = a * p.sa + b * p.sb + (top ? 0 : (long long)(p.n - 1) * p.s);
  const long long s = top ? p.s : -p.s;
  const double bcv = p.bc ? p.bc[t + (top ? 0 : lines)] : 0.0;
  ResidFin<double, float> fin;
  fin.mode = MODE;  // compile-time: the other modes' stores drop out
  fin.rin = rin + base;
  fin.u = u + base;
  fin.sigma = p.sigma;
  fin.out = rout ? rout + base : nullptr;
  const long long pbase = a * p.pa + b * p.pb + (top ? 0 : (long long)(p.n - 1) * p.pstride);
  fin.hi = hi ? hi + pbase : nullptr;
  fin.lo = lo ? lo + pbase : nullptr;
  fin.x32 = x32 ? x32 + pbase : nullptr;
  fin.pstride = top ? p.pstride : -p.pstride;
  fin.r32 = r32 ? r32 + base : nullptr;
  // xq != 0: the forward values in a separate array, row i of line t at
  // i * xq + t (the bottom lane walks it from row n-1 upwards)
  if (xq)
    solve_line_twist(top ? Rt : Rb, p.n, cnt, u + base, scratch + t + (top ? 0 : (long long)(p.n - 1) * xq),
                     s, top ? xq : -xq, bcv, fin, mask);
  else
    solve_line_twist(top ? Rt : Rb, p.n, cnt, u + base, scratch + base, s, s, bcv, fin, mask);
}

// ---- the same residual entirely on the FP32 pipe (double-float sweeps)
//
// The moment-form stencil sum is kept as a float pair, and the two sweeps
// and the final combination run in double-float arithmetic; intermediate
// arrays between the passes are float pairs (8 bytes, like FP64).  The
// sweeps are well conditioned (|ft|, |dt| < 1), so ~2^-48 relative rounding
// per operation gives a residual as accurate as the FP64 evaluation, which
// on GB300 would be bound by the FP64 pipe (1/57 of FP32).

template <int W>
__device__ __forceinline__ FF moment_sum_ff(const TriRow& r, const float (&v)[W], float ref, int skip) {
  float h = 0.f, l = 0.f;
#pragma unroll
  for (int m = 0; m < W; ++m) {
    if (m == skip) continue;
    float dh, dl;
    two_sum(v[m], -ref, dh, dl);
    const float ph = r.wh[m] * dh;
    float pl = fmaf(r.wh[m], dh, -ph);
    pl = fmaf(r.wh[m], dl, pl);
    pl = fmaf(r.wl[m], dh, pl);
    float sh, se;
    two_sum(h, ph, sh, se);
    h = sh;
    l += se + pl;
  }
  const float ph = r.rh * ref;
  float pl = fmaf(r.rh, ref, -ph);
  pl = fmaf(r.rl, ref, pl);
  float sh, se;
  two_sum(h, ph, sh, se);
  return ff_norm(sh, l + se + pl);
}

// cbc~ (bc - u_i) for a boundary row, bc an FP64 value.
__device__ __forceinline__ FF bc_term_ff(const TriRow& r, double bc, float ui) {
  return ff_mul({r.cbh, r.cbl}, ff_add(ff_from_double(bc), {-ui, 0.f}));
}

__device__ __forceinline__ FF ff_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ float2 f2_of(FF v) { return make_float2(v.h, v.l); }

// Final combination of one row (see ResidFin for the modes).
struct FinFF {
  int mode;
  FF sigma;
  float2* out;         // modes 0, 1: float-pair result, offset to the line
  __nv_bfloat16* hi;   // modes 2, 3: operand planes / FP32 operand, padded offsets
  __nv_bfloat16* lo;
  float* x32;
  long long pstride;
  float* r32;          // mode 3
  __device__ __forceinline__ void put(int i, long long idx, FF y, FF r, float u) const {
    if (mode == 0) r = ff_add(r, ff_neg(ff_mul_f(sigma, u)));
    const FF v = ff_add(r, ff_neg(y));
    if (mode <= 1) {
      out[idx] = f2_of(v);
      return;
    }
    const float f = ff_to_float(v);
    if (x32) {
      x32[i * pstride] = f;
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(f);
      hi[i * pstride] = h;
      lo[i * pstride] = __float2bfloat16_rn(f - __bfloat162float(h));
    }
    if (mode == 3) r32[idx] = f;
  }
};

template <bool kRinDouble>
__device__ __forceinline__ FF load_rin(const double* rd, const float2* rf, long long o) {
  if constexpr (kRinDouble)
    return ff_from_double(rd[o]);
  else
    return ff_of(rf[o]);
}

template <bool kRinDouble>
__device__ __forceinline__ void solve_line_ff(const TriRow* __restrict__ R, int n, const float* u,
                                              const double* rind, const float2* rinf, float2* xs,
                                              long long s, double lo, double hi, const FinFF& fin) {
  float f[7], g[7];
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    f[m] = u[(long long)m * s];
    g[m] = u[(long long)(n - 7 + m) * s];
  }
  // rows 0 and 1: 7-wide stencils on u_0..u_6, boundary value lo
  const FF x0 = ff_add(moment_sum_ff<7>(R[0], f, f[0], 0), bc_term_ff(R[0], lo, f[0]));
  const FF x1 = ff_add(ff_add(moment_sum_ff<7>(R[1], f, f[1], 1), bc_term_ff(R[1], lo, f[1])),
                       ff_neg(ff_mul({R[1].fth, R[1].ftl}, x0)));
  xs[0] = f2_of(x0);
  xs[s] = f2_of(x1);
  FF xm = x1;
  float w[5] = {f[0], f[1], f[2], f[3], f[4]};
  float pf[kAhead];
#pragma unroll
  for (int k = 0; k < kAhead; ++k) pf[k] = (5 + k < n) ? u[(long long)(5 + k) * s] : 0.f;
  int i = 2;
  for (; i + kAhead <= n - 2; i += kAhead) {
    float nb[kAhead];
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const int j = i + 3 + kAhead + k;
      nb[k] = (j < n) ? u[(long long)j * s] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const TriRow& r = R[i + k];
      const FF x = ff_add(moment_sum_ff<5>(r, w, w[2], 2), ff_neg(ff_mul({r.fth, r.ftl}, xm)));
      xs[(long long)(i + k) * s] = f2_of(x);
      xm = x;
      w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4]; w[4] = pf[k];
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) pf[k] = nb[k];
  }
  for (; i < n - 2; ++i) {
    const TriRow& r = R[i];
    const FF x = ff_add(moment_sum_ff<5>(r, w, w[2], 2), ff_neg(ff_mul({r.fth, r.ftl}, xm)));
    xs[(long long)i * s] = f2_of(x);
    xm = x;
    w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
    if (i + 3 < n) w[4] = u[(long long)(i + 3) * s];
  }
  // rows n-2 and n-1: 7-wide stencils on u_{n-7}..u_{n-1}, boundary value hi
  const TriRow& rA = R[n - 2];
  const TriRow& rB = R[n - 1];
  const FF xA = ff_add(ff_add(moment_sum_ff<7>(rA, g, g[5], 5), bc_term_ff(rA, hi, g[5])),
                       ff_neg(ff_mul({rA.fth, rA.ftl}, xm)));
  const FF xB = ff_add(ff_add(moment_sum_ff<7>(rB, g, g[6], 6), bc_term_ff(rB, hi, g[6])),
                       ff_neg(ff_mul({rB.fth, rB.ftl}, xA)));
  // back substitution with the final combination of each row; the forward
  // value, rin and (first pass) u of row i - k are loaded kAhead rows ahead
  const bool need_u = fin.mode == 0;
  auto uval = [&](long long o) { return need_u ? u[o] : 0.f; };
  FF y1 = xB;
  {
    const long long o = (long long)(n - 1) * s;
    fin.put(n - 1, o, xB, load_rin<kRinDouble>(rind, rinf, o), uval(o));
  }
  FF y = ff_add(xA, ff_neg(ff_mul({rA.dth, rA.dtl}, y1)));
  {
    const long long o = (long long)(n - 2) * s;
    fin.put(n - 2, o, y, load_rin<kRinDouble>(rind, rinf, o), uval(o));
  }
  y1 = y;
  i = n - 3;
  float2 rb[kAhead];
  FF rr[kAhead];
  float ru[kAhead];
#pragma unroll
  for (int k = 0; k < kAhead; ++k) {
    const bool in = i - k >= 0;
    const long long o = (long long)(i - k) * s;
    rb[k] = in ? xs[o] : make_float2(0.f, 0.f);
    rr[k] = in ? load_rin<kRinDouble>(rind, rinf, o) : FF{0.f, 0.f};
    ru[k] = (in && need_u) ? u[o] : 0.f;
  }
  for (; i - (kAhead - 1) >= 0; i -= kAhead) {
    float2 nb[kAhead];
    FF nr[kAhead];
    float nu[kAhead];
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const int j = i - kAhead - k;
      const long long o = (long long)j * s;
      nb[k] = (j >= 0) ? xs[o] : make_float2(0.f, 0.f);
      nr[k] = (j >= 0) ? load_rin<kRinDouble>(rind, rinf, o) : FF{0.f, 0.f};
      nu[k] = (j >= 0 && need_u) ? u[o] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      const TriRow& r = R[i - k];
      const FF yy = ff_add(ff_of(rb[k]), ff_neg(ff_mul({r.dth, r.dtl}, y1)));
      fin.put(i - k, (long long)(i - k) * s, yy, rr[k], ru[k]);
      y1 = yy;
    }
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
      rb[k] = nb[k];
      rr[k] = nr[k];
      ru[k] = nu[k];
    }
  }
  for (; i >= 0; --i) {
    const long long o = (long long)i * s;
    const TriRow& r = R[i];
    const FF yy = ff_add(ff_of(xs[o]), ff_neg(ff_mul({r.dth, r.dtl}, y1)));
    fin.put(i, o, yy, load_rin<kRinDouble>(rind, rinf, o), uval(o));
    y1 = yy;
  }
}

template <bool kRinDouble>
__global__ void __launch_bounds__(128) k_resid_ff(ResidPass<double> p, const TriRow* __restrict__ R,
                                                  const float* u, const double* rind,
                                                  const float2* rinf, float2* scratch, float2* rout,
                                                  __nv_bfloat16* hi, __nv_bfloat16* lo, float* x32,
                                                  float* r32, float sig_h, float sig_l) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)p.na * p.nb) return;
  const int a = (int)(t % p.na), b = (int)(t / p.na);
  const long long base = a * p.sa + b * p.sb;
  double blo = 0.0, bhi = 0.0;
  if (p.bc) {
    blo = p.bc[t];
    bhi = p.bc[t + (long long)p.na * p.nb];
  }
  FinFF fin;
  fin.mode = p.mode;
  fin.sigma = {sig_h, sig_l};
  fin.out = rout ? rout + base : nullptr;
  const long long pbase = a * p.pa + b * p.pb;
  fin.hi = hi ? hi + pbase : nullptr;
  fin.lo = lo ? lo + pbase : nullptr;
  fin.x32 = x32 ? x32 + pbase : nullptr;
  fin.pstride = p.pstride;
  fin.r32 = r32 ? r32 + base : nullptr;
  solve_line_ff<kRinDouble>(R, p.n, u + base, rind ? rind + base : nullptr, rinf ? rinf + base : nullptr,
                            scratch + base, p.s, blo, bhi, fin);
}

// solf(1:n1,1:n2,1:n3) = u1 + C, widened exactly and summed in FP64.
// Grid: x over i (blocks of 256), y = j, z strides over k (kPlanes planes
// per thread, loads issued together).
constexpr int kPlanes = 8;
__global__ void k_finalize(const float* __restrict__ u1, const float* __restrict__ c,
                           double* __restrict__ solf, int n1, int n2, int n3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1) return;
  const long long plane = (long long)n1 * n2, oplane = (long long)(n1 + 2) * (n2 + 2);
  const long long base = i + (long long)n1 * j;
  const long long obase = (i + 1) + (long long)(n1 + 2) * (j + 1);
  for (int k0 = blockIdx.z * kPlanes; k0 < n3; k0 += gridDim.z * kPlanes) {
    float a[kPlanes], b[kPlanes];
#pragma unroll
    for (int q = 0; q < kPlanes; ++q) {
      const int k = k0 + q;
      a[q] = k < n3 ? u1[base + plane * k] : 0.f;
      b[q] = (c && k < n3) ? c[base + plane * k] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < kPlanes; ++q)
      if (k0 + q < n3) solf[obase + oplane * (k0 + q + 1)] = widen(a[q]) + widen(b[q]);
  }
}

// Null-mode projection (all-Neumann or periodic operators at sigma = 0).
// The eigenvalue division zeroes the coefficient of the null mode, so the
// solution depends on a residual r only through
//   r_c = r - c v,   c = l . r,   l = l_x (x) l_y (x) l_z,  v = v_x (x) v_y (x) v_z,
// with l_a the row of V_a^-1 and v_a the column of V_a of the null eigenvalue
// (l . v = 1), and has c = 0 itself.  A residual keeps the rhs component c,
// which no iterate can remove; narrowed to FP32 together with it, r would
// lose its small part to the rounding of c and the refinement would stall.
// Likewise the operator cannot see an error along v, so the refinement
// cannot correct the solution's own null coefficient.  Kernels: per-plane
// partial sums of c, their sum in a fixed order, the projected residual
// narrowed into the operand of the next approximate solve, and the
// projection of the FP64 solution in place.
constexpr int kNullThreads = 256;
constexpr int kNullRows = 16;  // y rows per CTA of the partial sums

// part[k * G + g] = l_z(k) sum_i l_x(i) sum_{j in chunk g} l_y(j) r(i, j, k),
// r(i, j, k) = r[i + sy j + sz k].  Grid (n3, G = ceil(n2 / kNullRows));
// fixed summation order.
template <class T>
__global__ void __launch_bounds__(kNullThreads) k_null_part(const T* __restrict__ r, long long sy, long long sz,
                                                            const double* __restrict__ lx,
                                                            const double* __restrict__ ly,
                                                            const double* __restrict__ lz, int n1, int n2,
                                                            double* __restrict__ part) {
  __shared__ double red[kNullThreads];
  const int k = blockIdx.x, j0 = blockIdx.y * kNullRows, j1 = min(n2, j0 + kNullRows);
  const T* rk = r + sz * k;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n1; i += kNullThreads) {
    double s = 0.0;
#pragma unroll 4
    for (int j = j0; j < j1; ++j) s = fma(ly[j], (double)rk[i + sy * j], s);
    acc = fma(lx[i], s, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = kNullThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)k * gridDim.y + blockIdx.y] = red[0] * lz[k];
}

// part[count] = sum of part[0..count), one CTA, fixed order.
__global__ void __launch_bounds__(kNullThreads) k_null_sum(double* __restrict__ part, int count) {
  __shared__ double red[kNullThreads];
  double acc = 0.0;
  for (int q = threadIdx.x; q < count; q += kNullThreads) acc += part[q];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = kNullThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[count] = red[0];
}

// v = narrow(r - c v_x(i) v_y(j) v_z(k)) (r dense, FP64 or FP32; c = 0 when
// coef is null) into the operand of the next approximate solve (x32 for 3xTF32, else BF16 hi/lo
// planes; padded layout i + P1 (j + P2 k)) and, with r32, into the FP32
// residual copy.  Grid: x over i (blocks of 256), y = j, z strides over k.
template <class T>
__global__ void k_null_split(const T* __restrict__ r, const double* __restrict__ coef,
                             const double* __restrict__ vx, const double* __restrict__ vy,
                             const double* __restrict__ vz, int n1, int n2, int n3, int P1, int P2,
                             __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                             float* __restrict__ x32, float* __restrict__ r32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1) return;
  const double cxy = coef ? coef[0] * vx[i] * vy[j] : 0.0;
  const long long plane = (long long)n1 * n2, pplane = (long long)P1 * P2;
  const long long base = i + (long long)n1 * j, pbase = i + (long long)P1 * j;
  for (int k = blockIdx.z; k < n3; k += gridDim.z) {
    const double x = coef ? fma(-cxy, vz[k], (double)r[base + plane * k]) : (double)r[base + plane * k];
    float v;
    if constexpr (sizeof(T) == 8)
      v = narrow(x);
    else
      v = (float)x;
    const long long o = pbase + pplane * k;
    if (x32) {
      x32[o] = v;
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[o] = h;
      lo[o] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
    if (r32) r32[base + plane * k] = v;
  }
}

// u(i, j, k) -= c v_x(i) v_y(j) v_z(k) in place, u(i, j, k) = u[i + sy j + sz k].
// Grid as k_null_split.
__global__ void k_null_remove(double* __restrict__ u, long long sy, long long sz,
                              const double* __restrict__ coef, const double* __restrict__ vx,
                              const double* __restrict__ vy, const double* __restrict__ vz, int n1,
                              int n3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1) return;
  const double cxy = coef[0] * vx[i] * vy[j];
  for (int k = blockIdx.z; k < n3; k += gridDim.z) {
    double& x = u[i + sy * j + sz * k];
    x = fma(-cxy, vz[k], x);
  }
}

// rhs minus the boundary folds, in FP32, split straight into BF16 planes
// (padded layout).  Only feeds the first approximate solve of the mixed
// path: the FP64 residual that follows carries the boundary data exactly.
struct FoldArgsF {
  const float* ix[4];
  const float* iy[4];
  const float* iz[4];
  const float* bx;  // c * bc products: x faces [4][n3][bxp] (rows padded to bxp, plane stride bxs)
  const float* by;  // y faces [4][n1*n3], z faces [4][n1*n2]
  const float* bz;
  long long bxp, bxs;
};

// Fold of the boundary data into the right-hand side and store of the first
// transform's operand (mixed path): v = narrow(rhs) - sum over the four
// boundary columns of each axis of inv_lhs(:, c) * (ddr_c * bc), then FP32
// or split BF16 in the padded rotating layout.  kFoldJ rows j per thread:
// grid x over i (128-thread blocks), y over groups of kFoldJ rows, z strides
// over k.  The y-face products of (i, k) are loaded once and used for the
// thread's kFoldJ rows (one row per thread would re-read them for every j,
// ~250 MB of L2 traffic at 257^3); the z-face products of (i, j) and the
// y-rows of inv_lhs stay in registers for the whole k loop.
constexpr int kFoldJ = 8;
constexpr int kFoldKz = 16;
__global__ void __launch_bounds__(128) k_fold_split_rows(const double* __restrict__ rhs, FoldArgsF a,
                                                         __nv_bfloat16* hi, __nv_bfloat16* lo, float* x32,
                                                         int n1, int n2, int n3, int P1, int P2, int P3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j0 = blockIdx.y * kFoldJ;
  if (i >= P1) return;
  const bool in_i = i < n1;
  const long long sy = (long long)n1 * n3, sz = (long long)n1 * n2;
  float cx[4] = {0.f, 0.f, 0.f, 0.f}, cy[kFoldJ][4], fz[kFoldJ][4];
  if (in_i)
#pragma unroll
    for (int c = 0; c < 4; ++c) cx[c] = a.ix[c][i];
#pragma unroll
  for (int jj = 0; jj < kFoldJ; ++jj) {
    const int j = j0 + jj;
    const bool ok = in_i && j < n2;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      cy[jj][c] = ok ? a.iy[c][j] : 0.f;
      fz[jj][c] = ok ? a.bz[c * sz + i + (long long)n1 * j] : 0.f;
    }
  }
  for (int k = blockIdx.z; k < P3; k += gridDim.z) {
    const bool in_k = in_i && k < n3;
    float by[4] = {0.f, 0.f, 0.f, 0.f}, iz[4] = {0.f, 0.f, 0.f, 0.f};
    double r[kFoldJ];
    if (in_k) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        by[c] = a.by[c * sy + i + (long long)n1 * k];
        iz[c] = a.iz[c][k];
      }
    }
#pragma unroll
    for (int jj = 0; jj < kFoldJ; ++jj) {
      const int j = j0 + jj;
      r[jj] = (in_k && j < n2) ? rhs[i + (long long)n1 * (j + (long long)n2 * k)] : 0.0;
    }
    // per row jj: v = narrow(rhs), then for each boundary column c the
    // x-, y- and z-face terms, in that order; the x-face products of the
    // eight rows come as two aligned float4 (the same for the whole warp)
    float v[kFoldJ];
#pragma unroll
    for (int jj = 0; jj < kFoldJ; ++jj) v[jj] = narrow(r[jj]);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float bxv[kFoldJ];
      if (in_k) {
        const float4* q = reinterpret_cast<const float4*>(a.bx + c * a.bxs + a.bxp * k + j0);
        const float4 q0 = q[0], q1 = q[1];
        bxv[0] = q0.x; bxv[1] = q0.y; bxv[2] = q0.z; bxv[3] = q0.w;
        bxv[4] = q1.x; bxv[5] = q1.y; bxv[6] = q1.z; bxv[7] = q1.w;
      } else {
#pragma unroll
        for (int jj = 0; jj < kFoldJ; ++jj) bxv[jj] = 0.f;
      }
#pragma unroll
      for (int jj = 0; jj < kFoldJ; ++jj) {
        v[jj] -= cx[c] * bxv[jj];
        v[jj] -= cy[jj][c] * by[c];
        v[jj] -= iz[c] * fz[jj][c];
      }
    }
#pragma unroll
    for (int jj = 0; jj < kFoldJ; ++jj) {
      const int j = j0 + jj;
      const float vv = (in_k && j < n2) ? v[jj] : 0.f;  // padding stays zero
      const long long idx = i + (long long)P1 * (j + (long long)P2 * k);
      if (x32) {
        x32[idx] = vv;
      } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(vv);
        hi[idx] = h;
        lo[idx] = __float2bfloat16_rn(vv - __bfloat162float(h));
      }
    }
  }
}

// The four products of a face pair, plane c at out + c ps; face point t
// (rows of length r) at (t % r) + rp (t / r): rows padded to rp for aligned
// vector loads (rp = r, ps = nf: unpadded).
__global__ void k_fold_faces(const double* __restrict__ bc, double4 cc, float* out, long long nf, long long r,
                             long long rp, long long ps) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  const double lo = bc[t], hi = bc[t + nf];
  const long long o = (t % r) + rp * (t / r);
  out[o] = (float)(cc.x * lo);
  out[o + ps] = (float)(cc.y * lo);
  out[o + 2 * ps] = (float)(cc.z * hi);
  out[o + 3 * ps] = (float)(cc.w * hi);
}


// Extracts the interior of a (nx,ny,nz) field into an (nx-2,ny-2,nz-2) array.
__global__ void k_extract_interior(const double* __restrict__ g, double* __restrict__ out, int n1,
                                   int n2, int n3) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)n1 * n2 * n3;
  if (idx >= tot) return;
  const int i = (int)(idx % n1);
  const long long jk = idx / n1;
  const int j = (int)(jk % n2), k = (int)(jk / n2);
  out[idx] = g[(i + 1) + (long long)(n1 + 2) * ((j + 1) + (long long)(n2 + 2) * (k + 1))];
}

static inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// Profiler kinds (see mf_solver3d_profile_read in the C ABI).
enum ProfKind { kProfTc = 0, kProfResidX = 1, kProfResidYZ = 2, kProfNull = 3, kProfFold = 4,
                kProfFaces = 5, kProfGemm64 = 6, kProfCopy = 7, kProfTcDivide = 8,
                kProfTcUpdate = 9, kProfResid32 = 10 };

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------

template <class T>
static int upload(DevBuf& b, const std::vector<T>& v) {
  int rc = b.ensure(v.size() * sizeof(T));
  if (rc) return rc;
  MF_CUDA(cudaMemcpy(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return MF_OK;
}

static void split_bf16(const std::vector<double>& m, int n, int P, std::vector<__nv_bfloat16>& hi,
                       std::vector<__nv_bfloat16>& lo) {
  hi.assign((size_t)P * P, __float2bfloat16_rn(0.f));
  lo.assign((size_t)P * P, __float2bfloat16_rn(0.f));
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      const float v = (float)m[(size_t)r * n + c];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[(size_t)r * P + c] = h;
      lo[(size_t)r * P + c] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// Nearest TF32 value of x (ties away from zero), kept as an FP32 number:
// the 13 low mantissa bits are rounded off on the bit pattern.
static float tf32_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// hi = tf32(m), lo = tf32(m - hi), zero-padded to P x P.
static void split_tf32(const std::vector<double>& m, int n, int P, std::vector<float>& hi,
                       std::vector<float>& lo) {
  hi.assign((size_t)P * P, 0.f);
  lo.assign((size_t)P * P, 0.f);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      const double v = m[(size_t)r * n + c];
      const float h = tf32_round((float)v);
      hi[(size_t)r * P + c] = h;
      lo[(size_t)r * P + c] = tf32_round((float)(v - (double)h));
    }
}

// Uploads eigen tables (row-major V, V^-1), their split-BF16 copies and
// their 3xTF32 planes.
static int axis_set_eigen(AxisDev& d, const std::vector<double>& eig, const std::vector<double>& V,
                          const std::vector<double>& Vinv) {
  int rc;
  if ((rc = upload(d.V, V)) || (rc = upload(d.Vinv, Vinv)) || (rc = upload(d.eig, eig))) return rc;
  std::vector<__nv_bfloat16> hi, lo;
  split_bf16(Vinv, d.n, d.P, hi, lo);
  if ((rc = upload(d.Vih, hi)) || (rc = upload(d.Vil, lo))) return rc;
  split_bf16(V, d.n, d.P, hi, lo);
  if ((rc = upload(d.Vh, hi)) || (rc = upload(d.Vl, lo))) return rc;
  std::vector<float> h32, l32;
  split_tf32(Vinv, d.n, d.P, h32, l32);
  if ((rc = upload(d.Vih32, h32)) || (rc = upload(d.Vil32, l32))) return rc;
  split_tf32(V, d.n, d.P, h32, l32);
  if ((rc = upload(d.Vh32, h32)) || (rc = upload(d.Vl32, l32))) return rc;
  std::vector<float> ef(d.P, 0.f);
  std::vector<uint8_t> nf(d.P, 0);
  int nnull = 0;
  for (int i = 0; i < d.n; ++i) {
    ef[i] = (float)eig[i];
    nf[i] = std::fabs(eig[i]) < kNullThresh ? 1 : 0;
    if (nf[i]) {
      d.null_idx = i;
      ++nnull;
    }
  }
  if ((rc = upload(d.eigf, ef)) || (rc = upload(d.nullf, nf))) return rc;
  if (nnull != 1) {
    d.null_idx = -1;
    d.null_row.release();
    d.null_col.release();
    return MF_OK;
  }
  std::vector<double> row(d.n), col(d.n);
  for (int i = 0; i < d.n; ++i) {
    row[i] = Vinv[(size_t)d.null_idx * d.n + i];
    col[i] = V[(size_t)i * d.n + d.null_idx];
  }
  if ((rc = upload(d.null_row, row)) || (rc = upload(d.null_col, col))) return rc;
  return MF_OK;
}

// TriRow table of an axis whose factored lhs is tridiagonal (p, e, alpha
// and beta all zero), from the packed rows p, f, 1/c, d, e, r0..r6.
static int build_tri_rows(AxisDev& d, const std::vector<double>& rows) {
  const int n = d.n;
  d.tri_ok = n >= 8;
  for (int i = 0; i < n && d.tri_ok; ++i)
    if (rows[(size_t)kRow * i + 0] != 0.0 || rows[(size_t)kRow * i + 4] != 0.0) d.tri_ok = false;
  if (!d.tri_ok) return MF_OK;
  std::vector<TriRow> tr(n);
  for (int i = 0; i < n; ++i) {
    const double* r = &rows[(size_t)kRow * i];
    const double inv_c = r[2];
    TriRow& t = tr[i];
    std::memset(&t, 0, sizeof(t));
    const int bcrow = i == 0 ? 0 : i == 1 ? 1 : i == n - 2 ? 2 : i == n - 1 ? 3 : -1;
    t.cbc = bcrow >= 0 ? d.bcc[bcrow] * inv_c : 0.0;
    long double rho = (long double)t.cbc;
    for (int m = 0; m < 7; ++m) {
      const double w = r[5 + m] * inv_c;
      rho += (long double)w;
      t.wh[m] = (float)w;
      t.wl[m] = (float)(w - (double)t.wh[m]);
    }
    const double rd = (double)rho;
    t.rh = (float)rd;
    t.rl = (float)(rd - (double)t.rh);
    t.ft = i > 0 ? r[1] * inv_c / rows[(size_t)kRow * (i - 1) + 2] : 0.0;
    t.dt = i < n - 1 ? r[3] * inv_c : 0.0;
    auto split = [](double v, float& h, float& l) {
      h = (float)v;
      l = (float)(v - (double)h);
    };
    split(t.ft, t.fth, t.ftl);
    split(t.dt, t.dth, t.dtl);
    split(t.cbc, t.cbh, t.cbl);
  }
  // bottom table of the two-sided sweeps: T = L U has T_{i,i-1} = ft_i,
  // T_ii = 1 + ft_i dt_{i-1}, T_{i,i+1} = dt_i; its U L pivots from the
  // bottom q_{n-1} = T_{n-1,n-1}, q_i = T_ii - T_{i,i+1} T_{i+1,i} / q_{i+1}
  // (rows n-1..m+1); entry k holds row i = n-1-k with the weights (and cbc)
  // divided by q_i in reversed stencil order, gt_i = dt_i / q_i as ft and
  // et_i = ft_i / q_i as dt.
  const int m = (n - 1) / 2, cb = n - 1 - m;
  std::vector<long double> q(n, 1.0L);
  auto tdiag = [&](int i) { return 1.0L + (i > 0 ? (long double)tr[i].ft * (long double)tr[i - 1].dt : 0.0L); };
  q[n - 1] = tdiag(n - 1);
  for (int i = n - 2; i > m; --i) q[i] = tdiag(i) - (long double)tr[i].dt * (long double)tr[i + 1].ft / q[i + 1];
  std::vector<TriRow> tb(cb);
  for (int k = 0; k < cb; ++k) {
    const int i = n - 1 - k;
    const double* r = &rows[(size_t)kRow * i];
    const long double iq = 1.0L / q[i];
    TriRow& t = tb[k];
    std::memset(&t, 0, sizeof(t));
    const int width = (i >= n - 2) ? 7 : 5;
    t.cbc = (double)((long double)tr[i].cbc * iq);
    long double rho = (long double)t.cbc;
    for (int mm = 0; mm < width; ++mm) {
      const double w = (double)((long double)(r[5 + (width - 1 - mm)] * r[2]) * iq);
      rho += (long double)w;
      t.wh[mm] = (float)w;
      t.wl[mm] = (float)(w - (double)t.wh[mm]);
    }
    const double rd = (double)rho;
    t.rh = (float)rd;
    t.rl = (float)(rd - (double)t.rh);
    t.ft = (double)((long double)tr[i].dt * iq);
    t.dt = (double)((long double)tr[i].ft * iq);
  }
  const long double tw = 1.0L / (1.0L - (long double)tr[m].dt * (long double)tb[cb - 1].dt);
  tr[m].tw = (double)tw;
  tb[cb - 1].tw = (double)tw;
  int rc = d.tri.ensure(sizeof(TriRow) * n);
  if (!rc) rc = d.trib.ensure(sizeof(TriRow) * cb);
  if (rc) return rc;
  MF_CUDA(cudaMemcpy(d.tri.ptr, tr.data(), sizeof(TriRow) * n, cudaMemcpyHostToDevice));
  MF_CUDA(cudaMemcpy(d.trib.ptr, tb.data(), sizeof(TriRow) * cb, cudaMemcpyHostToDevice));
  return MF_OK;
}

static int axis_upload(AxisDev& d, const SolverAxisHost& h) {
  const int n = h.n;
  d.n = n;
  d.P = (n + 63) / 64 * 64;
  d.bc[0] = h.bc[0];
  d.bc[1] = h.bc[1];
  d.bcc[0] = h.ddr[0];
  d.bcc[1] = h.ddr[8];
  d.bcc[2] = h.ddr[8 * (n - 2) + 7];
  d.bcc[3] = h.ddr[8 * (n - 1) + 6];
  for (int m = 0; m < 14; ++m) d.neum[m] = h.neum[m];
  int rc;
  std::vector<double> l4((size_t)4 * n);
  const int cols[4] = {0, 1, n - 2, n - 1};
  for (int c = 0; c < 4; ++c)
    for (int i = 0; i < n; ++i) l4[(size_t)c * n + i] = h.inv_lhs[(size_t)i * n + cols[c]];
  if ((rc = upload(d.invl4, l4))) return rc;
  std::vector<float> l4f(l4.begin(), l4.end());
  if ((rc = upload(d.invl4f, l4f))) return rc;
  // residual operator rows: factored lhs + 7-wide explicit stencil (see mf_line.cuh)
  std::vector<double> rows((size_t)kRow * n, 0.0);
  for (int i = 0; i < n; ++i) {
    double* r = &rows[(size_t)kRow * i];
    r[0] = h.ddl_lu[5 * i + 0];
    r[1] = h.ddl_lu[5 * i + 1];
    r[2] = 1.0 / h.ddl_lu[5 * i + 2];
    r[3] = h.ddl_lu[5 * i + 3];
    r[4] = h.ddl_lu[5 * i + 4];
    const double* dr = &h.ddr[8 * i];
    if (i == 0) {
      for (int m = 0; m < 6; ++m) r[5 + m] = dr[1 + m];
    } else if (i == 1) {
      for (int m = 0; m < 7; ++m) r[5 + m] = dr[1 + m];
    } else if (i == n - 2) {
      for (int m = 0; m < 7; ++m) r[5 + m] = dr[m];
    } else if (i == n - 1) {
      for (int m = 0; m < 6; ++m) r[6 + m] = dr[m];
    } else {
      for (int m = 0; m < 5; ++m) r[5 + m] = dr[m];
    }
  }
  if ((rc = upload(d.rows, rows))) return rc;
  // FP32 rows for the correction residual: factored lhs rounded, explicit
  // stencil as hi + lo pairs (see solve_line_comp)
  std::vector<float> rowsf((size_t)kRowF * n, 0.f);
  for (int i = 0; i < n; ++i) {
    const double* r = &rows[(size_t)kRow * i];
    float* o = &rowsf[(size_t)kRowF * i];
    for (int m = 0; m < 5; ++m) o[m] = (float)r[m];
    for (int m = 0; m < 7; ++m) {
      const float hi = (float)r[5 + m];
      o[5 + m] = hi;
      o[12 + m] = (float)(r[5 + m] - (double)hi);
    }
  }
  if ((rc = upload(d.rowsf, rowsf))) return rc;
  if ((rc = build_tri_rows(d, rows))) return rc;
  return axis_set_eigen(d, h.eigen, h.vect, h.inv_vect);
}

static int gemm_f64(StageProfiler& prof, const double* X, int M, int K, const double* A, int N,
                    double* Y, const GemmEpi& e, cudaStream_t st, int B = 1, long long xs = 0,
                    long long ys = 0, bool may_tune = true) {
  auto run = [&](int use64) -> int {
    if (use64)
      k_gemm_f64<64><<<dim3(blocks_for(M, 64), blocks_for(N, 64), B), 256, 0, st>>>(X, M, K, A, N, Y, e, xs,
                                                                                   ys);
    else
      k_gemm_f64<32><<<dim3(blocks_for(M, 32), blocks_for(N, 32), B), 256, 0, st>>>(X, M, K, A, N, Y, e, xs,
                                                                                   ys);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
  };
  // tile: 64 when it gives at least two CTAs per SM (heuristic), or the
  // measured choice for this shape (the variants differ only in speed: each
  // output sums its K products in the same order; every epilogue is a pure
  // store, so a timed repeat leaves the same result)
  const long long tiles64 = (long long)blocks_for(M, 64) * blocks_for(N, 64) * B;
  int use64 = tiles64 >= 2LL * num_sms() ? 1 : 0;
  if (may_tune && tune_mode() == 1) {
    int c = tune_lookup(kTuneGemm64, M, N, K, B);
    if (c < 0 && !stream_capturing(st)) {
      c = tune_measure(st, 2, run);
      if (c >= 0) tune_store(kTuneGemm64, M, N, K, B, c);
    }
    if (c >= 0) use64 = c;
  }
  prof.begin(kProfGemm64, st);
  if (run(use64)) {
    prof.end(st);
    return set_error(MF_ERR_CUDA, "k_gemm_f64 launch failed");
  }
  prof.end(st);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static int faces(mf_solver3d* sc, double* solf, const double* bcs[3], cudaStream_t st, int B = 1,
                 long long s_solf = 0, const long long* s_bc = nullptr) {
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const long long p1 = n1 + 2, p2 = n2 + 2;
  for (int axis = 0; axis < 3; ++axis) {
    const AxisDev& d = sc->ax[axis];
    FaceArgs f;
    if (axis == 0) { f.sA = 1; f.sa = p1; f.sb = p1 * p2; f.n = n1; f.na = n2; f.nb = n3; }
    if (axis == 1) { f.sA = p1; f.sa = 1; f.sb = p1 * p2; f.n = n2; f.na = n1; f.nb = n3; }
    if (axis == 2) { f.sA = p1 * p2; f.sa = 1; f.sb = p1; f.n = n3; f.na = n1; f.nb = n2; }
    f.bc0 = d.bc[0];
    f.bc1 = d.bc[1];
    for (int m = 0; m < 7; ++m) { f.nl[m] = d.neum[m]; f.nr[m] = d.neum[7 + m]; }
    sc->prof.begin(kProfFaces, st);
    k_faces<<<dim3(blocks_for((long long)f.na * f.nb, 128), B), 128, 0, st>>>(solf, bcs[axis], f, s_solf,
                                                                             s_bc ? s_bc[axis] : 0);
    sc->prof.end(st);
    MF_CUDA(cudaGetLastError());
  }
  return MF_OK;
}

static FoldArgs fold_args(mf_solver3d* sc) {
  FoldArgs a;
  for (int c = 0; c < 4; ++c) {
    a.ix[c] = sc->ax[0].invl4.as<double>() + (size_t)c * sc->n[0];
    a.iy[c] = sc->ax[1].invl4.as<double>() + (size_t)c * sc->n[1];
    a.iz[c] = sc->ax[2].invl4.as<double>() + (size_t)c * sc->n[2];
    a.cx[c] = sc->ax[0].bcc[c];
    a.cy[c] = sc->ax[1].bcc[c];
    a.cz[c] = sc->ax[2].bcc[c];
  }
  return a;
}

// Plain FP64 solve on device pointers.
// B problems of the same operator and sigma in one pass of launches: rhs,
// solf and the boundary arrays of problem b at b times their element
// strides (a stride of 0 shares one array between all problems).  Every
// stage indexes its problem from the grid (blockIdx.y or .z), so the
// per-problem arithmetic, and the result, is that of B separate solves.
static int solve_plain_batch(mf_solver3d* sc, int B, const double* rhs, long long s_rhs, double sigma,
                             double* solf, long long s_solf, const double* bcs[3], const long long s_bc[3],
                             cudaStream_t st) {
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const long long tot = (long long)n1 * n2 * n3;
  int rc;
  if ((rc = sc->w0.ensure((size_t)B * tot * sizeof(double))) ||
      (rc = sc->w1.ensure((size_t)B * tot * sizeof(double))))
    return rc;
  double* w0 = sc->w0.as<double>();
  double* w1 = sc->w1.as<double>();
  FoldBatch fb;
  fb.rhs = s_rhs;
  fb.out = tot;
  for (int a = 0; a < 3; ++a) fb.bc[a] = s_bc[a];
  sc->prof.begin(kProfFold, st);
  k_fold<<<dim3(blocks_for(tot, 256), B), 256, 0, st>>>(rhs, w0, bcs[0], bcs[1], bcs[2], fold_args(sc), n1,
                                                        n2, n3, fb);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  GemmEpi plain;
  const double* Vi[3] = {sc->ax[0].Vinv.as<double>(), sc->ax[1].Vinv.as<double>(),
                         sc->ax[2].Vinv.as<double>()};
  const double* Vf[3] = {sc->ax[0].V.as<double>(), sc->ax[1].V.as<double>(),
                         sc->ax[2].V.as<double>()};
  // forward transforms with V^-1: x, y, z (+ divide)
  if ((rc = gemm_f64(sc->prof, w0, n2 * n3, n1, Vi[0], n1, w1, plain, st, B, tot, tot))) return rc;
  if ((rc = gemm_f64(sc->prof, w1, n3 * n1, n2, Vi[1], n2, w0, plain, st, B, tot, tot))) return rc;
  GemmEpi div;
  div.kind = 1;
  div.lx = sc->ax[0].eig.as<double>();
  div.ly = sc->ax[1].eig.as<double>();
  div.lz = sc->ax[2].eig.as<double>();
  div.sigma = sigma;
  div.thresh = kNullThresh;
  div.n1 = n1;
  div.n2 = n2;
  if ((rc = gemm_f64(sc->prof, w0, n1 * n2, n3, Vi[2], n3, w1, div, st, B, tot, tot))) return rc;
  // inverse transforms with V, the last one written into solf's interior
  if ((rc = gemm_f64(sc->prof, w1, n2 * n3, n1, Vf[0], n1, w0, plain, st, B, tot, tot))) return rc;
  if ((rc = gemm_f64(sc->prof, w0, n3 * n1, n2, Vf[1], n2, w1, plain, st, B, tot, tot))) return rc;
  GemmEpi out;
  out.kind = 2;
  out.n1 = n1;
  out.n2 = n2;
  if ((rc = gemm_f64(sc->prof, w1, n1 * n2, n3, Vf[2], n3, solf, out, st, B, tot, s_solf))) return rc;
  return faces(sc, solf, bcs, st, B, s_solf, s_bc);
}

static int solve_plain_dev(mf_solver3d* sc, const double* rhs, double sigma, double* solf,
                           const double* bcs[3], cudaStream_t st) {
  const long long zero[3] = {0, 0, 0};
  return solve_plain_batch(sc, 1, rhs, 0, sigma, solf, 0, bcs, zero, st);
}

// Residual on device pointers, three passes (x, y, z):
//   r = rin - sigma*u - sum_a L_a u.
// rin/u/bcs describe the problem (bcs may be null: homogeneous data).  The
// last pass writes the FP64/FP32 array `r` (when planes and x32 are null),
// the split-BF16 planes or the FP32 operand x32 of the 3xTF32 transforms
// (and, with r32, an FP32 copy of r).
// The three passes in double-float arithmetic (tridiagonal operators, FP32
// iterate): x from the FP64 rin, y and z from float-pair intermediates.
// Selected by mf_solver3d_set_residual(MF_RESID_FF).  Measured at 257^3 on
// GB300 it is slower than the FP64 sweeps (1.02 vs 0.78 ms for the three
// passes): without FP64 operations the passes become bound by the issue and
// latency of the long dependent double-float chains of the sweeps.
static int residual_ff(mf_solver3d* sc, const double* rin, const float* u, double sigma,
                       const double* bcs[3], float2* s0, float2* s1, __nv_bfloat16* hi,
                       __nv_bfloat16* lo, float* x32, float* r32, cudaStream_t st) {
  const long long n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const float sh = (float)sigma, sl = (float)(sigma - (double)sh);
  auto pass = [&](int axis, int mode) {
    ResidPass<double> p;
    const AxisDev& d = sc->ax[axis];
    p.rows = nullptr;
    p.n = d.n;
    p.bc = bcs ? bcs[axis] : nullptr;
    p.bcc = make_double4(0, 0, 0, 0);
    p.sigma = sigma;
    p.mode = mode;
    p.pa = p.pb = p.pstride = 0;
    if (axis == 0) { p.na = (int)n2; p.nb = (int)n3; p.sa = n1; p.sb = n1 * n2; p.s = 1; }
    if (axis == 1) { p.na = (int)n1; p.nb = (int)n3; p.sa = 1; p.sb = n1 * n2; p.s = n1; }
    if (axis == 2) {
      p.na = (int)n1; p.nb = (int)n2; p.sa = 1; p.sb = n1; p.s = n1 * n2;
      p.pa = 1; p.pb = sc->P[0]; p.pstride = (long long)sc->P[0] * sc->P[1];
    }
    return p;
  };
  auto blocks = [&](const ResidPass<double>& p) { return blocks_for((long long)p.na * p.nb, 128); };
  ResidPass<double> px = pass(0, 0), py = pass(1, 1), pz = pass(2, r32 ? 3 : 2);
  sc->prof.begin(kProfResidX, st);
  k_resid_ff<true><<<blocks(px), 128, 0, st>>>(px, sc->ax[0].tri.as<TriRow>(), u, rin, nullptr, s0, s0,
                                               nullptr, nullptr, nullptr, nullptr, sh, sl);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  sc->prof.begin(kProfResidYZ, st);
  k_resid_ff<false><<<blocks(py), 128, 0, st>>>(py, sc->ax[1].tri.as<TriRow>(), u, nullptr, s0, s1, s1,
                                                nullptr, nullptr, nullptr, nullptr, sh, sl);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  sc->prof.begin(kProfResidYZ, st);
  k_resid_ff<false><<<blocks(pz), 128, 0, st>>>(pz, sc->ax[2].tri.as<TriRow>(), u, nullptr, s1, s0,
                                                nullptr, hi, lo, x32, r32, sh, sl);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

template <class T, class In>
static int residual_passes(mf_solver3d* sc, const T* rin, const In* u, double sigma,
                           const double* bcs[3], T* s0, T* s1, T* r, __nv_bfloat16* hi,
                           __nv_bfloat16* lo, float* x32, float* r32, int prof_kind_x,
                           int prof_kind_yz, cudaStream_t st) {
  const long long n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  auto pass = [&](int axis) {
    ResidPass<T> p;
    const AxisDev& d = sc->ax[axis];
    p.rows = sizeof(T) == 8 ? reinterpret_cast<const T*>(d.rows.ptr) : reinterpret_cast<const T*>(d.rowsf.ptr);
    p.n = d.n;
    p.bc = bcs ? bcs[axis] : nullptr;
    p.bcc = make_double4(d.bcc[0], d.bcc[1], d.bcc[2], d.bcc[3]);
    p.sigma = (T)sigma;
    p.pa = p.pb = p.pstride = 0;
    if (axis == 0) { p.na = (int)n2; p.nb = (int)n3; p.sa = n1; p.sb = n1 * n2; p.s = 1; }
    if (axis == 1) { p.na = (int)n1; p.nb = (int)n3; p.sa = 1; p.sb = n1 * n2; p.s = n1; }
    if (axis == 2) { p.na = (int)n1; p.nb = (int)n2; p.sa = 1; p.sb = n1; p.s = n1 * n2; }
    return p;
  };
  // FP32 iterate, FP64-accurate residual, tridiagonal operators: moment
  // form, with FP64 sweeps (default) or double-float sweeps
  bool tri = false;
  if constexpr (sizeof(T) == 8 && sizeof(In) == 4) {
    tri = sc->ax[0].tri_ok && sc->ax[1].tri_ok && sc->ax[2].tri_ok;
    if (tri && sc->resid_mode == MF_RESID_FF && (hi || x32))
      return residual_ff(sc, rin, u, sigma, bcs, reinterpret_cast<float2*>(s0),
                         reinterpret_cast<float2*>(s1), hi, lo, x32, r32, st);
  }
  int axis_of_pass = 0;
  // xt: a field-sized array free during the pass, for the forward values of
  // the unit-stride pass (nullptr: they go to scratch, in the field's layout)
  auto launch = [&](const ResidPass<T>& p, int kind, const T* in_r, T* scratch, T* rout,
                    __nv_bfloat16* h, __nv_bfloat16* l, float* x, float* r32p, T* xt) -> int {
    sc->prof.begin(kind, st);
    if constexpr (sizeof(T) == 8 && sizeof(In) == 4) {
      // The x pass (unit stride along the line) runs two-sided only with its
      // forward values stored across lines (xt): in the field's layout the
      // per-lane sector streams outgrow L1 (257^3 on GB300: 0.41 ms
      // two-sided, 0.33 ms one thread per line, 0.31 ms two-sided with xt;
      // the y and z passes drop from 0.25 to 0.19 ms each).  Without xt it
      // stays one thread per line.
      const bool across = p.s == 1 && xt;
      if (tri && (sc->resid_mode == MF_RESID_FP64_LINE || (p.s == 1 && !across))) {
        k_resid_tri<<<blocks_for((long long)p.na * p.nb, 128), 128, 0, st>>>(
            p, sc->ax[axis_of_pass].tri.template as<TriRow>(), u, in_r, across ? xt : scratch,
            across ? (long long)p.na * p.nb : 0LL, rout, h, l, x, r32p);
        sc->prof.end(st);
        MF_CUDA(cudaGetLastError());
        return MF_OK;
      }
      if (tri) {
        const AxisDev& d = sc->ax[axis_of_pass];
        auto kern = p.mode == 0 ? k_resid_twist<0> : p.mode == 1 ? k_resid_twist<1>
                  : p.mode == 2 ? k_resid_twist<2> : k_resid_twist<3>;
        kern<<<blocks_for(2 * (long long)p.na * p.nb, 128), 128, 0, st>>>(
            p, d.tri.template as<TriRow>(), d.trib.template as<TriRow>(), u, in_r, across ? xt : scratch,
            across ? (long long)p.na * p.nb : 0LL, rout, h, l, x, r32p);
        sc->prof.end(st);
        MF_CUDA(cudaGetLastError());
        return MF_OK;
      }
    }
    k_resid_lines<T, In><<<blocks_for((long long)p.na * p.nb, 128), 128, 0, st>>>(
        p, u, in_r, scratch, rout, h, l, x, r32p);
    sc->prof.end(st);
    MF_CUDA(cudaGetLastError());
    return MF_OK;
  };
  int rc;
  ResidPass<T> px = pass(0);
  px.mode = 0;
  axis_of_pass = 0;
  if ((rc = launch(px, prof_kind_x, rin, s0, s0, nullptr, nullptr, nullptr, nullptr, s1))) return rc;
  ResidPass<T> py = pass(1);
  py.mode = 1;
  axis_of_pass = 1;
  if ((rc = launch(py, prof_kind_yz, s0, s1, s1, nullptr, nullptr, nullptr, nullptr, nullptr))) return rc;
  ResidPass<T> pz = pass(2);
  axis_of_pass = 2;
  if (hi || x32) {
    pz.mode = r32 ? 3 : 2;
    pz.pa = 1;
    pz.pb = sc->P[0];
    pz.pstride = (long long)sc->P[0] * sc->P[1];
    return launch(pz, prof_kind_yz, s1, s0, nullptr, hi, lo, x32, r32, nullptr);
  }
  pz.mode = 1;
  return launch(pz, prof_kind_yz, s1, r, r, nullptr, nullptr, nullptr, nullptr, nullptr);
}

// Operand buffers and tensor-core plans of one mixed format (split-BF16 or
// 3xTF32), created on first use; the zeroing is ordered on the caller's
// stream st (a legacy-stream memset would not be ordered before work on a
// non-blocking stream).
static int mixed_prepare(mf_solver3d* sc, bool tf32, cudaStream_t st) {
  if (tf32 ? sc->mixed32_ready : sc->mixed_ready) return MF_OK;
  for (int a = 0; a < 3; ++a)
    if (sc->P[a] > 256)
      return set_error(MF_ERR_UNSUPPORTED,
                       "mixed-precision transforms support up to 256 interior points per axis "
                       "(axis %d has %d)", a, sc->n[a]);
  const long long tot = (long long)sc->n[0] * sc->n[1] * sc->n[2];
  const long long ptot = (long long)sc->P[0] * sc->P[1] * sc->P[2];
  int rc;
  if ((rc = sc->R.ensure(tot * 8)) || (rc = sc->R2.ensure(tot * 8)) || (rc = sc->U32.ensure(tot * 4)) ||
      (rc = sc->C32.ensure(tot * 4)) || (rc = sc->R1f.ensure(tot * 4)))
    return rc;
  // operands are zero-padded to P per axis; the padding stays zero because
  // the padded rows and columns of every matrix are zero
  DevBuf* xa[2] = {tf32 ? &sc->Xa32 : &sc->Xa_hi, tf32 ? nullptr : &sc->Xa_lo};
  DevBuf* xb[2] = {tf32 ? &sc->Xb32 : &sc->Xb_hi, tf32 ? nullptr : &sc->Xb_lo};
  const size_t bytes = (size_t)ptot * (tf32 ? 4 : 2);
  for (DevBuf* x : {xa[0], xa[1], xb[0], xb[1]}) {
    if (!x) continue;
    if ((rc = x->ensure(bytes))) return rc;
    MF_CUDA(cudaMemsetAsync(x->ptr, 0, bytes, st));
  }
  if ((rc = sc->err.ensure(sizeof(int)))) return rc;
  MF_CUDA(cudaMemsetAsync(sc->err.ptr, 0, sizeof(int), st));
  const int P1 = sc->P[0], P2 = sc->P[1], P3 = sc->P[2];
  struct Spec { DevBuf** x; int axis; bool inv; int M; };
  const Spec specs[6] = {{xa, 0, true, P2 * P3}, {xb, 1, true, P3 * P1}, {xa, 2, true, P1 * P2},
                         {xb, 0, false, P2 * P3}, {xa, 1, false, P3 * P1}, {xb, 2, false, P1 * P2}};
  TcPlan** plans = tf32 ? sc->plan32 : sc->plan;
  for (int t = 0; t < 6; ++t) {
    AxisDev& d = sc->ax[specs[t].axis];
    DevBuf& bh = tf32 ? (specs[t].inv ? d.Vih32 : d.Vh32) : (specs[t].inv ? d.Vih : d.Vh);
    DevBuf& bl = tf32 ? (specs[t].inv ? d.Vil32 : d.Vl32) : (specs[t].inv ? d.Vil : d.Vl);
    const void* xlo = specs[t].x[1] ? specs[t].x[1]->ptr : nullptr;
    if ((rc = tc_plan_create(&plans[t], tf32, specs[t].x[0]->ptr, xlo, bh.ptr, bl.ptr, specs[t].M,
                             d.P, d.P)))
      return rc;
  }
  (tf32 ? sc->mixed32_ready : sc->mixed_ready) = true;
  return MF_OK;
}

static int tc_run(mf_solver3d* sc, bool tf32, int t, const TcEpilogue& e, cudaStream_t st) {
  const TcPlan* p = (tf32 ? sc->plan32 : sc->plan)[t];
  int plan = 0;
  // 3xTF32 slice width: the process setting, or with the tuner on the
  // measured choice for this shape.  The two plans give identical results;
  // only epilogues that store (not the accumulating update) are repeated
  // for timing.
  if (tf32 && tc_has_wide(p) && tc_get_tf32_plan() == 0 && tune_mode() == 1 &&
      (e.kind != 2 || !e.accumulate)) {
    const int axis = t % 3, M = (axis == 0 ? sc->P[1] * sc->P[2] : axis == 1 ? sc->P[2] * sc->P[0]
                                                                             : sc->P[0] * sc->P[1]);
    const int N = sc->ax[axis].P;
    int c = tune_lookup(kTuneTcTf32, M, N, N, 0);
    if (c < 0 && !stream_capturing(st)) {
      c = tune_measure(st, 2, [&](int v) {
        return tc_transform(p, e, sc->err.as<int>(), st, v ? 2 : 1) == MF_OK ? 0 : 1;
      });
      if (c >= 0) tune_store(kTuneTcTf32, M, N, N, 0, c);
    }
    if (c >= 0) plan = c ? 2 : 1;
  }
  sc->prof.begin(e.kind == 0 ? kProfTc : e.kind == 1 ? kProfTcDivide : kProfTcUpdate, st);
  int rc = tc_transform(p, e, sc->err.as<int>(), st, plan);
  sc->prof.end(st);
  return rc;
}

// Points the store epilogue at operand buffer A (second = false) or B.
static void set_target(TcEpilogue& e, mf_solver3d* sc, bool tf32, bool to_b) {
  if (tf32) {
    e.y32 = (to_b ? sc->Xb32 : sc->Xa32).as<float>();
  } else {
    e.y_hi = (to_b ? sc->Xb_hi : sc->Xa_hi).as<__nv_bfloat16>();
    e.y_lo = (to_b ? sc->Xb_lo : sc->Xa_lo).as<__nv_bfloat16>();
  }
}

// One approximate solve of the folded right-hand side already stored in
// operand buffer A; the six transforms ping-pong between A and B.
static int approx_solve(mf_solver3d* sc, bool tf32, double sigma, float* dest, bool accumulate,
                        cudaStream_t st) {
  TcEpilogue e;
  int rc;
  e.kind = 0;
  set_target(e, sc, tf32, true);
  if ((rc = tc_run(sc, tf32, 0, e, st))) return rc;
  set_target(e, sc, tf32, false);
  if ((rc = tc_run(sc, tf32, 1, e, st))) return rc;
  TcEpilogue d;
  d.kind = 1;
  set_target(d, sc, tf32, true);
  d.lam_x = sc->ax[0].eigf.as<float>();
  d.lam_y = sc->ax[1].eigf.as<float>();
  d.lam_z = sc->ax[2].eigf.as<float>();
  d.null_x = sc->ax[0].nullf.as<uint8_t>();
  d.null_y = sc->ax[1].nullf.as<uint8_t>();
  d.null_z = sc->ax[2].nullf.as<uint8_t>();
  d.sigma = (float)sigma;
  d.sigma_null = std::fabs(sigma) < kNullThresh ? 1 : 0;
  d.n1 = sc->n[0]; d.n2 = sc->n[1]; d.n3 = sc->n[2];
  d.P1 = sc->P[0]; d.P2 = sc->P[1];
  if ((rc = tc_run(sc, tf32, 2, d, st))) return rc;
  set_target(e, sc, tf32, false);
  if ((rc = tc_run(sc, tf32, 3, e, st))) return rc;
  set_target(e, sc, tf32, true);
  if ((rc = tc_run(sc, tf32, 4, e, st))) return rc;
  TcEpilogue u;
  u.kind = 2;
  u.out = dest;
  u.accumulate = accumulate ? 1 : 0;
  u.n1 = sc->n[0]; u.n2 = sc->n[1]; u.n3 = sc->n[2];
  u.P1 = sc->P[0]; u.P2 = sc->P[1];
  return tc_run(sc, tf32, 5, u, st);
}

// First right-hand side of the mixed path: FP32 fold, stored into operand
// buffer A (split into BF16 planes, or as FP32).
static int fold_split(mf_solver3d* sc, bool tf32, const double* rhs, const double* bcs[3],
                      cudaStream_t st) {
  const long long n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const long long nf[3] = {n2 * n3, n1 * n3, n1 * n2};
  // x-face rows (j) padded to a multiple of 8 floats covering the padded
  // axis: the fold reads eight j of a row, up to P2 - 1, as two aligned float4
  const long long bxp = (std::max<long long>(n2, sc->P[1]) + 7) / 8 * 8, bxs = bxp * n3;
  const long long ps[3] = {bxs, nf[1], nf[2]};
  int rc;
  if ((rc = sc->foldf.ensure(sizeof(float) * 4 * (ps[0] + ps[1] + ps[2])))) return rc;
  float* f = sc->foldf.as<float>();
  float* fa[3] = {f, f + 4 * ps[0], f + 4 * (ps[0] + ps[1])};
  sc->prof.begin(kProfFold, st, 4);  // three face-product launches and the fold
  for (int a = 0; a < 3; ++a) {
    const AxisDev& d = sc->ax[a];
    const long long r = a == 0 ? n2 : nf[a], rp = a == 0 ? bxp : nf[a];
    k_fold_faces<<<blocks_for(nf[a], 256), 256, 0, st>>>(
        bcs[a], make_double4(d.bcc[0], d.bcc[1], d.bcc[2], d.bcc[3]), fa[a], nf[a], r, rp, ps[a]);
  }
  FoldArgsF args;
  for (int c = 0; c < 4; ++c) {
    args.ix[c] = sc->ax[0].invl4f.as<float>() + (size_t)c * n1;
    args.iy[c] = sc->ax[1].invl4f.as<float>() + (size_t)c * n2;
    args.iz[c] = sc->ax[2].invl4f.as<float>() + (size_t)c * n3;
  }
  args.bx = fa[0];
  args.by = fa[1];
  args.bz = fa[2];
  args.bxp = bxp;
  args.bxs = bxs;
  k_fold_split_rows<<<dim3(blocks_for(sc->P[0], 128), sc->P[1] / kFoldJ, kFoldKz), 128, 0, st>>>(
      rhs, args, tf32 ? nullptr : sc->Xa_hi.as<__nv_bfloat16>(),
      tf32 ? nullptr : sc->Xa_lo.as<__nv_bfloat16>(), tf32 ? sc->Xa32.as<float>() : nullptr,
      (int)n1, (int)n2, (int)n3, sc->P[0], sc->P[1], sc->P[2]);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

// A closed operator: every axis has exactly one null eigenvalue (Neumann at
// both ends), so the 3-D operator has a null mode at sigma = 0 and a
// near-null one at small sigma.  Its refinement residuals are formed in FP64
// (the FP32 residual update loses ~1e-9 relative on it: the low modes
// magnify the FP32 rounding of the residual), and at sigma = 0 they are
// projected (null_project).
static bool closed_operator(const mf_solver3d* sc) {
  return sc->ax[0].null_idx >= 0 && sc->ax[1].null_idx >= 0 && sc->ax[2].null_idx >= 0;
}

// Null coefficient c = l . r of r(i, j, k) = r[i + sy j + sz k], left in
// the device scalar returned through coef.
template <class T>
static int null_coef(mf_solver3d* sc, const T* r, long long sy, long long sz, const double** coef,
                     cudaStream_t st) {
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const int groups = (n2 + kNullRows - 1) / kNullRows;
  const int count = n3 * groups;
  int rc;
  if ((rc = sc->nullpart.ensure(sizeof(double) * (count + 1)))) return rc;
  double* part = sc->nullpart.as<double>();
  k_null_part<T><<<dim3(n3, groups), kNullThreads, 0, st>>>(r, sy, sz, sc->ax[0].null_row.as<double>(),
                                                            sc->ax[1].null_row.as<double>(),
                                                            sc->ax[2].null_row.as<double>(), n1, n2, part);
  k_null_sum<<<1, kNullThreads, 0, st>>>(part, count);
  *coef = part + count;
  return MF_OK;
}

// Dense FP64 residual r, minus its null-mode component when `project`,
// narrowed into the operand of the next approximate solve.
static int null_project(mf_solver3d* sc, const double* r, bool project, __nv_bfloat16* hi,
                        __nv_bfloat16* lo, float* x32, cudaStream_t st) {
  using T = double;
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const double* coef = nullptr;
  float* r32 = nullptr;
  int rc;
  sc->prof.begin(kProfNull, st, project ? 3 : 1);  // null_coef launches two kernels
  if (project && (rc = null_coef<T>(sc, r, n1, (long long)n1 * n2, &coef, st))) return rc;
  k_null_split<T><<<dim3(blocks_for(n1, 256), n2, std::min(n3, 16)), 256, 0, st>>>(
      r, coef, sc->ax[0].null_col.as<double>(), sc->ax[1].null_col.as<double>(),
      sc->ax[2].null_col.as<double>(), n1, n2, n3, sc->P[0], sc->P[1], hi, lo, x32, r32);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

// Removes the null-mode component of the interior of solf (in place).
static int null_remove(mf_solver3d* sc, double* solf, cudaStream_t st) {
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const long long sy = n1 + 2, sz = (long long)(n1 + 2) * (n2 + 2);
  double* u = solf + 1 + sy + sz;
  const double* coef = nullptr;
  int rc;
  sc->prof.begin(kProfNull, st, 3);
  if ((rc = null_coef<double>(sc, u, sy, sz, &coef, st))) return rc;
  k_null_remove<<<dim3(blocks_for(n1, 256), n2, std::min(n3, 16)), 256, 0, st>>>(
      u, sy, sz, coef, sc->ax[0].null_col.as<double>(), sc->ax[1].null_col.as<double>(),
      sc->ax[2].null_col.as<double>(), n1, n3);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

// Mixed-precision solve:
//   u1 = S~ (rhs - fold)                        (FP32 fold, tensor-core solve)
//   r1 = rhs - A u1                             (FP64 residual, boundary data)
//   C  = S~ r1;  for k >= 2: r_k = r1 - A C     (FP32 residual update)
//                            C += S~ r_k
//   solf = u1 + C                               (widened, summed in FP64)
// S~ is the approximate inverse by six tensor-core transforms (split-BF16
// or 3xTF32).  The cancellation in r_k = r1 - A C is relative to |r1|
// (~1e-5 |rhs|), so FP32 keeps it to ~1e-12 |rhs|; the FP64 residual of u1
// carries the accuracy.  On a closed operator (closed_operator) every
// residual is formed in FP64 (r_k = r1 - A C with r1 kept in FP64); at
// sigma = 0 each is projected (null_project) before it is narrowed, and the
// null component of the result is removed (null_remove).
static int solve_mixed_dev(mf_solver3d* sc, const double* rhs, double sigma, double* solf,
                           const double* bcs[3], int prec, int refine, cudaStream_t st) {
  if (prec != MF_PREC_SPLIT_BF16 && prec != MF_PREC_3XTF32)
    return set_error(MF_ERR_UNSUPPORTED, "precision mode %d is not available", prec);
  const bool tf32 = prec == MF_PREC_3XTF32;
  int rc;
  if ((rc = mixed_prepare(sc, tf32, st))) return rc;
  const int n1 = sc->n[0], n2 = sc->n[1], n3 = sc->n[2];
  const long long tot = (long long)n1 * n2 * n3;
  __nv_bfloat16* xh = tf32 ? nullptr : sc->Xa_hi.as<__nv_bfloat16>();
  __nv_bfloat16* xl = tf32 ? nullptr : sc->Xa_lo.as<__nv_bfloat16>();
  float* x32 = tf32 ? sc->Xa32.as<float>() : nullptr;
  float* u1 = sc->U32.as<float>();
  float* C = sc->C32.as<float>();
  const bool closed = closed_operator(sc), project = closed && std::fabs(sigma) < kNullThresh;
  if (closed && refine > 1 && (rc = sc->R1d.ensure(tot * 8))) return rc;
  if ((rc = fold_split(sc, tf32, rhs, bcs, st))) return rc;
  if ((rc = approx_solve(sc, tf32, sigma, u1, false, st))) return rc;
  for (int it = 0; it < refine; ++it) {
    if (closed) {
      // FP64 residuals: r1 = rhs - A u1 (kept in R1d when more steps follow),
      // r_k = r1 - A C; projected at sigma = 0, then narrowed
      double* r = (it == 0 && refine > 1) ? sc->R1d.as<double>() : sc->R.as<double>();
      if ((rc = residual_passes<double, float>(sc, it == 0 ? rhs : sc->R1d.as<double>(), it == 0 ? u1 : C,
                                               sigma, it == 0 ? bcs : nullptr, sc->R.as<double>(),
                                               sc->R2.as<double>(), r, (__nv_bfloat16*)nullptr,
                                               (__nv_bfloat16*)nullptr, (float*)nullptr, (float*)nullptr,
                                               kProfResidX, kProfResidYZ, st)) ||
          (rc = null_project(sc, r, project, xh, xl, x32, st)))
        return rc;
    } else if (it == 0) {
      // the FP32 copy of r1 only feeds later refinement steps
      if ((rc = residual_passes<double, float>(sc, rhs, u1, sigma, bcs, sc->R.as<double>(),
                                               sc->R2.as<double>(), (double*)nullptr, xh, xl, x32,
                                               refine > 1 ? sc->R1f.as<float>() : nullptr,
                                               kProfResidX, kProfResidYZ, st)))
        return rc;
    } else {
      float* f0 = reinterpret_cast<float*>(sc->R.ptr);
      float* f1 = reinterpret_cast<float*>(sc->R2.ptr);
      if ((rc = residual_passes<float, float>(sc, sc->R1f.as<float>(), C, sigma, nullptr, f0, f1,
                                              (float*)nullptr, xh, xl, x32, nullptr, kProfResid32,
                                              kProfResid32, st)))
        return rc;
    }
    if ((rc = approx_solve(sc, tf32, sigma, C, it > 0, st))) return rc;
  }
  sc->prof.begin(kProfCopy, st);
  k_finalize<<<dim3(blocks_for(n1, 256), n2, 4), 256, 0, st>>>(u1, refine > 0 ? C : nullptr, solf, n1,
                                                               n2, n3);
  sc->prof.end(st);
  MF_CUDA(cudaGetLastError());
  if (project && (rc = null_remove(sc, solf, st))) return rc;
  return faces(sc, solf, bcs, st);
}

// ---------------------------------------------------------------------------
int solver_axis_view(const ::mf_solver3d* sc, int axis, SolverAxisView* out) {
  if (!sc || !out || axis < 0 || axis > 2) return set_error(MF_ERR_ARG, "solver_axis_view: bad arguments");
  const AxisDev& d = sc->ax[axis];
  out->n = d.n;
  out->V = d.V.as<double>();
  out->Vinv = d.Vinv.as<double>();
  out->eig = d.eig.as<double>();
  out->invl4 = d.invl4.as<double>();
  for (int c = 0; c < 4; ++c) out->bcc[c] = d.bcc[c];
  out->bc[0] = d.bc[0];
  out->bc[1] = d.bc[1];
  for (int m = 0; m < 14; ++m) out->neum[m] = d.neum[m];
  return MF_OK;
}

// Allocation-free plain solve (mf_solve_3d_noalloc).
//
// For callers that cannot let a library call cudaMalloc: applications whose
// device memory is owned by their own pool allocator, which budgets every
// byte and forbids other allocations, and latency-bound host loops in which
// cudaMalloc's implicit device-wide synchronisation cannot be afforded.  The
// two FP64 work arrays of the plain path live in this fixed file-scope array
// instead of the handle's buffers.  Every GPU that loads the library holds
// it until exit.
constexpr long long kNoAllocMaxPoints = 1LL << 18;  // interior points n1*n2*n3 (64^3)
static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocMaxPoints];  // 4 MiB

// Device address of g_noalloc_scratch for the current device, looked up
// once per device by the first call on it (cudaGetSymbolAddress allocates
// nothing).
static int noalloc_scratch(double** out) {
  static std::mutex mu;
  static double* addr[64] = {nullptr};
  int dev = 0;
  MF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(MF_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    addr[dev] = static_cast<double*>(p);
  }
  *out = addr[dev];
  return MF_OK;
}

}  // namespace mf

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int mf_solver_coeffs_init_3d(const double* g1, const double* g2, const double* g3, int n1, int n2,
                             int n3, const int bct[6], int so, mf_solver3d_t** out) {
  if (!g1 || !g2 || !g3 || !bct || !out)
    return set_error(MF_ERR_ARG, "mf_solver_coeffs_init_3d: null argument");
  *out = nullptr;
  const double* grids[3] = {g1, g2, g3};
  const int nall[3] = {n1, n2, n3};
  SolverAxisHost host[3];
  for (int a = 0; a < 3; ++a) {
    std::string msg;
    int rc = solver_axis_setup(grids[a], nall[a], bct + 2 * a, so, host[a], msg);
    if (rc) return set_error(rc, "mf_solver_coeffs_init_3d: axis %d: %s", a, msg.c_str());
  }
  mf_solver3d* sc = new mf_solver3d();
  for (int a = 0; a < 3; ++a) {
    int rc = axis_upload(sc->ax[a], host[a]);
    if (rc) {
      mf_solver3d_destroy(sc);
      return rc;
    }
    sc->n[a] = host[a].n;
    sc->P[a] = sc->ax[a].P;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {  // uploads complete before use on any stream
    mf_solver3d_destroy(sc);
    return set_error(MF_ERR_CUDA, "mf_solver_coeffs_init_3d: upload failed");
  }
  *out = sc;
  return MF_OK;
}

int mf_solver3d_destroy(mf_solver3d_t* sc) {
  if (!sc) return MF_OK;
  for (int t = 0; t < 6; ++t) {
    tc_plan_destroy(sc->plan[t]);
    tc_plan_destroy(sc->plan32[t]);
  }
  for (auto& d : sc->ax) {
    for (DevBuf* b : {&d.V, &d.Vinv, &d.eig, &d.invl4, &d.rows, &d.Vh, &d.Vl, &d.Vih, &d.Vil,
                      &d.Vh32, &d.Vl32, &d.Vih32, &d.Vil32, &d.eigf, &d.nullf, &d.invl4f,
                      &d.rowsf, &d.tri, &d.null_row, &d.null_col})
      b->release();
  }
  for (DevBuf* b : {&sc->w0, &sc->w1, &sc->st_rhs, &sc->st_solf, &sc->st_bc[0], &sc->st_bc[1],
                    &sc->st_bc[2], &sc->R, &sc->R2, &sc->Xa_hi, &sc->Xa_lo, &sc->Xb_hi,
                    &sc->Xb_lo, &sc->Xa32, &sc->Xb32, &sc->err, &sc->foldf, &sc->U32, &sc->C32,
                    &sc->R1f, &sc->nullpart, &sc->R1d})
    b->release();
  for (int q = 0; q < kPipeSlots; ++q) {
    sc->pipe_rhs[q].release();
    sc->pipe_solf[q].release();
    for (int a = 0; a < 3; ++a) sc->pipe_bc[q][a].release();
    for (cudaEvent_t e : {sc->in_ready[q], sc->solved[q], sc->out_done[q]})
      if (e) cudaEventDestroy(e);
    if (sc->pipe_graph[q].exec) cudaGraphExecDestroy(sc->pipe_graph[q].exec);
  }
  if (sc->cin) cudaStreamDestroy(sc->cin);
  if (sc->cout) cudaStreamDestroy(sc->cout);
  if (sc->gcap) cudaStreamDestroy(sc->gcap);
  delete sc;
  return MF_OK;
}

}  // extern "C"

// Shared front end of the solve entry points: validates, stages host
// pointers, runs `body` on device pointers, copies solf back.
// Host solution array -> device staging buffer, edges only: of the
// (n1+2)(n2+2)(n3+2) field a solve writes the interior (the last transform's
// epilogue or k_finalize) and the face interiors (k_faces) before anything
// reads them, and leaves the 12 edge lines (corners included) as they were,
// as the reference's copy and boundary insert do.  So only the edges travel
// to the device (4 (N1 + N2 + N3) values instead of N1 N2 N3); the download
// of the whole array then returns the caller's edges unchanged.
static int stage_edges(DevBuf& buf, const double* src, int N1, int N2, int N3, cudaStream_t st) {
  const size_t e = sizeof(double);
  const long long P = (long long)N1 * N2;
  int rc;
  if ((rc = buf.ensure((size_t)P * N3 * e))) return rc;
  double* dst = buf.as<double>();
  for (int k : {0, N3 - 1})
    for (int j : {0, N2 - 1}) {  // x-edges: contiguous
      const long long off = (long long)j * N1 + (long long)k * P;
      MF_CUDA(cudaMemcpyAsync(dst + off, src + off, (size_t)N1 * e, cudaMemcpyDefault, st));
    }
  for (int k : {0, N3 - 1})
    for (int i : {0, N1 - 1}) {  // y-edges: stride N1
      const long long off = i + (long long)k * P;
      MF_CUDA(cudaMemcpy2DAsync(dst + off, (size_t)N1 * e, src + off, (size_t)N1 * e, e, (size_t)N2,
                                cudaMemcpyDefault, st));
    }
  for (int j : {0, N2 - 1})
    for (int i : {0, N1 - 1}) {  // z-edges: stride N1 N2
      const long long off = i + (long long)j * N1;
      MF_CUDA(cudaMemcpy2DAsync(dst + off, (size_t)P * e, src + off, (size_t)P * e, e, (size_t)N3,
                                cudaMemcpyDefault, st));
    }
  return MF_OK;
}

template <class Body>
static int solve_front(mf_solver3d_t* sc, const double* rhs, double* solf, const double* bcx,
                       const double* bcy, const double* bcz, int n1, int n2, int n3, void* stream,
                       Body body) {
  if (!sc || !rhs || !solf || !bcx || !bcy || !bcz)
    return set_error(MF_ERR_ARG, "solve_3d: null argument");
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "solve_3d: shape (%d,%d,%d) differs from the set-up (%d,%d,%d)",
                     n1, n2, n3, sc->n[0], sc->n[1], sc->n[2]);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t rb = (size_t)n1 * n2 * n3 * 8, sb = (size_t)(n1 + 2) * (n2 + 2) * (n3 + 2) * 8;
  const size_t bb[3] = {(size_t)n2 * n3 * 2 * 8, (size_t)n1 * n3 * 2 * 8, (size_t)n1 * n2 * 2 * 8};
  const double* bcs_in[3] = {bcx, bcy, bcz};
  const double* bcs[3];
  bool any_host = false;
  // Staging, solve and download; on an error part way, the copies already
  // queued from or to the caller's host arrays are waited for before the
  // error is returned.
  auto run = [&]() -> int {
    int rc;
    for (int a = 0; a < 3; ++a) {
      if (is_device_ptr(bcs_in[a])) {
        bcs[a] = bcs_in[a];
      } else {
        any_host = true;
        if ((rc = stage_in(sc->st_bc[a], bcs_in[a], bb[a], st))) return rc;
        bcs[a] = sc->st_bc[a].as<double>();
      }
    }
    const double* r = rhs;
    if (!is_device_ptr(rhs)) {
      any_host = true;
      if ((rc = stage_in(sc->st_rhs, rhs, rb, st))) return rc;
      r = sc->st_rhs.as<double>();
    }
    double* s = solf;
    const bool host_solf = !is_device_ptr(solf);
    if (host_solf) {
      any_host = true;
      if ((rc = stage_edges(sc->st_solf, solf, n1 + 2, n2 + 2, n3 + 2, st))) return rc;
      s = sc->st_solf.as<double>();
    }
    if ((rc = body(r, s, bcs, st))) return rc;
    if (host_solf) MF_CUDA(cudaMemcpyAsync(solf, s, sb, cudaMemcpyDeviceToHost, st));
    return MF_OK;
  };
  const int rc = run();
  if (rc) {
    if (any_host) cudaStreamSynchronize(st);
    return rc;
  }
  if (any_host) {
    MF_CUDA(cudaStreamSynchronize(st));
    if (sc->err.ptr) {
      int herr = 0;
      MF_CUDA(cudaMemcpy(&herr, sc->err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
      if (herr) return set_error(MF_ERR_TIMEOUT, "solve_3d: a tensor-core pipeline wait expired");
    }
  }
  return MF_OK;
}

extern "C" {

int mf_solve_3d(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                const double* bcx, const double* bcy, const double* bcz, int n1, int n2, int n3,
                void* stream) {
  return solve_front(sc, rhs, solf, bcx, bcy, bcz, n1, n2, n3, stream,
                     [&](const double* r, double* s, const double** bcs, cudaStream_t st) {
                       return solve_plain_dev(sc, r, sigma, s, bcs, st);
                     });
}

int mf_solve_3d_batch(mf_solver3d_t* sc, int count, const double* rhs, long long rhs_stride, double sigma,
                      double* solf, long long solf_stride, const double* bcx, long long bcx_stride,
                      const double* bcy, long long bcy_stride, const double* bcz, long long bcz_stride,
                      int n1, int n2, int n3, void* stream) {
  if (!sc || !rhs || !solf || !bcx || !bcy || !bcz || count < 1 || count > 65535 || rhs_stride < 0 ||
      bcx_stride < 0 || bcy_stride < 0 || bcz_stride < 0)
    return set_error(MF_ERR_ARG, "mf_solve_3d_batch: bad arguments");
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "mf_solve_3d_batch: shape (%d,%d,%d) differs from the set-up (%d,%d,%d)", n1,
                     n2, n3, sc->n[0], sc->n[1], sc->n[2]);
  const long long sfull = (long long)(n1 + 2) * (n2 + 2) * (n3 + 2);
  if (count > 1 && solf_stride < sfull)
    return set_error(MF_ERR_ARG, "mf_solve_3d_batch: solutions overlap (stride %lld < %lld)", solf_stride, sfull);
  for (const void* p : {(const void*)rhs, (const void*)solf, (const void*)bcx, (const void*)bcy, (const void*)bcz})
    if (!is_device_ptr(p)) return set_error(MF_ERR_ARG, "mf_solve_3d_batch: device arrays required");
  const double* bcs[3] = {bcx, bcy, bcz};
  const long long sb[3] = {bcx_stride, bcy_stride, bcz_stride};
  return solve_plain_batch(sc, count, rhs, rhs_stride, sigma, solf, solf_stride, bcs, sb,
                           static_cast<cudaStream_t>(stream));
}

int mf_solve_3d_mixed(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                      const double* bcx, const double* bcy, const double* bcz, int n1, int n2,
                      int n3, int precision, int refine, void* stream) {
  if (precision == MF_PREC_FP64)
    return mf_solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz, n1, n2, n3, stream);
  if (refine < 0) refine = 2;
  return solve_front(sc, rhs, solf, bcx, bcy, bcz, n1, n2, n3, stream,
                     [&](const double* r, double* s, const double** bcs, cudaStream_t st) {
                       return solve_mixed_dev(sc, r, sigma, s, bcs, precision, refine, st);
                     });
}

int mf_solve_3d_mixed_many(mf_solver3d_t* sc, int count, const double* const* rhs, double sigma,
                           double* const* solf, const double* const* bcx, const double* const* bcy,
                           const double* const* bcz, int n1, int n2, int n3, int precision, int refine,
                           void* stream) {
  if (!sc || count < 1 || !rhs || !solf || !bcx || !bcy || !bcz)
    return set_error(MF_ERR_ARG, "mf_solve_3d_mixed_many: bad arguments");
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "mf_solve_3d_mixed_many: shape (%d,%d,%d) differs from the set-up", n1, n2, n3);
  for (int b = 0; b < count; ++b)
    if (!rhs[b] || !solf[b] || !bcx[b] || !bcy[b] || !bcz[b])
      return set_error(MF_ERR_ARG, "mf_solve_3d_mixed_many: null array in problem %d", b);
  if (refine < 0) refine = 2;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t rb = (size_t)n1 * n2 * n3 * 8, sb = (size_t)(n1 + 2) * (n2 + 2) * (n3 + 2) * 8;
  const size_t bb[3] = {(size_t)n2 * n3 * 2 * 8, (size_t)n1 * n3 * 2 * 8, (size_t)n1 * n2 * 2 * 8};
  int rc;
  if (!sc->cin) {
    MF_CUDA(cudaStreamCreateWithFlags(&sc->cin, cudaStreamNonBlocking));
    MF_CUDA(cudaStreamCreateWithFlags(&sc->cout, cudaStreamNonBlocking));
    for (int q = 0; q < kPipeSlots; ++q)
      for (cudaEvent_t* e : {&sc->in_ready[q], &sc->solved[q], &sc->out_done[q]})
        MF_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  for (int q = 0; q < kPipeSlots; ++q) {
    if ((rc = sc->pipe_rhs[q].ensure(rb)) || (rc = sc->pipe_solf[q].ensure(sb))) return rc;
    for (int a = 0; a < 3; ++a)
      if ((rc = sc->pipe_bc[q][a].ensure(bb[a]))) return rc;
  }
  // Every copy and solve of the call is queued by `queue`; if it fails part
  // way, the copies already queued (downloads into the caller's arrays
  // among them) are waited for before the error is returned.
  auto queue = [&]() -> int {
    // the copy streams start after the work already queued on the caller's stream
    MF_CUDA(cudaEventRecord(sc->solved[0], st));
    MF_CUDA(cudaStreamWaitEvent(sc->cin, sc->solved[0], 0));
    const double* const* bsrc[3] = {bcx, bcy, bcz};
    for (int b = 0; b < count; ++b) {
      const int q = b % kPipeSlots;
      if (b >= kPipeSlots) {  // slot q is free once problem b - kPipeSlots is solved and downloaded
        MF_CUDA(cudaStreamWaitEvent(sc->cin, sc->solved[q], 0));
        MF_CUDA(cudaStreamWaitEvent(sc->cin, sc->out_done[q], 0));
      }
      MF_CUDA(cudaMemcpyAsync(sc->pipe_rhs[q].ptr, rhs[b], rb, cudaMemcpyDefault, sc->cin));
      if (is_device_ptr(solf[b])) {
        MF_CUDA(cudaMemcpyAsync(sc->pipe_solf[q].ptr, solf[b], sb, cudaMemcpyDefault, sc->cin));
      } else if ((rc = stage_edges(sc->pipe_solf[q], solf[b], n1 + 2, n2 + 2, n3 + 2, sc->cin))) {
        return rc;
      }
      const double* bcs[3];
      for (int a = 0; a < 3; ++a) {
        MF_CUDA(cudaMemcpyAsync(sc->pipe_bc[q][a].ptr, bsrc[a][b], bb[a], cudaMemcpyDefault, sc->cin));
        bcs[a] = sc->pipe_bc[q][a].as<double>();
      }
      MF_CUDA(cudaEventRecord(sc->in_ready[q], sc->cin));
      MF_CUDA(cudaStreamWaitEvent(st, sc->in_ready[q], 0));
      double* s = sc->pipe_solf[q].as<double>();
      if (precision != MF_PREC_FP64 && b > 0 && !sc->prof.on) {
        // Mixed solves after the first of the call (which has made every
        // buffer and plan these settings need) replay the slot's graph,
        // captured on first use or when a setting changed; a capture that
        // fails leaves the eager launches below to do the work.
        mf_solver3d::PipeGraph& G = sc->pipe_graph[q];
        const int plan = tc_get_tf32_plan(), tmode = tune_mode();
        if (!G.exec || G.sigma != sigma || G.precision != precision || G.refine != refine || G.plan != plan ||
            G.tune != tmode || G.resid != sc->resid_mode) {
          if (G.exec) {
            MF_CUDA(cudaGraphExecDestroy(G.exec));
            G.exec = nullptr;
          }
          if (!sc->gcap) MF_CUDA(cudaStreamCreateWithFlags(&sc->gcap, cudaStreamNonBlocking));
          if (cudaStreamBeginCapture(sc->gcap, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
            const int crc = solve_mixed_dev(sc, sc->pipe_rhs[q].as<double>(), sigma, s, bcs, precision, refine,
                                            sc->gcap);
            cudaGraph_t graph = nullptr;
            const cudaError_t e = cudaStreamEndCapture(sc->gcap, &graph);
            if (crc == MF_OK && e == cudaSuccess && graph &&
                cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess) {
              G.sigma = sigma;
              G.precision = precision;
              G.refine = refine;
              G.plan = plan;
              G.tune = tmode;
              G.resid = sc->resid_mode;
            } else {
              G.exec = nullptr;
            }
            if (graph) cudaGraphDestroy(graph);
            (void)cudaGetLastError();
          } else {
            (void)cudaGetLastError();
          }
        }
        if (G.exec) {
          MF_CUDA(cudaGraphLaunch(G.exec, st));
          MF_CUDA(cudaEventRecord(sc->solved[q], st));
          MF_CUDA(cudaStreamWaitEvent(sc->cout, sc->solved[q], 0));
          MF_CUDA(cudaMemcpyAsync(solf[b], s, sb, cudaMemcpyDefault, sc->cout));
          MF_CUDA(cudaEventRecord(sc->out_done[q], sc->cout));
          continue;
        }
      }
      rc = precision == MF_PREC_FP64
               ? solve_plain_dev(sc, sc->pipe_rhs[q].as<double>(), sigma, s, bcs, st)
               : solve_mixed_dev(sc, sc->pipe_rhs[q].as<double>(), sigma, s, bcs, precision, refine, st);
      if (rc) return rc;
      MF_CUDA(cudaEventRecord(sc->solved[q], st));
      MF_CUDA(cudaStreamWaitEvent(sc->cout, sc->solved[q], 0));
      MF_CUDA(cudaMemcpyAsync(solf[b], s, sb, cudaMemcpyDefault, sc->cout));
      MF_CUDA(cudaEventRecord(sc->out_done[q], sc->cout));
    }
    return MF_OK;
  };
  if ((rc = queue())) {
    cudaStreamSynchronize(sc->cin);
    cudaStreamSynchronize(sc->cout);
    cudaStreamSynchronize(st);
    return rc;
  }
  MF_CUDA(cudaStreamSynchronize(sc->cout));
  MF_CUDA(cudaStreamSynchronize(st));
  if (sc->err.ptr) {
    int herr = 0;
    MF_CUDA(cudaMemcpy(&herr, sc->err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return set_error(MF_ERR_TIMEOUT, "solve_3d: a tensor-core pipeline wait expired");
  }
  return MF_OK;
}

int mf_solver_3d(mf_solver3d_t* sc, const double* g, double* u, const double* bcx,
                 const double* bcy, const double* bcz, int nx, int ny, int nz, double sigma,
                 int precision, void* stream) {
  if (!sc || !g || !u) return set_error(MF_ERR_ARG, "mf_solver_3d: null argument");
  const int n1 = nx - 2, n2 = ny - 2, n3 = nz - 2;
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "mf_solver_3d: field (%d,%d,%d) does not match the set-up", nx, ny, nz);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long tot = (long long)n1 * n2 * n3;
  int rc;
  // interior of g -> contiguous rhs (class_field.f90:1092-1098)
  DevBuf& gr = sc->st_rhs;
  const double* gd = g;
  DevBuf gstage;
  if (!is_device_ptr(g)) {
    if ((rc = stage_in(gstage, g, (size_t)nx * ny * nz * 8, st))) return rc;
    gd = gstage.as<double>();
  }
  if ((rc = gr.ensure(tot * 8))) { gstage.release(); return rc; }
  k_extract_interior<<<blocks_for(tot, 256), 256, 0, st>>>(gd, gr.as<double>(), n1, n2, n3);
  if (cudaGetLastError() != cudaSuccess) { gstage.release(); return set_error(MF_ERR_CUDA, "extract"); }
  rc = (precision == MF_PREC_FP64)
           ? mf_solve_3d(sc, gr.as<double>(), sigma, u, bcx, bcy, bcz, n1, n2, n3, stream)
           : mf_solve_3d_mixed(sc, gr.as<double>(), sigma, u, bcx, bcy, bcz, n1, n2, n3, precision,
                               -1, stream);
  if (gstage.ptr) {
    cudaStreamSynchronize(st);
    gstage.release();
  }
  return rc;
}

int mf_solve_3d_noalloc(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                        const double* bcx, const double* bcy, const double* bcz, int n1, int n2,
                        int n3, void* stream) {
  if (!sc || !rhs || !solf || !bcx || !bcy || !bcz)
    return set_error(MF_ERR_ARG, "mf_solve_3d_noalloc: null argument");
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "mf_solve_3d_noalloc: shape (%d,%d,%d) differs from the set-up (%d,%d,%d)",
                     n1, n2, n3, sc->n[0], sc->n[1], sc->n[2]);
  const long long tot = (long long)n1 * n2 * n3;
  if (tot > kNoAllocMaxPoints)
    return set_error(MF_ERR_UNSUPPORTED,
                     "mf_solve_3d_noalloc: %lld interior points exceed the fixed scratch of %lld "
                     "points (use mf_solve_3d)", tot, kNoAllocMaxPoints);
  for (const void* p : {(const void*)rhs, (const void*)solf, (const void*)bcx, (const void*)bcy,
                        (const void*)bcz})
    if (!is_device_ptr(p))
      return set_error(MF_ERR_ARG, "mf_solve_3d_noalloc: device pointers only (host data needs staging buffers)");
  double* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // every entry of both work arrays is written before it is read, so the
  // previous call's contents need no clearing
  double* w0 = scratch;
  double* w1 = scratch + kNoAllocMaxPoints;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double* bcs[3] = {bcx, bcy, bcz};
  k_fold<<<blocks_for(tot, 256), 256, 0, st>>>(rhs, w0, bcx, bcy, bcz, fold_args(sc), n1, n2, n3);
  MF_CUDA(cudaGetLastError());
  StageProfiler off;  // no event timers on this path
  GemmEpi plain;
  const double* Vi[3] = {sc->ax[0].Vinv.as<double>(), sc->ax[1].Vinv.as<double>(),
                         sc->ax[2].Vinv.as<double>()};
  const double* Vf[3] = {sc->ax[0].V.as<double>(), sc->ax[1].V.as<double>(),
                         sc->ax[2].V.as<double>()};
  if ((rc = gemm_f64(off, w0, n2 * n3, n1, Vi[0], n1, w1, plain, st, 1, 0, 0, false))) return rc;
  if ((rc = gemm_f64(off, w1, n3 * n1, n2, Vi[1], n2, w0, plain, st, 1, 0, 0, false))) return rc;
  GemmEpi div;
  div.kind = 1;
  div.lx = sc->ax[0].eig.as<double>();
  div.ly = sc->ax[1].eig.as<double>();
  div.lz = sc->ax[2].eig.as<double>();
  div.sigma = sigma;
  div.thresh = kNullThresh;
  div.n1 = n1;
  div.n2 = n2;
  if ((rc = gemm_f64(off, w0, n1 * n2, n3, Vi[2], n3, w1, div, st, 1, 0, 0, false))) return rc;
  if ((rc = gemm_f64(off, w1, n2 * n3, n1, Vf[0], n1, w0, plain, st, 1, 0, 0, false))) return rc;
  if ((rc = gemm_f64(off, w0, n3 * n1, n2, Vf[1], n2, w1, plain, st, 1, 0, 0, false))) return rc;
  GemmEpi out;
  out.kind = 2;
  out.n1 = n1;
  out.n2 = n2;
  if ((rc = gemm_f64(off, w1, n1 * n2, n3, Vf[2], n3, solf, out, st, 1, 0, 0, false))) return rc;
  const long long p1 = n1 + 2, p2 = n2 + 2;
  for (int axis = 0; axis < 3; ++axis) {
    const AxisDev& d = sc->ax[axis];
    FaceArgs f;
    if (axis == 0) { f.sA = 1; f.sa = p1; f.sb = p1 * p2; f.n = n1; f.na = n2; f.nb = n3; }
    if (axis == 1) { f.sA = p1; f.sa = 1; f.sb = p1 * p2; f.n = n2; f.na = n1; f.nb = n3; }
    if (axis == 2) { f.sA = p1 * p2; f.sa = 1; f.sb = p1; f.n = n3; f.na = n1; f.nb = n2; }
    f.bc0 = d.bc[0];
    f.bc1 = d.bc[1];
    for (int m = 0; m < 7; ++m) { f.nl[m] = d.neum[m]; f.nr[m] = d.neum[7 + m]; }
    k_faces<<<blocks_for((long long)f.na * f.nb, 128), 128, 0, st>>>(solf, bcs[axis], f);
    MF_CUDA(cudaGetLastError());
  }
  return MF_OK;
}

}  // extern "C"

// The staging slots' graphs of mf_solve_3d_mixed_many were captured with the
// set-up's device pointers and the launch parameters derived from it (the
// null-mode projection of a closed operator, its rows and columns); new
// tables can release or change those, so the graphs are captured again.
static void drop_pipe_graphs(mf_solver3d* sc) {
  for (auto& G : sc->pipe_graph)
    if (G.exec) {
      cudaGraphExecDestroy(G.exec);
      G.exec = nullptr;
    }
}

extern "C" {

int mf_solver3d_set_eigen(mf_solver3d_t* sc, int axis, const double* eigen, const double* vect,
                          const double* inv_vect) {
  if (!sc || !eigen || !vect || !inv_vect || axis < 0 || axis > 2)
    return set_error(MF_ERR_ARG, "mf_solver3d_set_eigen: bad arguments");
  AxisDev& d = sc->ax[axis];
  const int n = d.n;
  std::vector<double> e(n), vc((size_t)n * n), ic((size_t)n * n);
  auto fetch = [&](const double* src, double* dst, size_t count) -> int {
    if (is_device_ptr(src)) {
      MF_CUDA(cudaMemcpy(dst, src, count * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      std::memcpy(dst, src, count * sizeof(double));
    }
    return MF_OK;
  };
  int rc;
  if ((rc = fetch(eigen, e.data(), n)) || (rc = fetch(vect, vc.data(), (size_t)n * n)) ||
      (rc = fetch(inv_vect, ic.data(), (size_t)n * n)))
    return rc;
  std::vector<double> V((size_t)n * n), Vi((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      V[(size_t)i * n + j] = vc[i + (size_t)n * j];
      Vi[(size_t)i * n + j] = ic[i + (size_t)n * j];
    }
  MF_CUDA(cudaDeviceSynchronize());
  drop_pipe_graphs(sc);
  if ((rc = axis_set_eigen(d, e, V, Vi))) return rc;
  MF_CUDA(cudaDeviceSynchronize());  // uploads complete before use on any stream
  return MF_OK;
}

int mf_solver3d_set_residual(mf_solver3d_t* sc, int mode) {
  if (!sc || (mode != MF_RESID_FF && mode != MF_RESID_FP64 && mode != MF_RESID_FP64_LINE))
    return set_error(MF_ERR_ARG, "mf_solver3d_set_residual: bad arguments");
  sc->resid_mode = mode;
  return MF_OK;
}

int mf_solver3d_device_status(mf_solver3d_t* sc) {
  if (!sc) return set_error(MF_ERR_ARG, "mf_solver3d_device_status: null handle");
  if (!sc->err.ptr) return MF_OK;
  MF_CUDA(cudaDeviceSynchronize());
  int herr = 0;
  MF_CUDA(cudaMemcpy(&herr, sc->err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  MF_CUDA(cudaMemset(sc->err.ptr, 0, sizeof(int)));
  MF_CUDA(cudaDeviceSynchronize());  // later work on non-blocking streams sees the reset
  if (herr) return set_error(MF_ERR_TIMEOUT, "tensor-core pipeline wait expired");
  return MF_OK;
}

int mf_solver3d_profile(mf_solver3d_t* sc, int enable) {
  if (!sc) return set_error(MF_ERR_ARG, "mf_solver3d_profile: null handle");
  sc->prof.reset();
  sc->prof.on = enable != 0;
  return MF_OK;
}

int mf_solver3d_profile_read(mf_solver3d_t* sc, int kind, double* total_ms, long long* launches) {
  if (!sc || !total_ms || !launches || kind < 0 || kind >= StageProfiler::kKinds)
    return set_error(MF_ERR_ARG, "mf_solver3d_profile_read: bad arguments");
  sc->prof.collect();
  *total_ms = sc->prof.total_ms[kind];
  *launches = sc->prof.launches[kind];
  return MF_OK;
}

int mf_solver_residual(mf_solver3d_t* sc, const double* g, const double* u, double sigma,
                       const double* bcx, const double* bcy, const double* bcz, double* r, int n1,
                       int n2, int n3, void* stream) {
  if (!sc || !g || !u || !bcx || !bcy || !bcz || !r)
    return set_error(MF_ERR_ARG, "mf_solver_residual: null argument");
  if (n1 != sc->n[0] || n2 != sc->n[1] || n3 != sc->n[2])
    return set_error(MF_ERR_ARG, "mf_solver_residual: shape mismatch");
  for (const void* p : {(const void*)g, (const void*)u, (const void*)bcx, (const void*)bcy,
                        (const void*)bcz, (const void*)r})
    if (!is_device_ptr(p)) return set_error(MF_ERR_ARG, "mf_solver_residual: device pointers only");
  int rc;
  const size_t tb = (size_t)n1 * n2 * n3 * 8;
  if ((rc = sc->R.ensure(tb)) || (rc = sc->R2.ensure(tb))) return rc;
  const double* bcs[3] = {bcx, bcy, bcz};
  return residual_passes<double, double>(sc, g, u, sigma, bcs, sc->R.as<double>(),
                                        sc->R2.as<double>(), r, nullptr, nullptr, nullptr, nullptr,
                                        kProfResidX, kProfResidYZ, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
