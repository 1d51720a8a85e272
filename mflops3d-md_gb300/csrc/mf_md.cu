// Influence-matrix multidomain coupling, every subdomain resident on one GPU.
//
// Reference path: multidomain_solve (class_field.f90:1295-1388) with the
// interface topology of md_influence_matrix_param (class_md.f90:1450-1680),
// the Dirac-column assembly of md_influence_matrix_set (class_field.f90:
// 1396-1510, class_md.f90:1049-1095), the rhs gather / solution scatter of
// md_vector_setvalues / md_vector_getvalues (class_md.f90:663-708,445-550)
// and the interface solve of md_solve (class_md.f90:379-438).
//
// GB300 form: the MPI ranks of the reference become subdomain handles on one
// device; the neighbour exchange becomes a gather of signed face derivatives
// into the interface vector and a scatter of the interface solution into the
// subdomains' boundary arrays (device kernels).  The PETSc KSP is replaced by
// a dense FP64 LU factorised once (cuSOLVER getrf at set-up).  Up to 12,000
// unknowns the inverse is formed from it (getrs against the identity) and a
// solve is one FP64 matrix-vector product; above that the two factors are
// inverted in place (trtri, a third of the inverse's flops) and a solve is two
// row-parallel triangular products.  Either way a solve reads n x n FP64 once
// at HBM rate, instead of two triangular solves whose rows depend on one
// another.  The blocked triangular solves on the LU factors remain as the
// path used when neither fits in device memory.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mf_internal.h"

namespace mf {

// Host restatement of the interface numbering (class_md.f90:1450-1680).
// dm[((((i*nd2)+j)*nd3+k)*3+l)*2+m]: interface id (1-based, -1 none) of face
// l side m of subdomain (i,j,k); kind/size/offset per interface.
struct MdTopology {
  int nd[3] = {1, 1, 1};
  int periods[3] = {0, 0, 0};
  std::vector<int> dm, kind, size, offset;
  int it = 0;
  long long ninf = 0;
  int& at(int i, int j, int k, int l, int m) {
    return dm[((((size_t)i * nd[1] + j) * nd[2] + k) * 3 + l) * 2 + m];
  }
  int get(int i, int j, int k, int l, int m) const {
    return dm[((((size_t)i * nd[1] + j) * nd[2] + k) * 3 + l) * 2 + m];
  }
};

static int topology_build(const int nd[3], const int periods[3], const int* const nint[3],
                          MdTopology& t) {
  for (int l = 0; l < 3; ++l) {
    if (nd[l] < 1) return set_error(MF_ERR_ARG, "md topology: nd must be >= 1");
    t.nd[l] = nd[l];
    t.periods[l] = periods[l] ? 1 : 0;
  }
  t.dm.assign((size_t)nd[0] * nd[1] * nd[2] * 6, -1);
  t.kind.clear();
  int count = 0;
  for (int i = 0; i < nd[0]; ++i)
    for (int j = 0; j < nd[1]; ++j)
      for (int k = 0; k < nd[2]; ++k) {
        const int idx[3] = {i, j, k};
        for (int l = 0; l < 3; ++l)
          if (idx[l] < nd[l] - 1 || t.periods[l]) {
            t.at(i, j, k, l, 1) = ++count;
            t.kind.push_back(l);
          }
      }
  // left face = right face of the left neighbour (periodic wrap)
  for (int i = 0; i < nd[0]; ++i)
    for (int j = 0; j < nd[1]; ++j)
      for (int k = 0; k < nd[2]; ++k) {
        const int idx[3] = {i, j, k};
        for (int l = 0; l < 3; ++l) {
          int nb[3] = {i, j, k};
          if (idx[l] > 0) {
            nb[l] = idx[l] - 1;
          } else if (t.periods[l]) {
            nb[l] = nd[l] - 1;
          } else {
            continue;
          }
          t.at(i, j, k, l, 0) = t.get(nb[0], nb[1], nb[2], l, 1);
        }
      }
  t.it = count;
  t.size.assign(count, 0);
  for (int i = 0; i < nd[0]; ++i)
    for (int j = 0; j < nd[1]; ++j)
      for (int k = 0; k < nd[2]; ++k)
        for (int l = 0; l < 3; ++l) {
          const int p = t.get(i, j, k, l, 1);
          if (p <= 0) continue;
          const int n[3] = {nint[0][i], nint[1][j], nint[2][k]};
          const int a = l == 0 ? 1 : 0, b = l == 2 ? 1 : 2;
          t.size[p - 1] = n[a] * n[b];
        }
  t.offset.assign(count, 0);
  long long acc = 0;
  for (int p = 0; p < count; ++p) {
    t.offset[p] = (int)acc;
    acc += t.size[p];
  }
  t.ninf = acc;
  if (acc >= (1LL << 31)) return set_error(MF_ERR_UNSUPPORTED, "md topology: interface too large");
  return MF_OK;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Signed normal derivatives of one face into a target vector:
//   out[row0 + q] += scale * (m == 0 ? -1 : +1) * du(face node q)
// q runs over the face interior points in Fortran order of the face array.
struct FaceGather {
  int l, m;             // face axis and side
  int nx, ny, nz;       // subdomain nodes
  long long row0;       // first row of the interface
  double scale;
};

// Signed face derivatives of u added into the interface vector, from the
// face rows of the line's derivative operator: for each line of the face
// grid, du_0 = sum_r W[r] u_r and du_{L-1} = sum_r W[L + r] u_r (plain lines,
// the operator the influence matrix is assembled with), kDotLanes lanes per
// line and a shuffle reduction.  row0[m] < 0: side m is not an interface.
// One read of the field per axis instead of a full derivative sweep whose
// interior rows are not used.
struct FaceDot {
  int l;                // face axis
  int nx, ny, nz;       // subdomain nodes
  long long row0[2];    // first interface row of sides 0 and 1, or -1
  double scale;
};
constexpr int kDotLanes = 8;
__global__ void k_face_dot(const double* __restrict__ u, const double* __restrict__ W, double* out,
                           FaceDot f) {
  const int na = (f.l == 0 ? f.ny : f.nx) - 2;
  const int nb = (f.l == 2 ? f.ny : f.nz) - 2;
  const int L = f.l == 0 ? f.nx : f.l == 1 ? f.ny : f.nz;
  const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / kDotLanes;
  const int sub = threadIdx.x % kDotLanes;
  const bool live = q < (long long)na * nb;
  double lo = 0.0, hi = 0.0;
  if (live) {
    const int a = (int)(q % na) + 1, b = (int)(q / na) + 1;
    long long base, s;
    if (f.l == 0) { base = (long long)f.nx * (a + (long long)f.ny * b); s = 1; }
    else if (f.l == 1) { base = a + (long long)f.nx * f.ny * b; s = f.nx; }
    else { base = a + (long long)f.nx * b; s = (long long)f.nx * f.ny; }
    for (int r = sub; r < L; r += kDotLanes) {
      const double v = u[base + r * s];
      lo = fma(W[r], v, lo);
      hi = fma(W[L + r], v, hi);
    }
  }
#pragma unroll
  for (int off = kDotLanes / 2; off > 0; off >>= 1) {
    lo += __shfl_xor_sync(0xffffffffu, lo, off);
    hi += __shfl_xor_sync(0xffffffffu, hi, off);
  }
  if (!live || sub != 0) return;
  // atomic: the two subdomains of an interface may add concurrently; two
  // additions onto the zeroed vector give the same sum in either order
  if (f.row0[0] >= 0) atomicAdd(out + f.row0[0] + q, -f.scale * lo);
  if (f.row0[1] >= 0) atomicAdd(out + f.row0[1] + q, f.scale * hi);
}

// Batched influence columns: problem b has a unit value at point q0 + b of
// side m of a face array with nf points per side (all else zero).
__global__ void k_dirac_batch(double* bc, long long nf, int m, long long q0, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  bc[(long long)b * 2 * nf + (long long)m * nf + q0 + b] = 1.0;
}

// Signed face values of B derivative fields (the Dirac-column assembly):
// problem blockIdx.y reads du + y * du_stride and adds into out + y *
// out_stride; face point q of side m of axis l, negated on side 0.
__global__ void k_face_gather_batch(const double* __restrict__ du, long long du_stride, double* out,
                                    long long out_stride, FaceGather f) {
  const int na = (f.l == 0 ? f.ny : f.nx) - 2;
  const int nb = (f.l == 2 ? f.ny : f.nz) - 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= na * nb) return;
  du += blockIdx.y * du_stride;
  out += blockIdx.y * out_stride;
  const int a = q % na + 1, b = q / na + 1;
  int i, j, k;
  if (f.l == 0) { i = f.m ? f.nx - 1 : 0; j = a; k = b; }
  else if (f.l == 1) { i = a; j = f.m ? f.ny - 1 : 0; k = b; }
  else { i = a; j = b; k = f.m ? f.nz - 1 : 0; }
  const double v = du[i + (long long)f.nx * (j + (long long)f.ny * k)];
  out[f.row0 + q] += f.scale * (f.m ? v : -v);
}

// bc face (l, m) of a subdomain: copy from the caller's array, then the
// interface faces get either 0 or the interface solution.
__global__ void k_face_set(double* bc, long long nf, int m, const double* __restrict__ src,
                           long long row0, int mode, double dirac_q) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nf) return;
  double v = 0.0;
  if (mode == 1) v = src[row0 + q];          // interface value
  if (mode == 2) v = (q == (long long)dirac_q) ? 1.0 : 0.0;  // Dirac column
  bc[q + nf * m] = v;
}

// Triangular solves with the LU factor (column-major n x n, unit lower L,
// upper U) on one right-hand side, in blocks of kTriBlock rows.
//  * The row interchanges of getrf are turned into one permutation at set-up
//    and applied as a parallel gather (k_permute), instead of n dependent
//    swaps.
//  * The inverses of the diagonal blocks of L and U are formed at set-up
//    (k_tri_block_inverse), so a block step is one launch (k_tri_step):
//    every CTA forms s_k = inv(D_k) v_k (a 128 x 128 product from L2), CTA 0
//    stores it, and each thread updates one row of the trailing part,
//    v_r -= sum_c T(r, k0 + c) s_k[c], reading the factor once, coalesced.
constexpr int kTriBlock = 128;

__global__ void k_permute(const double* __restrict__ x, const int* __restrict__ perm, double* __restrict__ y,
                          int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[perm[i]];
}

// Inverse of diagonal block b (rows/columns k0 = b kTriBlock ... k0 + nb) of
// L (upper = 0, unit diagonal) or U (upper = 1), by right-looking
// elimination on the identity in shared memory; out = column-major
// kTriBlock x kTriBlock per block.  One CTA per block.
__global__ void __launch_bounds__(256) k_tri_block_inverse(const double* __restrict__ A, int n, int upper,
                                                           double* __restrict__ out) {
  extern __shared__ double X[];  // kTriBlock x kTriBlock, row r at X[r * kTriBlock]
  const int k0 = blockIdx.x * kTriBlock, nb = min(kTriBlock, n - k0);
  for (int t = threadIdx.x; t < kTriBlock * kTriBlock; t += blockDim.x)
    X[t] = (t / kTriBlock == t % kTriBlock && t / kTriBlock < nb) ? 1.0 : 0.0;
  __syncthreads();
  if (!upper) {
    for (int c = 0; c < nb; ++c) {  // row c final; rows below: X[r,:] -= L[r,c] X[c,:]
      for (int t = threadIdx.x; t < (nb - c - 1) * (c + 1); t += blockDim.x) {
        const int r = c + 1 + t / (c + 1), j = t % (c + 1);
        X[r * kTriBlock + j] -= A[(k0 + r) + (long long)n * (k0 + c)] * X[c * kTriBlock + j];
      }
      __syncthreads();
    }
  } else {
    for (int c = nb - 1; c >= 0; --c) {  // X[c,:] /= U[c,c]; rows above: X[r,:] -= U[r,c] X[c,:]
      const double d = A[(k0 + c) + (long long)n * (k0 + c)];
      for (int j = c + threadIdx.x; j < nb; j += blockDim.x) X[c * kTriBlock + j] = X[c * kTriBlock + j] / d;
      __syncthreads();
      for (int t = threadIdx.x; t < c * (nb - c); t += blockDim.x) {
        const int r = t / (nb - c), j = c + t % (nb - c);
        X[r * kTriBlock + j] -= A[(k0 + r) + (long long)n * (k0 + c)] * X[c * kTriBlock + j];
      }
      __syncthreads();
    }
  }
  double* o = out + (size_t)blockIdx.x * kTriBlock * kTriBlock;
  for (int t = threadIdx.x; t < kTriBlock * kTriBlock; t += blockDim.x) {
    const int r = t % kTriBlock, c = t / kTriBlock;  // column-major store
    o[t] = X[r * kTriBlock + c];
  }
}

// sol[k0 + r] = (Dinv v[k0 : k0 + nb])_r: the first block of a triangular
// solve (one CTA).
__global__ void __launch_bounds__(128) k_tri_first(const double* __restrict__ Dinv, const double* __restrict__ v,
                                                   double* __restrict__ sol, int k0, int nb) {
  __shared__ double xs[kTriBlock];
  for (int t = threadIdx.x; t < nb; t += blockDim.x) xs[t] = v[k0 + t];
  __syncthreads();
  for (int r = threadIdx.x; r < nb; r += blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < nb; ++c) acc = fma(Dinv[r + kTriBlock * c], xs[c], acc);
    sol[k0 + r] = acc;
  }
}

// One block step of a blocked triangular solve.  sol[k0 : k0 + nb] is final;
// rows [r0, r1) of v get v_r -= sum_c A[r, k0 + c] sol[k0 + c] (128 rows per
// CTA, four column quarters per row, four accumulators each).  The CTA whose
// rows are the next block [nk0, nk0 + nnb) (it starts at nk0 by
// construction) then forms sol there = Dnext v, the same four-way split.
constexpr int kTriQ = 4;                       // column quarters per row
constexpr int kTriThreads = kTriBlock * kTriQ;  // 512
__global__ void __launch_bounds__(kTriThreads) k_tri_step(const double* __restrict__ A, double* v, double* sol,
                                                          int n, int k0, int nb, int r0, int r1,
                                                          const double* __restrict__ Dnext, int nk0, int nnb) {
  __shared__ double ss[kTriBlock], part[kTriQ][kTriBlock], vn[kTriBlock];
  for (int t = threadIdx.x; t < nb; t += blockDim.x) ss[t] = sol[k0 + t];
  __syncthreads();
  const int lr = threadIdx.x % kTriBlock, qt = threadIdx.x / kTriBlock;
  const int first = r0 + blockIdx.x * kTriBlock, r = first + lr;
  constexpr int kCols = kTriBlock / kTriQ;
  double acc = 0.0;
  if (r < r1) {
    const int c0 = qt * kCols, c1 = min(nb, c0 + kCols);
    const double* col = A + r + (long long)n * k0;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (c1 - c0 == kCols) {
      // full quarter: all loads issued before the products
      double e[kCols];
#pragma unroll
      for (int t = 0; t < kCols; ++t) e[t] = col[(long long)n * (c0 + t)];
#pragma unroll
      for (int t = 0; t < kCols; t += 4) {
        a0 = fma(e[t], ss[c0 + t], a0);
        a1 = fma(e[t + 1], ss[c0 + t + 1], a1);
        a2 = fma(e[t + 2], ss[c0 + t + 2], a2);
        a3 = fma(e[t + 3], ss[c0 + t + 3], a3);
      }
    } else {
      for (int c = c0; c < c1; ++c) a0 = fma(col[(long long)n * c], ss[c], a0);
    }
    acc = (a0 + a1) + (a2 + a3);
  }
  part[qt][lr] = acc;
  __syncthreads();
  if (qt == 0 && r < r1) {
    const double nv = v[r] - ((part[0][lr] + part[1][lr]) + (part[2][lr] + part[3][lr]));
    v[r] = nv;
    vn[lr] = nv;
  }
  if (Dnext && first == nk0) {
    __syncthreads();
    double s2 = 0.0;
    if (lr < nnb) {
      const int c0 = qt * kCols, c1 = min(nnb, c0 + kCols);
      for (int c2 = c0; c2 < c1; ++c2) s2 = fma(Dnext[lr + kTriBlock * c2], vn[c2], s2);
    }
    part[qt][lr] = s2;
    __syncthreads();
    if (qt == 0 && lr < nnb) sol[nk0 + lr] = (part[0][lr] + part[1][lr]) + (part[2][lr] + part[3][lr]);
  }
}

// ---------------------------------------------------------------------------
// Persistent triangular solves (default when cooperative launch is available)
//
// The block steps above pay a launch and a grid-wide drain per 128 rows.  On
// GB300 the solve is bound by the FP64 pipe (n^2/2 FMAs per triangle, about
// 1.8 ms at n = 46,860), not by the 8 n^2 bytes of the factor, so what
// matters is keeping every SM's FP64 units busy while the chain of diagonal
// blocks advances.  One cooperative launch per triangle does it:
//  * blocks of kPb = 64 rows; logical step t is block t (L, forward) or
//    block nb-1-t (U, backward); CTA g owns the steps t = g mod G and keeps
//    their right-hand sides acc_t (K vectors) in shared memory;
//  * when sol_t is published (global store, fence, release flag), every CTA
//    applies panel t to its owned blocks further down (64 x 64 FP64 products
//    read coalesced from the column-major factor);
//  * the diagonal chain is shortened with set-up products
//    W_t = inv(D_t) T(t, t-1): sol_t = z_t - W_t sol_{t-1}, where
//    z_t = inv(D_t) acc_t is formed as soon as acc_t has received every panel
//    but the last, off the critical path.  The owner of t+1 forms and
//    publishes sol_{t+1} right after it receives sol_t, before its other
//    work, so one 64 x 64 product and one flag hop separate consecutive
//    blocks;
//  * flags are zeroed by a memset before each launch; every wait is bounded
//    (about a second of clock) and raises *err instead of hanging.
// The products sum in a fixed order, so results are reproducible run to run.
constexpr int kPb = 64;
constexpr int kPThreads = 256;
constexpr int kPMaxOwned = 48;   // steps per CTA: nb <= kPMaxOwned * grid
constexpr long long kPWaitCycles = 2000000000LL;

// Inverse of diagonal block b (kPb rows) of L (unit) or U, as
// k_tri_block_inverse; out = column-major kPb x kPb per block.
__global__ void __launch_bounds__(256) k_pdinv(const double* __restrict__ A, int n, int upper,
                                               double* __restrict__ out) {
  __shared__ double X[kPb * kPb];  // row r at X[r * kPb]
  const int k0 = blockIdx.x * kPb, nb = min(kPb, n - k0);
  for (int t = threadIdx.x; t < kPb * kPb; t += blockDim.x)
    X[t] = (t / kPb == t % kPb && t / kPb < nb) ? 1.0 : 0.0;
  __syncthreads();
  if (!upper) {
    for (int c = 0; c < nb; ++c) {
      for (int t = threadIdx.x; t < (nb - c - 1) * (c + 1); t += blockDim.x) {
        const int r = c + 1 + t / (c + 1), j = t % (c + 1);
        X[r * kPb + j] -= A[(k0 + r) + (long long)n * (k0 + c)] * X[c * kPb + j];
      }
      __syncthreads();
    }
  } else {
    for (int c = nb - 1; c >= 0; --c) {
      const double d = A[(k0 + c) + (long long)n * (k0 + c)];
      for (int j = c + threadIdx.x; j < nb; j += blockDim.x) X[c * kPb + j] = X[c * kPb + j] / d;
      __syncthreads();
      for (int t = threadIdx.x; t < c * (nb - c); t += blockDim.x) {
        const int r = t / (nb - c), j = c + t % (nb - c);
        X[r * kPb + j] -= A[(k0 + r) + (long long)n * (k0 + c)] * X[c * kPb + j];
      }
      __syncthreads();
    }
  }
  double* o = out + (size_t)blockIdx.x * kPb * kPb;
  for (int t = threadIdx.x; t < kPb * kPb; t += blockDim.x) o[t] = X[(t % kPb) * kPb + t / kPb];
}

// W_b = inv(D_b) T(b, b-1) (L) or inv(D_b) T(b, b+1) (U), column-major
// kPb x kPb, zero outside the blocks' extents; one CTA per block (the first
// block of L and the last of U have none and stay zero).
__global__ void __launch_bounds__(256) k_pw(const double* __restrict__ A, int n, int upper,
                                            const double* __restrict__ dinv, double* __restrict__ W) {
  __shared__ double D[kPb * kPb], T[kPb * kPb];
  const int b = blockIdx.x, nbk = (n + kPb - 1) / kPb;
  const int ob = upper ? b + 1 : b - 1;
  double* o = W + (size_t)b * kPb * kPb;
  if (ob < 0 || ob >= nbk) {
    for (int t = threadIdx.x; t < kPb * kPb; t += blockDim.x) o[t] = 0.0;
    return;
  }
  const int r0 = b * kPb, rn = min(kPb, n - r0), c0 = ob * kPb, cn = min(kPb, n - c0);
  for (int t = threadIdx.x; t < kPb * kPb; t += blockDim.x) {
    const int r = t % kPb, c = t / kPb;
    D[t] = dinv[(size_t)b * kPb * kPb + t];
    T[t] = (r < rn && c < cn) ? A[(r0 + r) + (long long)n * (c0 + c)] : 0.0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kPb * kPb; t += blockDim.x) {
    const int r = t % kPb, c = t / kPb;
    double s = 0.0;
    for (int k = 0; k < kPb; ++k) s = fma(D[r + kPb * k], T[k + kPb * c], s);
    o[t] = s;
  }
}

// out[k][r] (=|-=) sum_c M(r, c) x[k][c] for a 64 x 64 column-major tile M
// with leading dimension ld (rows >= rn and columns >= cn are not read), K
// vectors x in shared memory.  Thread t: row t % 64, columns 16 (t / 64) ..
// +15; the four partial sums are added in a fixed order.
template <int K>
__device__ __forceinline__ void tile_gemv(const double* __restrict__ M, long long ld, int rn, int cn,
                                          const double (*x)[kPb], double (*part)[K][kPb], double (*out)[kPb],
                                          bool subtract) {
  const int r = threadIdx.x & (kPb - 1), g = threadIdx.x >> 6;
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  if (r < rn) {
    double e[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int c = 16 * g + q;
      e[q] = c < cn ? M[r + ld * c] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q)
#pragma unroll
      for (int k = 0; k < K; ++k) acc[k] = fma(e[q], x[k][16 * g + q], acc[k]);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) part[g][k][r] = acc[k];
  __syncthreads();
  if (threadIdx.x < kPb * K) {
    const int rr = threadIdx.x % kPb, k = threadIdx.x / kPb;
    const double s = (part[0][k][rr] + part[1][k][rr]) + (part[2][k][rr] + part[3][k][rr]);
    out[k][rr] = subtract ? out[k][rr] - s : s;
  }
  __syncthreads();
}

__device__ __forceinline__ int flag_acquire(const int* f) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
  return v;
}
__device__ __forceinline__ void flag_release(int* f, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(f), "r"(v) : "memory");
}

// One triangle: sol = inv(T) v for the unit lower L (upper = 0) or U
// (upper = 1) of the column-major factor A; K right-hand sides, vector k at
// v + k n and sol + k n.  flags[nb] zero on entry.
template <int K>
__global__ void __launch_bounds__(kPThreads) k_tri_persist(const double* __restrict__ A, int n, int upper,
                                                           const double* __restrict__ dinv,
                                                           const double* __restrict__ W,
                                                           const double* __restrict__ v, double* sol, int* flags,
                                                           int* err) {
  extern __shared__ double sm[];
  const int nb = (n + kPb - 1) / kPb, G = gridDim.x, g = blockIdx.x;
  const int owned = (nb - g + G - 1) / G;           // steps g, g + G, ...
  double (*acc)[K][kPb] = reinterpret_cast<double (*)[K][kPb]>(sm);                // [owned]
  double (*z)[K][kPb] = reinterpret_cast<double (*)[K][kPb]>(sm + (size_t)owned * K * kPb);
  double (*cur)[kPb] = reinterpret_cast<double (*)[kPb]>(sm + (size_t)2 * owned * K * kPb);  // [K]
  double (*nxt)[kPb] = cur + K;
  double (*part)[K][kPb] = reinterpret_cast<double (*)[K][kPb]>(nxt + K);              // [4]
  __shared__ int s_fail;
  auto blk = [&](int t) { return upper ? nb - 1 - t : t; };
  auto rows = [&](int t) { return min(kPb, n - blk(t) * kPb); };
  auto mine = [&](int t) { return t < nb && t % G == g; };
  auto slot = [&](int t) { return t / G; };
  // publish cur (= sol_t) and raise flag t
  auto publish = [&](int t, double (*x)[kPb]) {
    const int r0 = blk(t) * kPb, rn = rows(t);
    for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) {
      const int k = q / kPb, r = q % kPb;
      if (r < rn) __stcg(sol + (size_t)k * n + r0 + r, x[k][r]);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) flag_release(flags + t, 1);
  };
  // z_t = inv(D_t) acc_t
  auto form_z = [&](int t) {
    tile_gemv<K>(dinv + (size_t)blk(t) * kPb * kPb, kPb, rows(t), rows(t), acc[slot(t)], part, z[slot(t)], false);
  };
  if (threadIdx.x == 0) s_fail = 0;
  for (int s = 0; s < owned; ++s) {
    const int t = g + s * G, r0 = blk(t) * kPb, rn = rows(t);
    for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) {
      const int k = q / kPb, r = q % kPb;
      acc[s][k][r] = r < rn ? v[(size_t)k * n + r0 + r] : 0.0;
    }
  }
  __syncthreads();
  if (mine(0)) {
    form_z(0);
    for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) cur[q / kPb][q % kPb] = z[0][q / kPb][q % kPb];
    __syncthreads();
    publish(0, cur);
  }
  if (mine(1)) form_z(1);
  for (int t = 0; t + 1 < nb; ++t) {
    // sol_t into cur (computed here when this CTA owns t)
    if (!mine(t)) {
      if (threadIdx.x == 0) {
        const long long c0 = clock64();
        while (flag_acquire(flags + t) == 0) {
          __nanosleep(64);
          if (clock64() - c0 > kPWaitCycles) {
            atomicExch(err, 1);
            s_fail = 1;
            break;
          }
        }
      }
      __syncthreads();
      if (s_fail) return;
      const int r0 = blk(t) * kPb, rn = rows(t);
      for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) {
        const int k = q / kPb, r = q % kPb;
        cur[k][r] = r < rn ? __ldcg(sol + (size_t)k * n + r0 + r) : 0.0;
      }
      __syncthreads();
    }
    // the critical block first: sol_{t+1} = z_{t+1} - W_{t+1} sol_t
    if (mine(t + 1)) {
      const int s1 = slot(t + 1);
      for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) nxt[q / kPb][q % kPb] = z[s1][q / kPb][q % kPb];
      __syncthreads();
      tile_gemv<K>(W + (size_t)blk(t + 1) * kPb * kPb, kPb, rows(t + 1), rows(t), cur, part, nxt, true);
      publish(t + 1, nxt);
    }
    // panel t on the owned blocks two or more steps ahead
    const int cb = blk(t) * kPb, cn = rows(t);
    for (int s = 0; s < owned; ++s) {
      const int u = g + s * G;
      if (u < t + 2) continue;
      tile_gemv<K>(A + (size_t)blk(u) * kPb + (size_t)n * cb, n, rows(u), cn, cur, part, acc[s], true);
    }
    if (mine(t + 2)) form_z(t + 2);
    // the block published above is the next step's sol
    if (mine(t + 1)) {
      for (int q = threadIdx.x; q < K * kPb; q += blockDim.x) cur[q / kPb][q % kPb] = nxt[q / kPb][q % kPb];
      __syncthreads();
    }
  }
}

static size_t tri_persist_smem(int owned, int K) {
  return sizeof(double) * ((size_t)2 * owned * K * kPb + 2 * K * kPb + 4 * K * kPb);
}

// Influence-matrix assembly in the eigenbasis of the subdomain solver.  A
// Dirac datum at point (s1, s2) of face (l, m) folds into the right-hand
// side phi_{l,m}(i_l) delta(s1) delta(s2) (phi = -inv_lhs(:, ends) ddr bc),
// whose transform is separable: psi(p_l) Vinv_b1[q, s1] Vinv_b2[r, s2] with
// psi = Vinv_l phi.  The column entries are the normal derivatives of the
// solution on the interface faces, i.e. linear functionals omega(p) =
// sum_i W_eff[i] V[i, p] of the transformed solution along the target axis
// (W_eff: the face row of the full-line derivative, with the Neumann end
// extrapolated from the interior).  So a face-to-face block is
//   same axis:  (V_b1 (x) V_b2) diag(G) (Vinv_b1 (x) Vinv_b2),
//               G(q, r) = sum_p omega(p) psi(p) / den(p, q, r),
//   cross axes: sum_{p_k} V_k[i_k, p_k] H[i_l, i_l2, p_k] Vinv_k[p_k, i'_k],
// n^5 work per block instead of one n^4 solve per Dirac column.
struct Lam3 {
  const double* lam[3];  // eigenvalues of the x, y, z axes
};

// 1 / (lam_x + lam_y + lam_z + sigma), 0 for the null mode (the eigenvalue
// division of solve_3d, class_solver_3d.f90:202-225).
__device__ __forceinline__ double inv_den(const Lam3& L, const int idx[3], double sigma) {
  const double a = L.lam[0][idx[0]], b = L.lam[1][idx[1]], c = L.lam[2][idx[2]];
  if (fmax(fmax(fabs(sigma), fabs(a)), fmax(fabs(b), fabs(c))) < (double)1e-11f) return 0.0;
  return 1.0 / (((a + b) + c) + sigma);
}

// G[q + n1 r] = sum_p w[p] / den, with p on axis l, q on b1, r on b2.
__global__ void k_inf_g(Lam3 L, double sigma, int l, int b1, int b2, int nl, int n1, int n2,
                        const double* __restrict__ w, double* __restrict__ G) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  int idx[3];
  idx[b1] = t % n1;
  idx[b2] = t / n1;
  double acc = 0.0;
  for (int p = 0; p < nl; ++p) {
    idx[l] = p;
    acc = fma(w[p], inv_den(L, idx, sigma), acc);
  }
  G[t] = acc;
}

// F[p_l + nl (i2 + n2 p_k)] = sum_{p2} Y[p2 n2 + i2] / den(p_l, p2, p_k),
// axes l, l2, k; Y = diag(omega) Vinv_l2.
__global__ void k_inf_f(Lam3 L, double sigma, int l, int l2, int k, int nl, int n2, int nk,
                        const double* __restrict__ Y, double* __restrict__ F) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nl * n2 * nk) return;
  const int pl = (int)(t % nl), i2 = (int)((t / nl) % n2), pk = (int)(t / ((long long)nl * n2));
  int idx[3];
  idx[l] = pl;
  idx[k] = pk;
  double acc = 0.0;
  for (int p2 = 0; p2 < n2; ++p2) {
    idx[l2] = p2;
    acc = fma(Y[p2 * n2 + i2], inv_den(L, idx, sigma), acc);
  }
  F[t] = acc;
}

// H[i_l + nl (i2 + n2 p_k)] = sum_{p_l} Z[i_l nl + p_l] F[p_l + nl (i2 + n2 p_k)], Z = V_l diag(psi).
__global__ void k_inf_h(const double* __restrict__ Z, const double* __restrict__ F, int nl, int n2, int nk,
                        double* __restrict__ H) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nl * n2 * nk) return;
  const int il = (int)(t % nl);
  const long long rest = t / nl;
  const double* f = F + rest * nl;
  double acc = 0.0;
  for (int p = 0; p < nl; ++p) acc = fma(Z[il * nl + p], f[p], acc);
  H[t] = acc;
}

// Placement of a batched product in a linear array:
// index = r0 + i ri + b1 rb1 + b2 rb2 + ld (c0 + j cj + b1 cb1 + b2 cb2).
struct Place {
  long long r0, ri, rb1, rb2, c0, cj, cb1, cb2, ld;
  double scale;
  int add;  // 1: out += scale v; 0: out = scale v
};

// out_b[i, j] = sum_q A[i K + q] u_b[q] B[q nj + j] for batch b = (b1, b2),
// u_b[q] = U[b1 us1 + b2 us2 + q uq].  Grid (ceil(ni nj / 256), nb1 nb2).
__global__ void __launch_bounds__(256) k_inf_adb(const double* __restrict__ A, const double* __restrict__ B, int ni,
                                                 int nj, int K, const double* __restrict__ U, long long us1,
                                                 long long us2, long long uq, int nb1, double* out, Place P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ni * nj) return;
  const int j = t % nj, i = t / nj;
  const int b1 = (int)(blockIdx.y % nb1), b2 = (int)(blockIdx.y / nb1);
  const double* u = U + b1 * us1 + b2 * us2;
  const double* a = A + (long long)i * K;
  double acc = 0.0;
  for (int q = 0; q < K; ++q) acc = fma(a[q] * u[q * uq], B[(long long)q * nj + j], acc);
  const long long o = P.r0 + i * P.ri + b1 * P.rb1 + b2 * P.rb2 + P.ld * (P.c0 + j * P.cj + b1 * P.cb1 + b2 * P.cb2);
  out[o] = P.add ? out[o] + P.scale * acc : P.scale * acc;
}

// M[(row0 + q) + ld (col0 + q)] += v for q < npts (the Dirac's own end value
// on the derivative line through it).
__global__ void k_inf_direct(double* M, long long ld, long long row0, long long col0, long long npts, double v) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < npts) M[(row0 + q) + ld * (col0 + q)] += v;
}

// Largest interface system whose explicit inverse is formed at set-up.
constexpr long long kMaxInverseRows = 12000;

// Y[:, r] = A X[:, r] for K right-hand sides (columns of length n) with the
// row-major A (the interface inverse): one warp per row, kGemvRows rows per
// CTA.  Each row of A is read once for all K columns; the columns of X are
// staged through shared memory in chunks of kGemvChunk entries, so X comes
// from L2 once per CTA rather than once per row (without it, a 64 x 65 x 64
// channel step's three-column product took 4.7 times the HBM time of its
// 0.49 GB inverse).  Per column each lane accumulates columns lane + 64 i
// into one sum and lane + 32 + 64 i into another before the warp reduces:
// the same order for every K, so a column's result does not depend on how
// many columns share the call.
constexpr int kMdMaxRhs = 4;
constexpr int kGemvRows = 16;
constexpr int kGemvChunk = 512;  // a multiple of 64
template <int K>
__global__ void __launch_bounds__(32 * kGemvRows) k_gemm_rows(const double* __restrict__ A,
                                                              const double* __restrict__ X,
                                                              double* __restrict__ Y, int n) {
  __shared__ double xs[K][kGemvChunk];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long ri = (long long)blockIdx.x * kGemvRows + w;
  const bool live = ri < n;
  const double* row = A + (live ? ri : 0) * (long long)n;
  double a0[K], a1[K];
#pragma unroll
  for (int r = 0; r < K; ++r) a0[r] = a1[r] = 0.0;
  for (int c0 = 0; c0 < n; c0 += kGemvChunk) {
    const int len = min(kGemvChunk, n - c0);
    __syncthreads();  // the previous chunk is consumed
    for (int e = threadIdx.x; e < K * kGemvChunk; e += blockDim.x) {
      const int r = e / kGemvChunk, c = e % kGemvChunk;
      xs[r][c] = c < len ? X[(long long)r * n + c0 + c] : 0.0;
    }
    __syncthreads();
    if (!live) continue;
    const double* rc = row + c0;
    int c = lane;
    for (; c + 32 < len; c += 64) {
      const double e0 = rc[c], e1 = rc[c + 32];
#pragma unroll
      for (int r = 0; r < K; ++r) {
        a0[r] = fma(e0, xs[r][c], a0[r]);
        a1[r] = fma(e1, xs[r][c + 32], a1[r]);
      }
    }
    if (c < len) {
      const double e0 = rc[c];
#pragma unroll
      for (int r = 0; r < K; ++r) a0[r] = fma(e0, xs[r][c], a0[r]);
    }
  }
  if (!live) return;
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double v = a0[r] + a1[r];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) Y[(long long)r * n + ri] = v;
  }
}

// In-place transpose of the n x n matrix A (column-major to row-major, set-up
// only): CTA (bx, by), bx < by, swaps the 32 x 32 tiles (bx, by) and (by, bx)
// through shared memory, bx == by transposes its tile, bx > by returns.  Both
// tiles are read before either is written.  With L given, entries below the
// diagonal are taken from L instead of A (the two inverted factors, each
// inverted in its own copy, merge into one array on the way).
__global__ void __launch_bounds__(256) k_transpose_square(double* A, const double* __restrict__ L, int n) {
  const int bx = blockIdx.x, by = blockIdx.y;
  if (bx > by) return;
  __shared__ double t1[32][33], t2[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const long long N = n;
  for (int k = ty; k < 32; k += 8) {
    const long long i1 = bx * 32 + tx, j1 = by * 32 + k, i2 = by * 32 + tx, j2 = bx * 32 + k;
    if (i1 < N && j1 < N) t1[k][tx] = (L && i1 > j1) ? L[i1 + N * j1] : A[i1 + N * j1];
    if (i2 < N && j2 < N) t2[k][tx] = (L && i2 > j2) ? L[i2 + N * j2] : A[i2 + N * j2];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const long long i1 = bx * 32 + tx, j1 = by * 32 + k, i2 = by * 32 + tx, j2 = bx * 32 + k;
    if (i1 < N && j1 < N) A[i1 + N * j1] = t2[tx][k];
    if (bx != by && i2 < N && j2 < N) A[i2 + N * j2] = t1[tx][k];
  }
}

// Unit diagonal written into the n x n column-major A (the copy of the LU
// factor whose lower part is inverted as L).
__global__ void k_unit_diagonal(double* A, int n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + (long long)n * i] = 1.0;
}

// Products with the inverted LU factors of the interface system, both held
// row-major in one n x n array T: its strict lower part is L^-1 below the unit
// diagonal, its upper part with the diagonal U^-1.  UPPER = false: Y[:, r] =
// X[:, r] + (strict lower of T) X[:, r]; UPPER = true: Y[:, r] = (upper of T)
// X[:, r], for K right-hand sides (columns of length n).  Unlike the
// triangular solves on the factors, every row is independent: each warp owns
// rows r0 + w and r0 + 16 + w of its CTA and reads T[row, lo : hi) once for
// all K columns (lo = 0, hi = row below the diagonal; lo = row, hi = n
// above), four 256-byte loads in flight per row; X is staged through shared
// memory in chunks over the columns the CTA's rows need.  The lane and
// accumulator of a column depend only on the row pair and the chunk, so a
// column's result does not depend on K.
constexpr int kTmvRows = 32;     // rows per CTA, two per warp
constexpr int kTmvChunk = 1024;  // columns of X staged at a time
template <int K, bool UPPER>
__global__ void __launch_bounds__(512) k_trimv_rows(const double* __restrict__ T, const double* __restrict__ X,
                                                    double* __restrict__ Y, int n) {
  __shared__ double xs[K][kTmvChunk];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // heaviest row blocks first (the longest rows of L^-1 are the last ones)
  const int r0 = (UPPER ? blockIdx.x : gridDim.x - 1 - blockIdx.x) * kTmvRows;
  const int ra = r0 + w, rb = r0 + 16 + w;
  const bool la = ra < n, lb = rb < n;
  const int rlast = min(r0 + kTmvRows, n) - 1;
  const int clo = UPPER ? r0 : 0, chi = UPPER ? n : rlast;  // columns any row of the CTA needs
  const int loa = UPPER ? ra : 0, hia = la ? (UPPER ? n : ra) : 0;
  const int lob = UPPER ? rb : 0, hib = lb ? (UPPER ? n : rb) : 0;
  const double* rowa = T + (long long)(la ? ra : 0) * n;
  const double* rowb = T + (long long)(lb ? rb : 0) * n;
  double sa[2][K], sb[2][K];
#pragma unroll
  for (int r = 0; r < K; ++r) sa[0][r] = sa[1][r] = sb[0][r] = sb[1][r] = 0.0;
  for (int c0 = clo; c0 < chi; c0 += kTmvChunk) {
    const int len = min(kTmvChunk, chi - c0);
    __syncthreads();  // the previous chunk is consumed
    for (int e = threadIdx.x; e < K * kTmvChunk; e += blockDim.x) {
      const int r = e / kTmvChunk, c = e % kTmvChunk;
      xs[r][c] = c < len ? X[(long long)r * n + c0 + c] : 0.0;
    }
    __syncthreads();
    // local column ranges [ba, ea), [bb, eb) within the chunk, and their union
    const int ba = max(loa, c0) - c0, ea = min(hia, c0 + len) - c0;
    const int bb = max(lob, c0) - c0, eb = min(hib, c0 + len) - c0;
    const int b = min(ba < ea ? ba : len, bb < eb ? bb : len), e = max(ea, eb);
    for (int c = b + lane; c < e; c += 128) {
      double va[4], vb[4];
      bool pa[4], pb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cq = c + 32 * q;
        pa[q] = cq >= ba && cq < ea;
        pb[q] = cq >= bb && cq < eb;
        va[q] = pa[q] ? rowa[c0 + cq] : 0.0;
        vb[q] = pb[q] ? rowb[c0 + cq] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cq = c + 32 * q;
#pragma unroll
        for (int r = 0; r < K; ++r) {
          if (pa[q]) sa[q & 1][r] = fma(va[q], xs[r][cq], sa[q & 1][r]);
          if (pb[q]) sb[q & 1][r] = fma(vb[q], xs[r][cq], sb[q & 1][r]);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double a = sa[0][r] + sa[1][r], bsum = sb[0][r] + sb[1][r];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      bsum += __shfl_down_sync(0xffffffffu, bsum, off);
    }
    if (lane == 0) {
      if (la) Y[(long long)r * n + ra] = UPPER ? a : X[(long long)r * n + ra] + a;
      if (lb) Y[(long long)r * n + rb] = UPPER ? bsum : X[(long long)r * n + rb] + bsum;
    }
  }
}

// The same products in double-float arithmetic on the FP32 pipe (GB300
// issues FP64 FMAs at about a sixtieth of its FP32 rate, and at one FMA per
// 8-byte element the FP64 form above is bound by that pipe, not by HBM).
// T holds each entry a as the pair (hi, lo) of FP32 values with hi = fl32(a),
// lo = fl32(a - hi) (8 bytes, as the FP64 entry it replaced); X arrives split
// the same way after scaling by a power of two per column (k_df_prep); T is
// scaled by one power of two at set-up (its largest entry in [1, 2), undone
// by tscale), so no product or sum leaves the FP32 range.  Per element: p = hi_a hi_x (its rounding
// error recovered exactly by an FMA, the cross terms hi_a lo_x + lo_a hi_x
// added to it) is summed into a (hi, lo) accumulator with Knuth's TwoSum
// (Knuth, TAOCP vol. 2, 4.2.2), every operation an explicit round-to-nearest
// intrinsic so that no multiply is contracted into the sums.  The warp's
// partial sums are reduced in FP64 and scaled back; the unit diagonal of L^-1
// adds the FP64 entry itself (Xp).  Accuracy about 2^-48 per element against
// FP64's 2^-53.
struct DfAcc {
  float h, l;
};
__device__ __forceinline__ void df_fma(DfAcc& s, float2 a, float2 x) {
  const float p = __fmul_rn(a.x, x.x);
  float e = __fmaf_rn(a.x, x.x, -p);
  e = __fmaf_rn(a.x, x.y, e);
  e = __fmaf_rn(a.y, x.x, e);
  const float t = __fadd_rn(s.h, p);
  const float bv = __fsub_rn(t, s.h);
  const float err = __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bv)), __fsub_rn(p, bv));
  s.h = t;
  s.l = __fadd_rn(s.l, __fadd_rn(err, e));
}

template <int K, bool UPPER>
__global__ void __launch_bounds__(512) k_trimv_rows_df(const float2* __restrict__ T, const float2* __restrict__ X,
                                                       const double* __restrict__ Xp,
                                                       const double* __restrict__ unscale, double tscale,
                                                       double* __restrict__ Y, int n) {
  __shared__ float2 xs[K][kTmvChunk];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // heaviest row blocks first (the longest rows of L^-1 are the last ones)
  const int blk = UPPER ? blockIdx.x : gridDim.x - 1 - blockIdx.x;
  const int r0 = blk * kTmvRows;
  const int ra = r0 + w, rb = r0 + 16 + w;
  const bool la = ra < n, lb = rb < n;
  const int rlast = min(r0 + kTmvRows, n) - 1;
  const int clo = UPPER ? r0 : 0, chi = UPPER ? n : rlast;
  const int loa = UPPER ? ra : 0, hia = la ? (UPPER ? n : ra) : 0;
  const int lob = UPPER ? rb : 0, hib = lb ? (UPPER ? n : rb) : 0;
  const float2* rowa = T + (long long)(la ? ra : 0) * n;
  const float2* rowb = T + (long long)(lb ? rb : 0) * n;
  DfAcc sa[2][K], sb[2][K];
#pragma unroll
  for (int r = 0; r < K; ++r)
#pragma unroll
    for (int h = 0; h < 2; ++h) sa[h][r] = sb[h][r] = DfAcc{0.f, 0.f};
  const float2 zero2 = make_float2(0.f, 0.f);
  for (int c0 = clo; c0 < chi; c0 += kTmvChunk) {
    const int len = min(kTmvChunk, chi - c0);
    // local column ranges [ba, ea), [bb, eb) within the chunk, and their union
    const int ba = max(loa, c0) - c0, ea = min(hia, c0 + len) - c0;
    const int bb = max(lob, c0) - c0, eb = min(hib, c0 + len) - c0;
    const int b = min(ba < ea ? ba : len, bb < eb ? bb : len), e = max(ea, eb);
    // one right-hand side (bound by HBM): the first loads of the chunk go out
    // before X is staged and each iteration issues the next one's before its
    // arithmetic.  More right-hand sides are bound by the FP32 issue rate and
    // keep the registers for two CTAs per SM instead
    constexpr bool kAhead = K == 1;
    float2 va[4], vb[4];
    int c = b + lane;
    if (kAhead) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cq = c + 32 * q;
        va[q] = (cq >= ba && cq < ea) ? rowa[c0 + cq] : zero2;
        vb[q] = (cq >= bb && cq < eb) ? rowb[c0 + cq] : zero2;
      }
    }
    __syncthreads();  // the previous chunk is consumed
    for (int i = threadIdx.x; i < K * kTmvChunk; i += blockDim.x) {
      const int r = i / kTmvChunk, cc = i % kTmvChunk;
      xs[r][cc] = cc < len ? X[(long long)r * n + c0 + cc] : zero2;
    }
    __syncthreads();
    // columns where both rows are inside their ranges: all but the edges
    const int fb = max(ba, bb), fe = min(ea, eb);
    for (; c < e; c += 128) {
      if (!kAhead && c >= fb && c + 96 < fe) {
        // every column of this step lies in both rows' ranges: no predicates
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          va[q] = rowa[c0 + c + 32 * q];
          vb[q] = rowb[c0 + c + 32 * q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
          for (int r = 0; r < K; ++r) {
            const float2 xv = xs[r][c + 32 * q];
            df_fma(sa[q & 1][r], va[q], xv);
            df_fma(sb[q & 1][r], vb[q], xv);
          }
        }
        continue;
      }
      float2 na[4], nb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cq = (kAhead ? c + 128 : c) + 32 * q;
        na[q] = (cq >= ba && cq < ea) ? rowa[c0 + cq] : zero2;
        nb[q] = (cq >= bb && cq < eb) ? rowb[c0 + cq] : zero2;
      }
      if (!kAhead) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          va[q] = na[q];
          vb[q] = nb[q];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cq = c + 32 * q;
        const bool pa = cq >= ba && cq < ea, pb = cq >= bb && cq < eb;
#pragma unroll
        for (int r = 0; r < K; ++r) {
          const float2 xv = (pa || pb) ? xs[r][cq] : zero2;
          if (pa) df_fma(sa[q & 1][r], va[q], xv);
          if (pb) df_fma(sb[q & 1][r], vb[q], xv);
        }
      }
      if (kAhead) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          va[q] = na[q];
          vb[q] = nb[q];
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double a = ((double)sa[0][r].h + (double)sa[1][r].h) + ((double)sa[0][r].l + (double)sa[1][r].l);
    double bsum = ((double)sb[0][r].h + (double)sb[1][r].h) + ((double)sb[0][r].l + (double)sb[1][r].l);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      bsum += __shfl_down_sync(0xffffffffu, bsum, off);
    }
    if (lane == 0) {
      const double u = unscale[r] * tscale;
      if (la) Y[(long long)r * n + ra] = UPPER ? a * u : Xp[(long long)r * n + ra] + a * u;
      if (lb) Y[(long long)r * n + rb] = UPPER ? bsum * u : Xp[(long long)r * n + rb] + bsum * u;
    }
  }
}

// Right-hand side r (CTA r) for k_trimv_rows_df: x = in[perm[i]] (perm may be
// null), written to xp in FP64 when xp is given, and split after scaling by
// 2^-e (2^e <= max |x| < 2^(e+1); no scaling for a zero or non-finite
// maximum) into xdf = (hi, lo); unscale[r] = 2^e.
__global__ void __launch_bounds__(1024) k_df_prep(const double* __restrict__ in, const int* __restrict__ perm,
                                                  double* __restrict__ xp, float2* __restrict__ xdf,
                                                  double* __restrict__ unscale, int n) {
  __shared__ double part[32];
  const double* x = in + (size_t)blockIdx.x * n;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[perm ? perm[i] : i]));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  m = part[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, part[q]);
  const bool ok = m > 0.0 && m <= 1.7e308;
  const int ex = ok ? ilogb(m) : 0;
  const double s = scalbn(1.0, -ex);
  if (threadIdx.x == 0) unscale[blockIdx.x] = scalbn(1.0, ex);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = x[perm ? perm[i] : i];
    if (xp) xp[(size_t)blockIdx.x * n + i] = v;
    const double ws = v * s;
    const float h = __double2float_rn(ws);
    xdf[(size_t)blockIdx.x * n + i] = make_float2(h, __double2float_rn(ws - (double)h));
  }
}

// Set-up of the double-float factors: the largest |entry| of T (as the bits
// of a non-negative double, whose order is the numbers' order; NaN compares
// above every finite value), then the in-place conversion of each FP64 entry
// a, scaled by the power of two s that brings that maximum into [1, 2), into
// the pair (fl32(a s), fl32(a s - fl32(a s))).  Entries below 2^-126 of the
// largest fall into FP32's subnormal range, a contribution below 2^-126 of
// the row's largest product.
__global__ void k_df_range(const double* __restrict__ T, long long count, unsigned long long* __restrict__ maxbits) {
  double m = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = fabs(T[i]);
    m = (a != a || a > m) ? a : m;
  }
  atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}
__global__ void k_df_convert(double* T, long long count, double s) {
  float2* out = reinterpret_cast<float2*>(T);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = T[i] * s;
    const float h = __double2float_rn(a);
    out[i] = make_float2(h, __double2float_rn(a - (double)h));
  }
}

// Identity matrix, n x n column-major.
__global__ void k_identity(double* A, int n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  A[t] = (t % n == t / n) ? 1.0 : 0.0;
}

// Mean removal (single CTA reduction; interface vectors are small).
__global__ void k_remove_mean(double* x, int n) {
  __shared__ double part[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  const double mean = part[0] / n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] -= mean;
}

__global__ void k_set_scalar(double* x, long long i, double v) {
  if (blockIdx.x == 0 && threadIdx.x == 0) x[i] = v;
}

__global__ void k_pin_row0(double* M, int n) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) M[(long long)n * c] = (c == 0) ? 5.0 : 0.0;
}

__global__ void k_extract_int(const double* __restrict__ g, double* __restrict__ out, int n1, int n2,
                              int n3) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)n1 * n2 * n3;
  if (idx >= tot) return;
  const int i = (int)(idx % n1);
  const long long jk = idx / n1;
  const int j = (int)(jk % n2), k = (int)(jk / n2);
  out[idx] = g[(i + 1) + (long long)(n1 + 2) * ((j + 1) + (long long)(n2 + 2) * (k + 1))];
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int der_launch(const mf_der_t* dc, int axis, int order, int mode, const double* f, double* df,
               int nx, int ny, int nz, cudaStream_t st);

}  // namespace mf

using namespace mf;

struct mf_md {
  MdTopology topo;
  struct Sub {
    int n[3];          // nodes
    int bct[6];        // effective boundary types
    mf_solver3d_t* sc = nullptr;
    mf_der_t* dc[3] = {nullptr, nullptr, nullptr};
    DevBuf bc[3];      // face arrays (2 sides each)
    DevBuf rint;         // interior right-hand side of this subdomain
    DevBuf facew[3];     // rows 0 and n-1 of the plain first-derivative operator along each axis
    cudaStream_t stream = nullptr;  // this subdomain's branch of a solve
    cudaEvent_t done = nullptr;
  };
  cudaEvent_t fork = nullptr;
  std::vector<Sub> sub;  // index i + nd1*(j + nd2*k)
  DevBuf M, ipiv, vec, info, work, zero_int, rint, ufield;
  DevBuf perm, dinv, lu_v, lu_y;  // LU solve: row permutation, diagonal-block inverses, work vectors
  DevBuf pdinv, pw, pflags, perr; // persistent LU solve: 64-row block inverses, W blocks, flags, error flag
  bool persist_ok = false;
  int tri_form = 0;               // 0 persistent when possible, 1 one launch per block step
  DevBuf Minv, vec2;  // row-major inverse of the influence matrix, solve output
  DevBuf ub, dub[3], bcb;  // batched influence columns: fields, derivatives, Dirac faces
  bool inv_ok = false;
  bool trinv_ok = false;  // Minv holds the inverted LU factors, row-major (k_trimv_rows)
  bool trinv_df = false;  // ... as double-float pairs (k_trimv_rows_df), scaled by 1 / trinv_tscale
  double trinv_tscale = 1.0;
  DevBuf xdf, unscale, dfmax;  // double-float right-hand sides, their scales, the factors' max |entry|
  int iface_mode = MF_MD_IFACE_AUTO;
  cusolverDnHandle_t cs = nullptr;
  cublasHandle_t cb = nullptr;  // set-up only: the blocked triangular inverses
  int null_mode = 0;
  double sigma = 0.0;
  bool factored = false;
  uint64_t geom_key = 0;  // hash of the decomposition, grids, boundary types and order
  int assembly = MF_MD_ASSEMBLY_EIGEN;
  int precision = MF_PREC_FP64, refine = -1;  // subdomain solves of mf_md_solve
  DevBuf inf_w[5];  // eigenbasis assembly: small vectors/matrices, G, stage, F, H
};

namespace mf {

static int md_sub_index(const mf_md* md, int i, int j, int k) {
  return i + md->topo.nd[0] * (j + md->topo.nd[1] * k);
}

// 64-bit FNV-1a over raw bytes (the cache key of an influence matrix).
static uint64_t fnv1a(uint64_t h, const void* data, size_t bytes) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ULL;
  }
  return h;
}

static uint64_t factor_key(const mf_md* md, double sigma, int null_mode) {
  uint64_t h = fnv1a(md->geom_key, &sigma, sizeof(sigma));
  return fnv1a(h, &null_mode, sizeof(null_mode));
}

// Solves subdomain s with interior rhs `rint` and its internal bc arrays,
// writing the full field u (interior + faces).
static int md_sub_solve(mf_md* md, int s, const double* rint, double* u, cudaStream_t st) {
  mf_md::Sub& sd = md->sub[s];
  if (md->precision != MF_PREC_FP64)
    return mf_solve_3d_mixed(sd.sc, rint, md->sigma, u, sd.bc[0].as<double>(), sd.bc[1].as<double>(),
                             sd.bc[2].as<double>(), sd.n[0] - 2, sd.n[1] - 2, sd.n[2] - 2, md->precision,
                             md->refine, st);
  return mf_solve_3d(sd.sc, rint, md->sigma, u, sd.bc[0].as<double>(), sd.bc[1].as<double>(),
                     sd.bc[2].as<double>(), sd.n[0] - 2, sd.n[1] - 2, sd.n[2] - 2, st);
}

// Normal derivatives of u on every interface face of subdomain (i,j,k),
// added (times scale, signed like the reference) into out[rows]: one
// k_face_dot pass per axis with an interface face.
static int md_gather(mf_md* md, int i, int j, int k, const double* u, double* out, double scale,
                     cudaStream_t st) {
  const int s = md_sub_index(md, i, j, k);
  mf_md::Sub& sd = md->sub[s];
  for (int l = 0; l < 3; ++l) {
    FaceDot f{l, sd.n[0], sd.n[1], sd.n[2], {-1, -1}, scale};
    bool any = false;
    for (int m = 0; m < 2; ++m) {
      const int p = md->topo.get(i, j, k, l, m);
      if (p <= 0) continue;
      f.row0[m] = md->topo.offset[p - 1];
      any = true;
    }
    if (!any) continue;
    const int a = l == 0 ? 1 : 0, b = l == 2 ? 1 : 2;
    const long long lines = (long long)(sd.n[a] - 2) * (sd.n[b] - 2);
    k_face_dot<<<nblk(lines * kDotLanes, 256), 256, 0, st>>>(u, sd.facew[l].as<double>(), out, f);
    MF_CUDA(cudaGetLastError());
  }
  return MF_OK;
}

// Rows 0 and L-1 of the plain first-derivative operator of subdomain sd
// along axis a (L nodes), from the derivative of the L unit pencils; stored
// on the device as [row 0 | row L-1] for k_face_dot.
static int face_weights(mf_md::Sub& sd, int a) {
  const int L = sd.n[a];
  std::vector<double> I((size_t)L * L, 0.0), D((size_t)L * L), w((size_t)2 * L);
  for (int q = 0; q < L; ++q) I[(size_t)q * L + q] = 1.0;
  int rc = mf_der_lines(sd.dc[a], 1, 0, I.data(), D.data(), L, nullptr);
  if (rc) return rc;
  for (int q = 0; q < L; ++q) {
    w[q] = D[(size_t)q * L];
    w[(size_t)L + q] = D[(size_t)q * L + L - 1];
  }
  if ((rc = sd.facew[a].ensure(sizeof(double) * 2 * L))) return rc;
  MF_CUDA(cudaMemcpy(sd.facew[a].ptr, w.data(), sizeof(double) * 2 * L, cudaMemcpyHostToDevice));
  return MF_OK;
}

// Face sizes of subdomain s along axis l.
static long long face_points(const mf_md::Sub& sd, int l) {
  const int a = l == 0 ? 1 : 0, b = l == 2 ? 1 : 2;
  return (long long)(sd.n[a] - 2) * (sd.n[b] - 2);
}

template <int K>
static int launch_tri_persist(mf_md* md, int upper, const double* v, double* sol, cudaStream_t st, bool* done) {
  *done = false;
  const int n = (int)md->topo.ninf, nb = (n + kPb - 1) / kPb;
  static int sms = 0, occ[5] = {0, 0, 0, 0, 0};
  if (!sms) {
    int dev = 0;
    MF_CUDA(cudaGetDevice(&dev));
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  // grid: one CTA per SM, fewer when there are fewer blocks
  const int G = std::min(nb, sms);
  const int owned = (nb + G - 1) / G;
  if (owned > kPMaxOwned) return MF_OK;
  const size_t smem = tri_persist_smem(owned, K);
  if (smem > 200 * 1024) return MF_OK;
  MF_CUDA(cudaFuncSetAttribute(k_tri_persist<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (!occ[K]) {
    int o = 0;
    MF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_tri_persist<K>, kPThreads, smem));
    occ[K] = o;
  }
  if (occ[K] < 1) return MF_OK;  // not co-resident: the block steps take over
  const size_t half = (size_t)nb * kPb * kPb;
  const double* A = md->M.as<double>();
  const double* dinv = md->pdinv.as<double>() + (upper ? half : 0);
  const double* W = md->pw.as<double>() + (upper ? half : 0);
  int* flags = md->pflags.as<int>() + (upper ? nb : 0);
  int* err = md->perr.as<int>();
  MF_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * nb, st));
  int nn = n, up = upper;
  void* args[] = {(void*)&A, (void*)&nn, (void*)&up, (void*)&dinv, (void*)&W, (void*)&v, (void*)&sol,
                  (void*)&flags, (void*)&err};
  MF_CUDA(cudaLaunchCooperativeKernel((const void*)k_tri_persist<K>, dim3(G), dim3(kPThreads), args, smem, st));
  *done = true;
  return MF_OK;
}

// Persistent triangular solves of K right-hand sides stored one after the
// other at x (n each): x = U^-1 L^-1 P x.  *done is false when the
// persistent form does not apply (the caller then uses md_lu_solve).
template <int K>
static int md_lu_solve_persist(mf_md* md, double* x, cudaStream_t st, bool* done) {
  *done = false;
  if (!md->persist_ok) return MF_OK;
  const int n = (int)md->topo.ninf;
  double* v = md->lu_v.as<double>();
  double* y = md->lu_y.as<double>();
  for (int k = 0; k < K; ++k)
    k_permute<<<nblk(n, 256), 256, 0, st>>>(x + (size_t)k * n, md->perm.as<int>(), v + (size_t)k * n, n);
  MF_CUDA(cudaGetLastError());
  bool d1 = false, d2 = false;
  int rc = launch_tri_persist<K>(md, 0, v, y, st, &d1);
  if (rc || !d1) return rc;
  if ((rc = launch_tri_persist<K>(md, 1, y, x, st, &d2))) return rc;
  if (!d2) return set_error(MF_ERR_CUDA, "persistent triangular solve: second launch not possible");
  *done = true;
  return MF_OK;
}

// Blocked triangular solves with the LU factor in md->M: x = U^-1 L^-1 P x.
static int md_lu_solve(mf_md* md, double* x, cudaStream_t st) {
  const int n = (int)md->topo.ninf;
  const int nblocks = (n + kTriBlock - 1) / kTriBlock;
  const size_t bs = (size_t)kTriBlock * kTriBlock;
  const double* A = md->M.as<double>();
  const double* dl = md->dinv.as<double>();
  const double* du = dl + (size_t)nblocks * bs;
  double* v = md->lu_v.as<double>();
  double* y = md->lu_y.as<double>();
  auto nbk = [&](int b) { return std::min(kTriBlock, n - b * kTriBlock); };
  k_permute<<<nblk(n, 256), 256, 0, st>>>(x, md->perm.as<int>(), v, n);
  // L y = P x: y_0 first, then each step updates the rows below and forms the next block
  k_tri_first<<<1, kTriBlock, 0, st>>>(dl, v, y, 0, nbk(0));
  for (int b = 0; b + 1 < nblocks; ++b) {
    const int k0 = b * kTriBlock, rows = n - k0 - kTriBlock;
    k_tri_step<<<(rows + kTriBlock - 1) / kTriBlock, kTriThreads, 0, st>>>(
        A, v, y, n, k0, kTriBlock, k0 + kTriBlock, n, dl + (size_t)(b + 1) * bs, k0 + kTriBlock, nbk(b + 1));
  }
  // U x = y: the last block first, then upwards (y is updated in place)
  const int kl = (nblocks - 1) * kTriBlock;
  k_tri_first<<<1, kTriBlock, 0, st>>>(du + (size_t)(nblocks - 1) * bs, y, x, kl, nbk(nblocks - 1));
  for (int b = nblocks - 1; b > 0; --b) {
    const int k0 = b * kTriBlock;
    k_tri_step<<<k0 / kTriBlock, kTriThreads, 0, st>>>(A, y, x, n, k0, nbk(b), 0, k0,
                                                         du + (size_t)(b - 1) * bs, k0 - kTriBlock, kTriBlock);
  }
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

}  // namespace mf

extern "C" {

int mf_md_topology(const int nd[3], const int periods[3], const int* nint_x, const int* nint_y,
                   const int* nint_z, int* dm_int, int* kind, int* size, int* offset, int* it,
                   long long* ninf) {
  if (!nd || !periods || !nint_x || !nint_y || !nint_z)
    return set_error(MF_ERR_ARG, "mf_md_topology: null argument");
  const int* nint[3] = {nint_x, nint_y, nint_z};
  MdTopology t;
  int rc = topology_build(nd, periods, nint, t);
  if (rc) return rc;
  if (dm_int) {
    // Fortran order dm_int(nd1,nd2,nd3,3,2)
    for (int i = 0; i < nd[0]; ++i)
      for (int j = 0; j < nd[1]; ++j)
        for (int k = 0; k < nd[2]; ++k)
          for (int l = 0; l < 3; ++l)
            for (int m = 0; m < 2; ++m)
              dm_int[i + nd[0] * (j + nd[1] * (k + nd[2] * (l + 3 * m)))] = t.get(i, j, k, l, m);
  }
  for (int p = 0; p < t.it; ++p) {
    if (kind) kind[p] = t.kind[p];
    if (size) size[p] = t.size[p];
    if (offset) offset[p] = t.offset[p];
  }
  if (it) *it = t.it;
  if (ninf) *ninf = t.ninf;
  return MF_OK;
}

int mf_md_create(const int nd[3], const int periods[3], const double* const* gridx, const int* nx,
                 const double* const* gridy, const int* ny, const double* const* gridz, const int* nz,
                 const int bct[6], int so, mf_md_t** out) {
  if (!nd || !periods || !gridx || !gridy || !gridz || !nx || !ny || !nz || !bct || !out)
    return set_error(MF_ERR_ARG, "mf_md_create: null argument");
  *out = nullptr;
  std::vector<int> nint[3];
  const int* sizes[3] = {nx, ny, nz};
  for (int l = 0; l < 3; ++l)
    for (int s = 0; s < nd[l]; ++s) nint[l].push_back(sizes[l][s] - 2);
  const int* np[3] = {nint[0].data(), nint[1].data(), nint[2].data()};
  mf_md* md = new mf_md();
  int rc = topology_build(nd, periods, np, md->topo);
  if (rc) {
    delete md;
    return rc;
  }
  const int ns = nd[0] * nd[1] * nd[2];
  md->sub.resize(ns);
  size_t max_field = 0;
  for (int k = 0; k < nd[2]; ++k)
    for (int j = 0; j < nd[1]; ++j)
      for (int i = 0; i < nd[0]; ++i) {
        mf_md::Sub& sd = md->sub[md_sub_index(md, i, j, k)];
        sd.n[0] = nx[i];
        sd.n[1] = ny[j];
        sd.n[2] = nz[k];
        for (int f = 0; f < 6; ++f) sd.bct[f] = bct[f];
        for (int l = 0; l < 3; ++l)
          for (int m = 0; m < 2; ++m)
            if (md->topo.get(i, j, k, l, m) > 0) sd.bct[2 * l + m] = 1;  // md_bc_init
        const double* g[3] = {gridx[i], gridy[j], gridz[k]};
        if ((rc = mf_solver_coeffs_init_3d(g[0], g[1], g[2], sd.n[0], sd.n[1], sd.n[2], sd.bct, so,
                                           &sd.sc)))
          break;
        for (int l = 0; l < 3 && !rc; ++l) rc = mf_der_coeffs_init(g[l], sd.n[l], 1, so, &sd.dc[l]);
        if (rc) break;
        for (int l = 0; l < 3 && !rc; ++l) rc = face_weights(sd, l);
        if (rc) break;
        for (int l = 0; l < 3 && !rc; ++l) rc = sd.bc[l].ensure(sizeof(double) * 2 * face_points(sd, l));
        if (rc) break;
        max_field = std::max(max_field, (size_t)sd.n[0] * sd.n[1] * sd.n[2]);
      }
  if (!rc) {
    // cache key of the geometry: decomposition, periods, every slab's grid,
    // boundary types and scheme order
    uint64_t h = 1469598103934665603ULL;
    h = fnv1a(h, "MFMD1", 5);
    h = fnv1a(h, nd, 3 * sizeof(int));
    h = fnv1a(h, periods, 3 * sizeof(int));
    const double* const* grids[3] = {gridx, gridy, gridz};
    for (int l = 0; l < 3; ++l)
      for (int q = 0; q < nd[l]; ++q) {
        h = fnv1a(h, &sizes[l][q], sizeof(int));
        h = fnv1a(h, grids[l][q], sizeof(double) * sizes[l][q]);
      }
    h = fnv1a(h, bct, 6 * sizeof(int));
    h = fnv1a(h, &so, sizeof(int));
    md->geom_key = h;
  }
  if (!rc)
  if (!rc) rc = md->rint.ensure(max_field * 8);
  if (!rc) rc = md->zero_int.ensure(max_field * 8);
  if (!rc) rc = md->ufield.ensure(max_field * 8);
  if (!rc) rc = md->vec.ensure(sizeof(double) * kMdMaxRhs * std::max<long long>(1, md->topo.ninf));
  if (!rc && (cudaMemset(md->zero_int.ptr, 0, max_field * 8) != cudaSuccess ||
              cudaDeviceSynchronize() != cudaSuccess))
    rc = set_error(MF_ERR_CUDA, "mf_md_create: memset failed");
  // the dense solver's handle (its first creation in a process loads the
  // library, which belongs to set-up rather than to a matrix assembly)
  if (!rc && cusolverDnCreate(&md->cs) != CUSOLVER_STATUS_SUCCESS)
    rc = set_error(MF_ERR_CUDA, "cusolverDnCreate failed");
  if (rc) {
    mf_md_destroy(md);
    return rc;
  }
  *out = md;
  return MF_OK;
}

int mf_md_destroy(mf_md_t* md) {
  if (!md) return MF_OK;
  for (auto& sd : md->sub) {
    mf_solver3d_destroy(sd.sc);
    for (int l = 0; l < 3; ++l) {
      mf_der_destroy(sd.dc[l]);
      sd.bc[l].release();
      sd.facew[l].release();
    }
    sd.rint.release();
    if (sd.stream) cudaStreamDestroy(sd.stream);
    if (sd.done) cudaEventDestroy(sd.done);
  }
  if (md->fork) cudaEventDestroy(md->fork);
  for (DevBuf* b : {&md->Minv, &md->vec2, &md->ub, &md->dub[0], &md->dub[1], &md->dub[2], &md->bcb}) b->release();
  for (DevBuf* b : {&md->pdinv, &md->pw, &md->pflags, &md->perr})
    b->release();
  for (DevBuf* b : {&md->perm, &md->dinv, &md->lu_v, &md->lu_y, &md->M, &md->ipiv, &md->vec, &md->info,
                    &md->work, &md->zero_int, &md->rint, &md->ufield})
    b->release();
  if (md->cs) cusolverDnDestroy(md->cs);
  if (md->cb) cublasDestroy(md->cb);
  delete md;
  return MF_OK;
}

int mf_md_ninf(const mf_md_t* md, long long* ninf, int* it) {
  if (!md) return set_error(MF_ERR_ARG, "mf_md_ninf: null handle");
  if (ninf) *ninf = md->topo.ninf;
  if (it) *it = md->topo.it;
  return MF_OK;
}

// Influence columns by solves: all Dirac columns of one subdomain face
// solved together, in chunks of B problems: one batched solve (zero
// right-hand side and zero data on the other faces shared between the
// problems), one batched derivative sweep per axis (the B fields stacked
// along z, or viewed as (nx*ny, nz, B) for z lines, all lines plain: the
// gathered face values come from interior lines only), and one batched
// gather into B consecutive columns.
static int md_assemble_solves(mf_md* md, double* M, cudaStream_t st) {
  const long long n = md->topo.ninf;
  const MdTopology& t = md->topo;
  int rc;
  for (int k = 0; k < t.nd[2]; ++k)
    for (int j = 0; j < t.nd[1]; ++j)
      for (int i = 0; i < t.nd[0]; ++i) {
        const int s = md_sub_index(md, i, j, k);
        mf_md::Sub& sd = md->sub[s];
        const int nx = sd.n[0], ny = sd.n[1], nz = sd.n[2];
        const long long nfull = (long long)nx * ny * nz;
        const long long nint = (long long)(nx - 2) * (ny - 2) * (nz - 2);
        for (int l2 = 0; l2 < 3; ++l2)
          MF_CUDA(cudaMemsetAsync(sd.bc[l2].ptr, 0, sizeof(double) * 2 * face_points(sd, l2), st));
        bool need[3] = {false, false, false};
        for (int l2 = 0; l2 < 3; ++l2)
          for (int m2 = 0; m2 < 2; ++m2)
            if (t.get(i, j, k, l2, m2) > 0) need[l2] = true;
        // chunk size: fields, three derivative fields and the solver's two
        // work arrays per problem within about 2 GB
        const long long per = 8 * (4 * nfull + 2 * nint);
        const int bmax = (int)std::max(1LL, std::min(65535LL, (2LL << 30) / per));
        for (int m = 0; m < 2; ++m)
          for (int l = 0; l < 3; ++l) {
            const int p = t.get(i, j, k, l, m);
            if (p <= 0) continue;
            const long long nf = face_points(sd, l);
            for (long long q0 = 0; q0 < t.size[p - 1]; q0 += bmax) {
              const int B = (int)std::min<long long>(bmax, t.size[p - 1] - q0);
              if ((rc = md->ub.ensure((size_t)B * nfull * 8)) || (rc = md->bcb.ensure((size_t)B * 2 * nf * 8)))
                return rc;
              for (int l2 = 0; l2 < 3; ++l2)
                if (need[l2] && (rc = md->dub[l2].ensure((size_t)B * nfull * 8))) return rc;
              double* U = md->ub.as<double>();
              MF_CUDA(cudaMemsetAsync(U, 0, (size_t)B * nfull * 8, st));
              MF_CUDA(cudaMemsetAsync(md->bcb.ptr, 0, (size_t)B * 2 * nf * 8, st));
              k_dirac_batch<<<nblk(B, 128), 128, 0, st>>>(md->bcb.as<double>(), nf, m, q0, B);
              MF_CUDA(cudaGetLastError());
              const double* bc[3] = {sd.bc[0].as<double>(), sd.bc[1].as<double>(), sd.bc[2].as<double>()};
              long long bs[3] = {0, 0, 0};
              bc[l] = md->bcb.as<double>();
              bs[l] = 2 * nf;
              if ((rc = mf_solve_3d_batch(sd.sc, B, md->zero_int.as<double>(), 0, md->sigma, U, nfull, bc[0], bs[0],
                                          bc[1], bs[1], bc[2], bs[2], nx - 2, ny - 2, nz - 2, st)))
                return rc;
              if (need[0] && (rc = der_launch(sd.dc[0], 0, 1, 1, U, md->dub[0].as<double>(), nx, ny,
                                              (int)(nz * B), st)))
                return rc;
              if (need[1] && (rc = der_launch(sd.dc[1], 1, 1, 1, U, md->dub[1].as<double>(), nx, ny,
                                              (int)(nz * B), st)))
                return rc;
              if (need[2] && (rc = der_launch(sd.dc[2], 1, 1, 1, U, md->dub[2].as<double>(), nx * ny, nz, B, st)))
                return rc;
              double* col0 = M + (long long)n * (t.offset[p - 1] + q0);
              for (int l2 = 0; l2 < 3; ++l2)
                for (int m2 = 0; m2 < 2; ++m2) {
                  const int p2 = t.get(i, j, k, l2, m2);
                  if (p2 <= 0) continue;
                  FaceGather f{l2, m2, nx, ny, nz, (long long)t.offset[p2 - 1], -1.0};
                  k_face_gather_batch<<<dim3(nblk(t.size[p2 - 1], 128), B), 128, 0, st>>>(
                      md->dub[l2].as<double>(), nfull, col0, (long long)n, f);
                  MF_CUDA(cudaGetLastError());
                }
            }
          }
      }
  return MF_OK;
}

// Influence columns in the eigenbasis of each subdomain solver (see
// k_inf_g): per subdomain and pair of interface faces one block of n^5
// work.  The face-row derivative weights come from the subdomain's own
// derivative coefficients applied to unit vectors, the Neumann ends are the
// solver's extrapolation of the interior, and every block is placed
// straight into the matrix with the sign of the gathered derivatives.
static int md_assemble_eigen(mf_md* md, double* M, cudaStream_t st) {
  const long long n = md->topo.ninf;
  const MdTopology& t = md->topo;
  int rc;
  // the batched products put one face-point pair per CTA row (grid.y): fall
  // back to the solves beyond 65,535
  for (const mf_md::Sub& sd : md->sub)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        if ((long long)(sd.n[a] - 2) * (sd.n[b] - 2) > 65535) return md_assemble_solves(md, M, st);
  for (int k = 0; k < t.nd[2]; ++k)
    for (int j = 0; j < t.nd[1]; ++j)
      for (int i = 0; i < t.nd[0]; ++i) {
        bool any = false;
        for (int l = 0; l < 3; ++l)
          for (int m = 0; m < 2; ++m) any = any || t.get(i, j, k, l, m) > 0;
        if (!any) continue;
        mf_md::Sub& sd = md->sub[md_sub_index(md, i, j, k)];
        SolverAxisView ax[3];
        std::vector<double> V[3], Vi[3], omega[3][2], psi[3][2], W[3][2];
        for (int a = 0; a < 3; ++a) {
          if ((rc = solver_axis_view(sd.sc, a, &ax[a]))) return rc;
          const int na = ax[a].n, L = na + 2;
          V[a].resize((size_t)na * na);
          Vi[a].resize((size_t)na * na);
          std::vector<double> l4((size_t)4 * na);
          MF_CUDA(cudaMemcpy(V[a].data(), ax[a].V, sizeof(double) * na * na, cudaMemcpyDeviceToHost));
          MF_CUDA(cudaMemcpy(Vi[a].data(), ax[a].Vinv, sizeof(double) * na * na, cudaMemcpyDeviceToHost));
          MF_CUDA(cudaMemcpy(l4.data(), ax[a].invl4, sizeof(double) * 4 * na, cudaMemcpyDeviceToHost));
          // rows 0 and L-1 of the full-line derivative (plain lines, as the
          // gathered face derivatives), from unit pencils
          std::vector<double> I((size_t)L * L, 0.0), D((size_t)L * L);
          for (int q = 0; q < L; ++q) I[(size_t)q * L + q] = 1.0;
          if ((rc = mf_der_lines(sd.dc[a], 1, 0, I.data(), D.data(), L, st))) return rc;
          for (int m2 = 0; m2 < 2; ++m2) {
            W[a][m2].resize(L);
            for (int q = 0; q < L; ++q) W[a][m2][q] = D[(size_t)q * L + (m2 ? L - 1 : 0)];
            std::vector<double> weff(W[a][m2].begin() + 1, W[a][m2].begin() + 1 + na);
            const double* d = ax[a].neum;
            if (ax[a].bc[0] == 2 || ax[a].bc[0] == 3)
              for (int mm = 1; mm <= 6 && mm - 1 < na; ++mm) weff[mm - 1] += W[a][m2][0] * (-d[mm] * (1.0 / d[0]));
            if (ax[a].bc[1] == 2 || ax[a].bc[1] == 3)
              for (int mm = 0; mm < 6; ++mm)
                if (na - 6 + mm >= 0) weff[na - 6 + mm] += W[a][m2][L - 1] * (-d[7 + mm] * (1.0 / d[13]));
            omega[a][m2].assign(na, 0.0);
            for (int p = 0; p < na; ++p) {
              double acc = 0.0;
              for (int q = 0; q < na; ++q) acc += weff[q] * V[a][(size_t)q * na + p];
              omega[a][m2][p] = acc;
            }
          }
          for (int m = 0; m < 2; ++m) {
            const int c0 = m ? 2 : 0, c1 = m ? 3 : 1;
            std::vector<double> phi(na);
            for (int q = 0; q < na; ++q)
              phi[q] = -(l4[(size_t)c0 * na + q] * ax[a].bcc[c0] + l4[(size_t)c1 * na + q] * ax[a].bcc[c1]);
            psi[a][m].assign(na, 0.0);
            for (int p = 0; p < na; ++p) {
              double acc = 0.0;
              for (int q = 0; q < na; ++q) acc += Vi[a][(size_t)p * na + q] * phi[q];
              psi[a][m][p] = acc;
            }
          }
        }
        const Lam3 L3{{ax[0].eig, ax[1].eig, ax[2].eig}};
        const long long n3max = (long long)std::max({ax[0].n, ax[1].n, ax[2].n});
        if ((rc = md->inf_w[0].ensure(sizeof(double) * 2 * n3max * n3max)) ||
            (rc = md->inf_w[1].ensure(sizeof(double) * n3max * n3max)) ||
            (rc = md->inf_w[2].ensure(sizeof(double) * n3max * n3max * n3max)) ||
            (rc = md->inf_w[3].ensure(sizeof(double) * n3max * n3max * n3max)) ||
            (rc = md->inf_w[4].ensure(sizeof(double) * n3max * n3max * n3max)))
          return rc;
        double* small = md->inf_w[0].as<double>();
        double* G = md->inf_w[1].as<double>();
        double* Ust = md->inf_w[2].as<double>();
        double* F = md->inf_w[3].as<double>();
        double* H = md->inf_w[4].as<double>();
        for (int m = 0; m < 2; ++m)
          for (int l = 0; l < 3; ++l) {
            const int p = t.get(i, j, k, l, m);
            if (p <= 0) continue;
            const long long col0 = t.offset[p - 1];
            for (int m2 = 0; m2 < 2; ++m2)
              for (int l2 = 0; l2 < 3; ++l2) {
                const int p2 = t.get(i, j, k, l2, m2);
                if (p2 <= 0) continue;
                const long long row0 = t.offset[p2 - 1];
                const double scale = m2 ? -1.0 : 1.0;
                if (l2 == l) {
                  const int b1 = l == 0 ? 1 : 0, b2 = l == 2 ? 1 : 2;
                  const int nl = ax[l].n, n1 = ax[b1].n, n2 = ax[b2].n;
                  std::vector<double> w(nl);
                  for (int q = 0; q < nl; ++q) w[q] = omega[l][m2][q] * psi[l][m][q];
                  MF_CUDA(cudaMemcpyAsync(small, w.data(), sizeof(double) * nl, cudaMemcpyHostToDevice, st));
                  k_inf_g<<<nblk((long long)n1 * n2, 256), 256, 0, st>>>(L3, md->sigma, l, b1, b2, nl, n1, n2, small, G);
                  const Place PA{0, n1, 1, 0, 0, (long long)n1 * n2, 0, 0, 1, 1.0, 0};
                  k_inf_adb<<<dim3(nblk((long long)n2 * n2, 256), n1), 256, 0, st>>>(
                      ax[b2].V, ax[b2].Vinv, n2, n2, n2, G, 1, 0, n1, n1, Ust, PA);
                  const Place PB{row0, 1, n1, 0, col0, 1, 0, n1, n, scale, 1};
                  k_inf_adb<<<dim3(nblk((long long)n1 * n1, 256), n2 * n2), 256, 0, st>>>(
                      ax[b1].V, ax[b1].Vinv, n1, n1, n1, Ust, n1, (long long)n1 * n2, 1, n2, M, PB);
                  k_inf_direct<<<nblk((long long)n1 * n2, 256), 256, 0, st>>>(
                      M, n, row0, col0, (long long)n1 * n2, scale * W[l][m2][m ? nl + 1 : 0]);
                } else {
                  const int k3 = 3 - l - l2;
                  const int nl = ax[l].n, n2 = ax[l2].n, nk = ax[k3].n;
                  std::vector<double> YZ((size_t)n2 * n2 + (size_t)nl * nl);
                  for (int q = 0; q < n2; ++q)
                    for (int c = 0; c < n2; ++c) YZ[(size_t)q * n2 + c] = omega[l2][m2][q] * Vi[l2][(size_t)q * n2 + c];
                  double* Zh = YZ.data() + (size_t)n2 * n2;
                  for (int r = 0; r < nl; ++r)
                    for (int q = 0; q < nl; ++q) Zh[(size_t)r * nl + q] = V[l][(size_t)r * nl + q] * psi[l][m][q];
                  MF_CUDA(cudaMemcpyAsync(small, YZ.data(), sizeof(double) * YZ.size(), cudaMemcpyHostToDevice, st));
                  MF_CUDA(cudaStreamSynchronize(st));  // YZ is a host temporary
                  const long long cube = (long long)nl * n2 * nk;
                  k_inf_f<<<nblk(cube, 256), 256, 0, st>>>(L3, md->sigma, l, l2, k3, nl, n2, nk, small, F);
                  k_inf_h<<<nblk(cube, 256), 256, 0, st>>>(small + (size_t)n2 * n2, F, nl, n2, nk, H);
                  long long ri, rb1, cj, cb2;
                  if (l < k3) { rb1 = 1; ri = nl; } else { ri = 1; rb1 = nk; }
                  if (l2 < k3) { cb2 = 1; cj = n2; } else { cj = 1; cb2 = nk; }
                  const Place PC{row0, ri, rb1, 0, col0, cj, 0, cb2, n, scale, 1};
                  k_inf_adb<<<dim3(nblk((long long)nk * nk, 256), nl * n2), 256, 0, st>>>(
                      ax[k3].V, ax[k3].Vinv, nk, nk, nk, H, 1, nl, (long long)nl * n2, nl, M, PC);
                }
                MF_CUDA(cudaGetLastError());
                MF_CUDA(cudaStreamSynchronize(st));  // the host vectors of this block are reused
              }
          }
      }
  return MF_OK;
}

static int md_factor_finish(mf_md* md, cudaStream_t st);

int mf_md_influence_matrix_set(mf_md_t* md, double sigma, int null_mode, void* stream) {
  if (!md || null_mode < 0 || null_mode > 2)
    return set_error(MF_ERR_ARG, "mf_md_influence_matrix_set: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long n = md->topo.ninf;
  if (n == 0) return set_error(MF_ERR_ARG, "mf_md_influence_matrix_set: no interface");
  md->sigma = sigma;
  md->null_mode = null_mode;
  int rc;
  if ((rc = md->M.ensure(sizeof(double) * n * n)) || (rc = md->ipiv.ensure(sizeof(int) * n)) ||
      (rc = md->info.ensure(sizeof(int))))
    return rc;
  MF_CUDA(cudaMemsetAsync(md->M.ptr, 0, sizeof(double) * n * n, st));
  double* M = md->M.as<double>();
  double* u = md->ufield.as<double>();
  const MdTopology& t = md->topo;
  // md_influence_matrix_set: a Dirac on every interface point of every
  // subdomain, solved with g = 0; the signed normal derivatives on the
  // subdomain's interface faces, negated, form that point's column.
  // All Dirac columns of one subdomain face are solved together, in chunks
  // of B problems: one batched solve (zero right-hand side and zero data on
  // the other faces shared between the problems), one batched derivative
  // sweep per axis (the B fields stacked along z, or viewed as (nx*ny, nz, B)
  // for z lines, all lines plain: the gathered face values come from
  // interior lines only), and one batched gather into B consecutive columns.
  (void)u;
  if ((rc = md->assembly == MF_MD_ASSEMBLY_SOLVES ? md_assemble_solves(md, M, st) : md_assemble_eigen(md, M, st)))
    return rc;
  if (null_mode >= 1) {
    k_pin_row0<<<nblk(n, 256), 256, 0, st>>>(M, (int)n);
    MF_CUDA(cudaGetLastError());
  }
  // LU factorisation (set-up): cuSOLVER getrf, FP64
  if (!md->cs && cusolverDnCreate(&md->cs) != CUSOLVER_STATUS_SUCCESS)
    return set_error(MF_ERR_CUDA, "cusolverDnCreate failed");
  cusolverDnSetStream(md->cs, st);
  int lwork = 0;
  if (cusolverDnDgetrf_bufferSize(md->cs, (int)n, (int)n, M, (int)n, &lwork) != CUSOLVER_STATUS_SUCCESS)
    return set_error(MF_ERR_CUDA, "getrf buffer query failed");
  if ((rc = md->work.ensure(sizeof(double) * std::max(1, lwork)))) return rc;
  if (cusolverDnDgetrf(md->cs, (int)n, (int)n, M, (int)n, md->work.as<double>(), md->ipiv.as<int>(),
                       md->info.as<int>()) != CUSOLVER_STATUS_SUCCESS)
    return set_error(MF_ERR_CUDA, "getrf failed");
  int hinfo = 0;
  MF_CUDA(cudaMemcpyAsync(&hinfo, md->info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  MF_CUDA(cudaStreamSynchronize(st));
  if (hinfo != 0)
    return set_error(MF_ERR_SINGULAR, "influence matrix is singular (getrf info %d)%s", hinfo,
                     null_mode ? "" : "; an all-Neumann problem needs a null-space mode");
  return md_factor_finish(md, st);
}

// After the LU factor and the pivots are in md->M, md->ipiv: the set-up of
// the triangular solves and, when wanted, the explicit inverse.
// In-place inverse of the n x n upper (or lower) triangular block at A
// (column-major, leading dimension lda, non-unit diagonal).  cuSOLVER's trtri
// is called on blocks of at most 2^28 entries (above 2^31 it fails: 46,860^2
// does; the lower limit puts systems above 16,384 unknowns, 18,252 in the
// tests, through the blocked form); a larger block is split in halves, both
// inverted the same way, and
// the off-diagonal block formed by two in-place triangular products:
// U12 <- -U11^-1 U12 U22^-1, L21 <- -L22^-1 L21 L11^-1.  n^3 / 3 flops either
// way.
static int tri_invert(mf_md* md, double* A, long long lda, long long n, bool upper, cudaStream_t st) {
  if (n * n <= (1LL << 28)) {
    const cublasFillMode_t fill = upper ? CUBLAS_FILL_MODE_UPPER : CUBLAS_FILL_MODE_LOWER;
    size_t dws = 0, hws = 0;
    if (cusolverDnXtrtri_bufferSize(md->cs, fill, CUBLAS_DIAG_NON_UNIT, n, CUDA_R_64F, A, lda, &dws, &hws) !=
        CUSOLVER_STATUS_SUCCESS)
      return set_error(MF_ERR_CUDA, "trtri buffer query failed (n %lld)", n);
    int rc;
    if ((rc = md->work.ensure(std::max(dws, (size_t)8)))) return rc;
    std::vector<char> hwork(std::max(hws, (size_t)8));
    if (cusolverDnXtrtri(md->cs, fill, CUBLAS_DIAG_NON_UNIT, n, CUDA_R_64F, A, lda, md->work.ptr, dws, hwork.data(),
                         hws, md->info.as<int>()) != CUSOLVER_STATUS_SUCCESS)
      return set_error(MF_ERR_CUDA, "trtri (inverse of an LU factor block, n %lld) failed", n);
    int hinfo = 0;
    MF_CUDA(cudaMemcpyAsync(&hinfo, md->info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    MF_CUDA(cudaStreamSynchronize(st));  // the host workspace lives until here
    if (hinfo != 0) return set_error(MF_ERR_SINGULAR, "trtri info %d", hinfo);
    return MF_OK;
  }
  const long long n1 = (n / 2 + 31) / 32 * 32, n2 = n - n1;
  double* A11 = A;
  double* A22 = A + n1 + lda * n1;
  int rc;
  if ((rc = tri_invert(md, A11, lda, n1, upper, st)) || (rc = tri_invert(md, A22, lda, n2, upper, st))) return rc;
  if (!md->cb && cublasCreate(&md->cb) != CUBLAS_STATUS_SUCCESS)
    return set_error(MF_ERR_CUDA, "cublasCreate failed");
  cublasSetStream(md->cb, st);
  const double one = 1.0, minus = -1.0;
  const cublasFillMode_t fill = upper ? CUBLAS_FILL_MODE_UPPER : CUBLAS_FILL_MODE_LOWER;
  bool ok;
  if (upper) {  // A12: n1 x n2 at column n1
    double* B = A + lda * n1;
    ok = cublasDtrmm_64(md->cb, CUBLAS_SIDE_LEFT, fill, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n1, n2, &one, A11, lda,
                        B, lda, B, lda) == CUBLAS_STATUS_SUCCESS &&
         cublasDtrmm_64(md->cb, CUBLAS_SIDE_RIGHT, fill, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n1, n2, &minus, A22,
                        lda, B, lda, B, lda) == CUBLAS_STATUS_SUCCESS;
  } else {  // A21: n2 x n1 at row n1
    double* B = A + n1;
    ok = cublasDtrmm_64(md->cb, CUBLAS_SIDE_RIGHT, fill, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n2, n1, &one, A11, lda,
                        B, lda, B, lda) == CUBLAS_STATUS_SUCCESS &&
         cublasDtrmm_64(md->cb, CUBLAS_SIDE_LEFT, fill, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n2, n1, &minus, A22,
                        lda, B, lda, B, lda) == CUBLAS_STATUS_SUCCESS;
  }
  if (!ok) return set_error(MF_ERR_CUDA, "trmm (blocked triangular inverse) failed");
  return MF_OK;
}

static int md_factor_finish(mf_md* md, cudaStream_t st) {
  const long long n = md->topo.ninf;
  double* M = md->M.as<double>();
  int rc, hinfo = 0;
  cusolverDnSetStream(md->cs, st);
  {
    // LU solve set-up: the interchanges as one permutation, the inverses of
    // the diagonal blocks of L and U
    std::vector<int> piv(n), perm(n);
    MF_CUDA(cudaMemcpy(piv.data(), md->ipiv.ptr, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (long long i = 0; i < n; ++i) perm[i] = (int)i;
    for (long long k = 0; k < n; ++k) std::swap(perm[k], perm[piv[k] - 1]);
    const int nblocks = (int)((n + kTriBlock - 1) / kTriBlock);
    const size_t smem = sizeof(double) * kTriBlock * kTriBlock;
    if ((rc = md->perm.ensure(sizeof(int) * n)) || (rc = md->lu_v.ensure(sizeof(double) * n)) ||
        (rc = md->lu_y.ensure(sizeof(double) * n)) ||
        (rc = md->dinv.ensure(2 * (size_t)nblocks * smem)))
      return rc;
    MF_CUDA(cudaMemcpy(md->perm.ptr, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    // persistent solves: 64-row block inverses and the W blocks of both factors
    {
      int coop = 0, dev = 0;
      MF_CUDA(cudaGetDevice(&dev));
      MF_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
      const int pnb = (int)((n + kPb - 1) / kPb);
      const size_t pbs = (size_t)kPb * kPb * sizeof(double);
      md->persist_ok = false;
      if (coop && (rc = md->pdinv.ensure(2 * (size_t)pnb * pbs)) == MF_OK &&
          (rc = md->pw.ensure(2 * (size_t)pnb * pbs)) == MF_OK &&
          (rc = md->pflags.ensure(2 * sizeof(int) * pnb)) == MF_OK &&
          (rc = md->perr.ensure(sizeof(int))) == MF_OK &&
          (rc = md->lu_v.ensure(sizeof(double) * kMdMaxRhs * n)) == MF_OK &&
          (rc = md->lu_y.ensure(sizeof(double) * kMdMaxRhs * n)) == MF_OK) {
        double* pd = md->pdinv.as<double>();
        double* pw = md->pw.as<double>();
        const size_t half = (size_t)pnb * kPb * kPb;
        k_pdinv<<<pnb, 256, 0, st>>>(M, (int)n, 0, pd);
        k_pdinv<<<pnb, 256, 0, st>>>(M, (int)n, 1, pd + half);
        k_pw<<<pnb, 256, 0, st>>>(M, (int)n, 0, pd, pw);
        k_pw<<<pnb, 256, 0, st>>>(M, (int)n, 1, pd + half, pw + half);
        MF_CUDA(cudaMemsetAsync(md->perr.ptr, 0, sizeof(int), st));
        MF_CUDA(cudaGetLastError());
        md->persist_ok = true;
      }
      if (rc) return rc;
    }
    MF_CUDA(cudaFuncSetAttribute(k_tri_block_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_tri_block_inverse<<<nblocks, 256, smem, st>>>(M, (int)n, 0, md->dinv.as<double>());
    k_tri_block_inverse<<<nblocks, 256, smem, st>>>(M, (int)n, 1,
                                                    md->dinv.as<double>() + (size_t)nblocks * kTriBlock * kTriBlock);
    MF_CUDA(cudaGetLastError());
  }
  // the inverse, row-major: A^T X = I gives X = A^-T column-major, i.e. A^-1
  // stored by rows.  Forming it costs 2 n^3 FP64 flops (three times the LU),
  // a few seconds at n = 12,000 on the FP64 pipe; above that, when it does
  // not fit, or when the triangular form is selected, the solves stay on the
  // LU factors.
  md->inv_ok = false;
  if ((md->iface_mode == MF_MD_IFACE_AUTO && n <= kMaxInverseRows) || md->iface_mode == MF_MD_IFACE_INVERSE) {
    const size_t bytes = sizeof(double) * (size_t)n * (size_t)n;
    size_t freeb = 0, totalb = 0;
    MF_CUDA(cudaMemGetInfo(&freeb, &totalb));
    if (bytes < freeb / 2 && md->Minv.ensure(bytes) == MF_OK && md->vec2.ensure(sizeof(double) * kMdMaxRhs * n) == MF_OK) {
      double* X = md->Minv.as<double>();
      k_identity<<<nblk((long long)n * n, 256), 256, 0, st>>>(X, (int)n);
      MF_CUDA(cudaGetLastError());
      if (cusolverDnDgetrs(md->cs, CUBLAS_OP_T, (int)n, (int)n, M, (int)n, md->ipiv.as<int>(), X,
                           (int)n, md->info.as<int>()) != CUSOLVER_STATUS_SUCCESS)
        return set_error(MF_ERR_CUDA, "getrs (inverse of the influence matrix) failed");
      MF_CUDA(cudaMemcpyAsync(&hinfo, md->info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
      MF_CUDA(cudaStreamSynchronize(st));
      if (hinfo != 0) return set_error(MF_ERR_SINGULAR, "getrs info %d", hinfo);
      md->inv_ok = true;
    } else {
      (void)cudaGetLastError();  // a refused allocation is not an error here
      md->Minv.release();
    }
  }
  // the inverted factors, row-major (above 12,000 unknowns by default): U
  // inverted in one copy of the LU factor, L in another with its diagonal set
  // to one (trtri, n^3 / 3 FP64 flops each: together the cost of the getrf;
  // each call is trusted with its own triangle only), the strict lower part of
  // the second merged into the first while it is transposed so that a row is
  // contiguous.  A solve reads the n x n array once, as the triangular solves
  // do, but its rows are independent.  The LU factor stays as it is (factor
  // cache, the MF_MD_IFACE_LU form).
  md->trinv_ok = md->trinv_df = false;
  if (!md->inv_ok && ((md->iface_mode == MF_MD_IFACE_AUTO && n > kMaxInverseRows) ||
                      md->iface_mode == MF_MD_IFACE_TRIANGULAR_INVERSE ||
                      md->iface_mode == MF_MD_IFACE_TRIANGULAR_INVERSE_FP64)) {
    const size_t bytes = sizeof(double) * (size_t)n * (size_t)n;
    size_t freeb = 0, totalb = 0;
    MF_CUDA(cudaMemGetInfo(&freeb, &totalb));
    DevBuf lcopy;
    struct Release {
      DevBuf& b;
      ~Release() { b.release(); }
    } release_lcopy{lcopy};  // every return below frees the copy of L
    if (bytes < freeb / 3 && md->Minv.ensure(bytes) == MF_OK && lcopy.ensure(bytes) == MF_OK &&
        md->vec2.ensure(sizeof(double) * kMdMaxRhs * n) == MF_OK) {
      double* T = md->Minv.as<double>();
      double* Lc = lcopy.as<double>();
      MF_CUDA(cudaMemcpyAsync(T, M, bytes, cudaMemcpyDeviceToDevice, st));
      MF_CUDA(cudaMemcpyAsync(Lc, M, bytes, cudaMemcpyDeviceToDevice, st));
      k_unit_diagonal<<<nblk(n, 256), 256, 0, st>>>(Lc, (int)n);
      MF_CUDA(cudaGetLastError());
      if ((rc = tri_invert(md, T, n, n, true, st)) || (rc = tri_invert(md, Lc, n, n, false, st))) return rc;
      const unsigned tiles = (unsigned)((n + 31) / 32);
      k_transpose_square<<<dim3(tiles, tiles), 256, 0, st>>>(T, Lc, (int)n);
      MF_CUDA(cudaGetLastError());
      MF_CUDA(cudaStreamSynchronize(st));  // before the copy of L is freed
      lcopy.release();
      md->trinv_ok = true;
      // double-float pairs in place, unless FP64 arithmetic is asked for or
      // the factors hold a non-finite entry
      rc = MF_OK;
      if (md->iface_mode != MF_MD_IFACE_TRIANGULAR_INVERSE_FP64 &&
          (rc = md->dfmax.ensure(sizeof(unsigned long long))) == MF_OK &&
          (rc = md->xdf.ensure(sizeof(float2) * kMdMaxRhs * n)) == MF_OK &&
          (rc = md->unscale.ensure(sizeof(double) * kMdMaxRhs)) == MF_OK) {
        const long long count = n * n;
        MF_CUDA(cudaMemsetAsync(md->dfmax.ptr, 0, sizeof(unsigned long long), st));
        k_df_range<<<1216, 256, 0, st>>>(T, count, md->dfmax.as<unsigned long long>());
        MF_CUDA(cudaGetLastError());
        unsigned long long bits = 0;
        MF_CUDA(cudaMemcpyAsync(&bits, md->dfmax.ptr, sizeof(bits), cudaMemcpyDeviceToHost, st));
        MF_CUDA(cudaStreamSynchronize(st));
        double tmax;
        std::memcpy(&tmax, &bits, sizeof(tmax));
        if (tmax > 0.0 && tmax <= 1.7e308) {
          const int ex = std::ilogb(tmax);
          k_df_convert<<<1216, 256, 0, st>>>(T, count, std::scalbn(1.0, -ex));
          MF_CUDA(cudaGetLastError());
          md->trinv_tscale = std::scalbn(1.0, ex);
          md->trinv_df = true;
        }
      }
      if (rc) return rc;
    } else {
      (void)cudaGetLastError();
      md->Minv.release();
    }
  }
  md->factored = true;
  return MF_OK;
}

// Factor cache: one raw little-endian file per influence matrix.  Layout:
// magic "MFMDLU01", uint64 key, int64 n, sigma, int32 null_mode, then the LU
// factor (n x n FP64, column-major) and the pivots (n int32), in chunks.
constexpr char kFacMagic[8] = {'M', 'F', 'M', 'D', 'L', 'U', '0', '1'};
constexpr size_t kFacChunk = (size_t)32 << 20;  // doubles per transfer (256 MB)

int mf_md_factor_key(const mf_md_t* md, double sigma, int null_mode, char key[17]) {
  if (!md || !key) return set_error(MF_ERR_ARG, "mf_md_factor_key: null argument");
  std::snprintf(key, 17, "%016llx", (unsigned long long)factor_key(md, sigma, null_mode));
  return MF_OK;
}

int mf_md_save_factor(const mf_md_t* md, const char* path) {
  if (!md || !path) return set_error(MF_ERR_ARG, "mf_md_save_factor: null argument");
  if (!md->factored) return set_error(MF_ERR_ARG, "mf_md_save_factor: influence matrix not set");
  MF_CUDA(cudaDeviceSynchronize());
  const long long n = md->topo.ninf;
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(MF_ERR_ARG, "mf_md_save_factor: cannot open %s", path);
  const uint64_t key = factor_key(md, md->sigma, md->null_mode);
  bool ok = std::fwrite(kFacMagic, 1, 8, f) == 8 && std::fwrite(&key, 8, 1, f) == 1 &&
            std::fwrite(&n, 8, 1, f) == 1 && std::fwrite(&md->sigma, 8, 1, f) == 1 &&
            std::fwrite(&md->null_mode, 4, 1, f) == 1;
  std::vector<double> buf(std::min<size_t>(kFacChunk, (size_t)n * n));
  for (size_t off = 0; ok && off < (size_t)n * n; off += buf.size()) {
    const size_t cnt = std::min<size_t>(buf.size(), (size_t)n * n - off);
    ok = cudaMemcpy(buf.data(), md->M.as<double>() + off, cnt * 8, cudaMemcpyDeviceToHost) == cudaSuccess &&
         std::fwrite(buf.data(), 8, cnt, f) == cnt;
  }
  std::vector<int> piv(n);
  ok = ok && cudaMemcpy(piv.data(), md->ipiv.ptr, sizeof(int) * n, cudaMemcpyDeviceToHost) == cudaSuccess &&
       std::fwrite(piv.data(), 4, n, f) == (size_t)n;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MF_OK : set_error(MF_ERR_CUDA, "mf_md_save_factor: writing %s failed", path);
}

int mf_md_load_factor(mf_md_t* md, double sigma, int null_mode, const char* path, void* stream) {
  if (!md || !path || null_mode < 0 || null_mode > 2)
    return set_error(MF_ERR_ARG, "mf_md_load_factor: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MF_CUDA(cudaStreamSynchronize(st));
  const long long n = md->topo.ninf;
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(MF_ERR_ARG, "mf_md_load_factor: cannot open %s", path);
  char magic[8];
  uint64_t key = 0;
  long long fn = 0;
  double fsigma = 0.0;
  int fnull = -1;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kFacMagic, 8) == 0 &&
            std::fread(&key, 8, 1, f) == 1 && std::fread(&fn, 8, 1, f) == 1 && std::fread(&fsigma, 8, 1, f) == 1 &&
            std::fread(&fnull, 4, 1, f) == 1 && key == factor_key(md, sigma, null_mode) && fn == n;
  if (!ok) {
    std::fclose(f);
    return set_error(MF_ERR_ARG, "mf_md_load_factor: %s is not the factor of this problem", path);
  }
  int rc;
  if ((rc = md->M.ensure(sizeof(double) * n * n)) || (rc = md->ipiv.ensure(sizeof(int) * n)) ||
      (rc = md->info.ensure(sizeof(int)))) {
    std::fclose(f);
    return rc;
  }
  md->factored = false;
  std::vector<double> buf(std::min<size_t>(kFacChunk, (size_t)n * n));
  for (size_t off = 0; ok && off < (size_t)n * n; off += buf.size()) {
    const size_t cnt = std::min<size_t>(buf.size(), (size_t)n * n - off);
    ok = std::fread(buf.data(), 8, cnt, f) == cnt &&
         cudaMemcpy(md->M.as<double>() + off, buf.data(), cnt * 8, cudaMemcpyHostToDevice) == cudaSuccess;
  }
  std::vector<int> piv(n);
  ok = ok && std::fread(piv.data(), 4, n, f) == (size_t)n;
  for (long long k = 0; ok && k < n; ++k) ok = piv[k] >= 1 && piv[k] <= n;
  ok = ok && cudaMemcpy(md->ipiv.ptr, piv.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  std::fclose(f);
  if (!ok) return set_error(MF_ERR_ARG, "mf_md_load_factor: %s is truncated or damaged", path);
  md->sigma = sigma;
  md->null_mode = null_mode;
  return md_factor_finish(md, st);
}

int mf_md_influence_matrix_cached(mf_md_t* md, double sigma, int null_mode, const char* dir, void* stream) {
  if (!md || !dir) return set_error(MF_ERR_ARG, "mf_md_influence_matrix_cached: null argument");
  char key[17];
  int rc = mf_md_factor_key(md, sigma, null_mode, key);
  if (rc) return rc;
  const std::string path = std::string(dir) + "/" + key + ".mffac";
  if (FILE* f = std::fopen(path.c_str(), "rb")) {
    std::fclose(f);
    if (mf_md_load_factor(md, sigma, null_mode, path.c_str(), stream) == MF_OK) return MF_OK;
  }
  if ((rc = mf_md_influence_matrix_set(md, sigma, null_mode, stream))) return rc;
  return mf_md_save_factor(md, path.c_str());
}

// multidomain_solve for nrhs right-hand sides of the same operator; the
// pointer arrays hold nrhs x (subdomain count) entries, right-hand side
// major.  The subdomain work of the right-hand sides runs one after the other
// on each subdomain's stream; the interface system is solved for all of them
// in one pass over the inverse (or column by column on the LU factors).
// The interface systems of nrhs right-hand sides stored one after the other
// at vecs (n each), solved in place in the form selected at set-up; null-space
// handling as md_rhs_nullspace / md_vector_zero_lastpoint (class_md.f90).
static int md_interface_system(mf_md* md, int nrhs, double* vecs, cudaStream_t st) {
  const long long n = md->topo.ninf;
  int rc = MF_OK;
  for (int r = 0; r < nrhs; ++r) {
    if (md->null_mode == 1) k_remove_mean<<<1, 256, 0, st>>>(vecs + (size_t)r * n, (int)n);
    if (md->null_mode >= 1) k_set_scalar<<<1, 1, 0, st>>>(vecs + (size_t)r * n, 0, 0.0);
  }
  if (md->inv_ok && md->iface_mode != MF_MD_IFACE_LU) {
    const double* A = md->Minv.as<double>();
    double* y = md->vec2.as<double>();
    const unsigned blocks = nblk(n, kGemvRows), threads = 32 * kGemvRows;
    if (nrhs == 1) k_gemm_rows<1><<<blocks, threads, 0, st>>>(A, vecs, y, (int)n);
    if (nrhs == 2) k_gemm_rows<2><<<blocks, threads, 0, st>>>(A, vecs, y, (int)n);
    if (nrhs == 3) k_gemm_rows<3><<<blocks, threads, 0, st>>>(A, vecs, y, (int)n);
    if (nrhs == 4) k_gemm_rows<4><<<blocks, threads, 0, st>>>(A, vecs, y, (int)n);
    MF_CUDA(cudaGetLastError());
    MF_CUDA(cudaMemcpyAsync(vecs, y, sizeof(double) * n * nrhs, cudaMemcpyDeviceToDevice, st));
  } else if (md->trinv_ok && md->trinv_df && md->iface_mode != MF_MD_IFACE_LU) {
    // x = U^-1 (L^-1 (P x)) in double-float: the pivots gathered (FP64 copy
    // for the unit diagonal) and split, the lower product into vecs, its
    // result split, the upper product into vecs
    const float2* T = reinterpret_cast<const float2*>(md->Minv.as<double>());
    double* y = md->vec2.as<double>();
    float2* xd = md->xdf.as<float2>();
    double* us = md->unscale.as<double>();
    const double ts = md->trinv_tscale;
    const int* perm = md->perm.as<int>();
    const unsigned blocks = nblk(n, kTmvRows);
    k_df_prep<<<nrhs, 1024, 0, st>>>(vecs, perm, y, xd, us, (int)n);
    switch (nrhs) {
      case 1: k_trimv_rows_df<1, false><<<blocks, 512, 0, st>>>(T, xd, y, us, ts, vecs, (int)n); break;
      case 2: k_trimv_rows_df<2, false><<<blocks, 512, 0, st>>>(T, xd, y, us, ts, vecs, (int)n); break;
      case 3: k_trimv_rows_df<3, false><<<blocks, 512, 0, st>>>(T, xd, y, us, ts, vecs, (int)n); break;
      default: k_trimv_rows_df<4, false><<<blocks, 512, 0, st>>>(T, xd, y, us, ts, vecs, (int)n); break;
    }
    k_df_prep<<<nrhs, 1024, 0, st>>>(vecs, nullptr, nullptr, xd, us, (int)n);
    switch (nrhs) {
      case 1: k_trimv_rows_df<1, true><<<blocks, 512, 0, st>>>(T, xd, nullptr, us, ts, vecs, (int)n); break;
      case 2: k_trimv_rows_df<2, true><<<blocks, 512, 0, st>>>(T, xd, nullptr, us, ts, vecs, (int)n); break;
      case 3: k_trimv_rows_df<3, true><<<blocks, 512, 0, st>>>(T, xd, nullptr, us, ts, vecs, (int)n); break;
      default: k_trimv_rows_df<4, true><<<blocks, 512, 0, st>>>(T, xd, nullptr, us, ts, vecs, (int)n); break;
    }
    MF_CUDA(cudaGetLastError());
  } else if (md->trinv_ok && md->iface_mode != MF_MD_IFACE_LU) {
    // x = U^-1 (L^-1 (P x)): the pivots as a gather, then two row-parallel products
    const double* T = md->Minv.as<double>();
    double* y = md->vec2.as<double>();
    for (int r = 0; r < nrhs; ++r)
      k_permute<<<nblk(n, 256), 256, 0, st>>>(vecs + (size_t)r * n, md->perm.as<int>(), y + (size_t)r * n, (int)n);
    const unsigned blocks = nblk(n, kTmvRows);
    switch (nrhs) {
      case 1: k_trimv_rows<1, false><<<blocks, 512, 0, st>>>(T, y, vecs, (int)n);
              k_trimv_rows<1, true><<<blocks, 512, 0, st>>>(T, vecs, y, (int)n); break;
      case 2: k_trimv_rows<2, false><<<blocks, 512, 0, st>>>(T, y, vecs, (int)n);
              k_trimv_rows<2, true><<<blocks, 512, 0, st>>>(T, vecs, y, (int)n); break;
      case 3: k_trimv_rows<3, false><<<blocks, 512, 0, st>>>(T, y, vecs, (int)n);
              k_trimv_rows<3, true><<<blocks, 512, 0, st>>>(T, vecs, y, (int)n); break;
      default: k_trimv_rows<4, false><<<blocks, 512, 0, st>>>(T, y, vecs, (int)n);
               k_trimv_rows<4, true><<<blocks, 512, 0, st>>>(T, vecs, y, (int)n); break;
    }
    MF_CUDA(cudaGetLastError());
    MF_CUDA(cudaMemcpyAsync(vecs, y, sizeof(double) * n * nrhs, cudaMemcpyDeviceToDevice, st));
  } else {
    bool done = false;
    if (md->tri_form != 1) {
      if (nrhs == 1) rc = md_lu_solve_persist<1>(md, vecs, st, &done);
      if (nrhs == 2) rc = md_lu_solve_persist<2>(md, vecs, st, &done);
      if (nrhs == 3) rc = md_lu_solve_persist<3>(md, vecs, st, &done);
      if (nrhs == 4) rc = md_lu_solve_persist<4>(md, vecs, st, &done);
      if (rc) return rc;
    }
    for (int r = 0; r < nrhs && !done; ++r)
      if ((rc = md_lu_solve(md, vecs + (size_t)r * n, st))) return rc;
  }
  if (md->null_mode == 1)
    for (int r = 0; r < nrhs; ++r) k_remove_mean<<<1, 256, 0, st>>>(vecs + (size_t)r * n, (int)n);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static int md_solve_impl(mf_md_t* md, int nrhs, const double* const* g, double* const* u,
                         const double* const* bcx, const double* const* bcy, const double* const* bcz,
                         void* stream) {
  if (!md || !g || !u || !bcx || !bcy || !bcz || nrhs < 1 || nrhs > kMdMaxRhs)
    return set_error(MF_ERR_ARG, "mf_md_solve: bad arguments");
  if (!md->factored) return set_error(MF_ERR_ARG, "mf_md_solve: influence matrix not set");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const MdTopology& t = md->topo;
  const long long n = t.ninf;
  const int ns = (int)md->sub.size();
  for (int s = 0; s < ns * nrhs; ++s)
    for (const void* p : {(const void*)g[s], (const void*)u[s], (const void*)bcx[s],
                          (const void*)bcy[s], (const void*)bcz[s]})
      if (!is_device_ptr(p)) return set_error(MF_ERR_ARG, "mf_md_solve: device pointers only");
  int rc;
  // Each subdomain's work runs on its own stream, forked from and joined back
  // to the caller's stream (inside a CUDA graph: parallel branches).  Streams,
  // events and per-subdomain scratch are created by the first call.
  if (!md->fork) {
    MF_CUDA(cudaEventCreateWithFlags(&md->fork, cudaEventDisableTiming));
    for (auto& sd : md->sub) {
      MF_CUDA(cudaStreamCreateWithFlags(&sd.stream, cudaStreamNonBlocking));
      MF_CUDA(cudaEventCreateWithFlags(&sd.done, cudaEventDisableTiming));
      const size_t nfull = (size_t)sd.n[0] * sd.n[1] * sd.n[2];
      if ((rc = sd.rint.ensure(nfull * 8))) return rc;
    }
  }
  auto fork = [&]() -> int {
    MF_CUDA(cudaEventRecord(md->fork, st));
    for (auto& sd : md->sub) MF_CUDA(cudaStreamWaitEvent(sd.stream, md->fork, 0));
    return MF_OK;
  };
  auto join = [&]() -> int {
    for (auto& sd : md->sub) {
      MF_CUDA(cudaEventRecord(sd.done, sd.stream));
      MF_CUDA(cudaStreamWaitEvent(st, sd.done, 0));
    }
    return MF_OK;
  };
  MF_CUDA(cudaMemsetAsync(md->vec.ptr, 0, sizeof(double) * n * nrhs, st));
  double* vec = nullptr;  // interface vector of the right-hand side in hand
  int q = 0;              // its pointer-array offset, r * ns
  auto load_bc = [&](int s, int i, int j, int k, int mode) -> int {
    mf_md::Sub& sd = md->sub[s];
    const double* src[3] = {bcx[q + s], bcy[q + s], bcz[q + s]};
    for (int l = 0; l < 3; ++l) {
      const long long nf = face_points(sd, l);
      MF_CUDA(cudaMemcpyAsync(sd.bc[l].ptr, src[l], sizeof(double) * 2 * nf, cudaMemcpyDeviceToDevice,
                              sd.stream));
      for (int m = 0; m < 2; ++m) {
        const int p = t.get(i, j, k, l, m);
        if (p <= 0) continue;
        k_face_set<<<nblk(nf, 128), 128, 0, sd.stream>>>(sd.bc[l].as<double>(), nf, m, vec, t.offset[p - 1],
                                                         mode, 0.0);
        MF_CUDA(cudaGetLastError());
      }
    }
    return MF_OK;
  };
  // 1. homogeneous-interface solves and the signed derivative jumps
  if ((rc = fork())) return rc;
  for (int r = 0; r < nrhs; ++r) {
    vec = md->vec.as<double>() + (size_t)r * n;
    q = r * ns;
    for (int k = 0; k < t.nd[2]; ++k)
      for (int j = 0; j < t.nd[1]; ++j)
        for (int i = 0; i < t.nd[0]; ++i) {
          const int s = md_sub_index(md, i, j, k);
          mf_md::Sub& sd = md->sub[s];
          if ((rc = load_bc(s, i, j, k, 0))) return rc;
          const long long tot = (long long)(sd.n[0] - 2) * (sd.n[1] - 2) * (sd.n[2] - 2);
          k_extract_int<<<nblk(tot, 256), 256, 0, sd.stream>>>(g[q + s], sd.rint.as<double>(), sd.n[0] - 2,
                                                                sd.n[1] - 2, sd.n[2] - 2);
          MF_CUDA(cudaGetLastError());
          if ((rc = md_sub_solve(md, s, sd.rint.as<double>(), u[q + s], sd.stream))) return rc;
          if ((rc = md_gather(md, i, j, k, u[q + s], vec, 1.0, sd.stream))) return rc;
        }
  }
  if ((rc = join())) return rc;
  // 2. interface systems
  double* vecs = md->vec.as<double>();
  if ((rc = md_interface_system(md, nrhs, vecs, st))) return rc;
  // 3. final solves with the interface values
  if ((rc = fork())) return rc;
  for (int r = 0; r < nrhs; ++r) {
    vec = vecs + (size_t)r * n;
    q = r * ns;
    for (int k = 0; k < t.nd[2]; ++k)
      for (int j = 0; j < t.nd[1]; ++j)
        for (int i = 0; i < t.nd[0]; ++i) {
          const int s = md_sub_index(md, i, j, k);
          mf_md::Sub& sd = md->sub[s];
          if ((rc = load_bc(s, i, j, k, 1))) return rc;
          const long long tot = (long long)(sd.n[0] - 2) * (sd.n[1] - 2) * (sd.n[2] - 2);
          k_extract_int<<<nblk(tot, 256), 256, 0, sd.stream>>>(g[q + s], sd.rint.as<double>(), sd.n[0] - 2,
                                                                sd.n[1] - 2, sd.n[2] - 2);
          MF_CUDA(cudaGetLastError());
          if ((rc = md_sub_solve(md, s, sd.rint.as<double>(), u[q + s], sd.stream))) return rc;
        }
  }
  return join();
}

int mf_md_solve(mf_md_t* md, const double* const* g, double* const* u, const double* const* bcx,
                const double* const* bcy, const double* const* bcz, void* stream) {
  return md_solve_impl(md, 1, g, u, bcx, bcy, bcz, stream);
}

int mf_md_solve_many(mf_md_t* md, int nrhs, const double* const* g, double* const* u,
                     const double* const* bcx, const double* const* bcy, const double* const* bcz,
                     void* stream) {
  return md_solve_impl(md, nrhs, g, u, bcx, bcy, bcz, stream);
}

int mf_md_set_assembly(mf_md_t* md, int mode) {
  if (!md || (mode != MF_MD_ASSEMBLY_EIGEN && mode != MF_MD_ASSEMBLY_SOLVES))
    return set_error(MF_ERR_ARG, "mf_md_set_assembly: bad arguments");
  md->assembly = mode;
  return MF_OK;
}

int mf_md_interface_solve(mf_md_t* md, int nrhs, const double* rhs, double* sol, void* stream) {
  if (!md || !rhs || !sol || nrhs < 1 || nrhs > kMdMaxRhs)
    return set_error(MF_ERR_ARG, "mf_md_interface_solve: bad arguments");
  if (!md->factored) return set_error(MF_ERR_ARG, "mf_md_interface_solve: influence matrix not set");
  if (!is_device_ptr(rhs) || !is_device_ptr(sol))
    return set_error(MF_ERR_ARG, "mf_md_interface_solve: device pointers only");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t bytes = sizeof(double) * (size_t)md->topo.ninf * nrhs;
  double* vecs = md->vec.as<double>();
  MF_CUDA(cudaMemcpyAsync(vecs, rhs, bytes, cudaMemcpyDeviceToDevice, st));
  int rc = md_interface_system(md, nrhs, vecs, st);
  if (rc) return rc;
  MF_CUDA(cudaMemcpyAsync(sol, vecs, bytes, cudaMemcpyDeviceToDevice, st));
  return MF_OK;
}

int mf_md_set_precision(mf_md_t* md, int precision, int refine) {
  if (!md || (precision != MF_PREC_FP64 && precision != MF_PREC_SPLIT_BF16 && precision != MF_PREC_3XTF32))
    return set_error(MF_ERR_ARG, "mf_md_set_precision: bad arguments");
  md->precision = precision;
  md->refine = refine;
  return MF_OK;
}

int mf_md_set_interface_solve(mf_md_t* md, int mode) {
  if (!md || (mode != MF_MD_IFACE_AUTO && mode != MF_MD_IFACE_LU && mode != MF_MD_IFACE_INVERSE &&
              mode != MF_MD_IFACE_TRIANGULAR_INVERSE && mode != MF_MD_IFACE_TRIANGULAR_INVERSE_FP64))
    return set_error(MF_ERR_ARG, "mf_md_set_interface_solve: bad arguments");
  md->iface_mode = mode;
  return MF_OK;
}

int mf_md_interface_form(const mf_md_t* md, int* form) {
  if (!md || !form) return set_error(MF_ERR_ARG, "mf_md_interface_form: null argument");
  if (!md->factored) return set_error(MF_ERR_ARG, "mf_md_interface_form: influence matrix not set");
  *form = MF_MD_IFACE_LU;
  if (md->iface_mode != MF_MD_IFACE_LU && md->inv_ok) *form = MF_MD_IFACE_INVERSE;
  if (md->iface_mode != MF_MD_IFACE_LU && md->trinv_ok)
    *form = md->trinv_df ? MF_MD_IFACE_TRIANGULAR_INVERSE : MF_MD_IFACE_TRIANGULAR_INVERSE_FP64;
  return MF_OK;
}

int mf_md_set_triangular_form(mf_md_t* md, int form) {
  if (!md || (form != MF_MD_TRI_PERSISTENT && form != MF_MD_TRI_STEPS))
    return set_error(MF_ERR_ARG, "mf_md_set_triangular_form: bad arguments");
  md->tri_form = form;
  return MF_OK;
}

int mf_md_device_status(const mf_md_t* md) {
  if (!md) return set_error(MF_ERR_ARG, "mf_md_device_status: null handle");
  if (!md->perr.ptr) return MF_OK;
  int e = 0;
  MF_CUDA(cudaDeviceSynchronize());
  MF_CUDA(cudaMemcpy(&e, md->perr.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return set_error(MF_ERR_TIMEOUT, "multidomain triangular solve: a block wait expired");
  return MF_OK;
}

int mf_md_interface(const mf_md_t* md, double* lambda) {
  if (!md || !lambda) return set_error(MF_ERR_ARG, "mf_md_interface: null argument");
  MF_CUDA(cudaDeviceSynchronize());
  MF_CUDA(cudaMemcpy(lambda, md->vec.ptr, sizeof(double) * md->topo.ninf, cudaMemcpyDeviceToHost));
  return MF_OK;
}

}  // extern "C"
