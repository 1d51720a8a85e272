// Compact finite-difference derivatives on GB300: batched quasi-pentadiagonal
// line solves over the pencils of an (nx,ny,nz) FP64 field.
//
// Reference path: class_field.f90:629-978 (pencil drivers) ->
// class_derivatives.f90:186-260 (der/dder/der_s/dder_s) -> derx_rhs (:262-295)
// + pentares (:425-466) with coefficients from der_coeffs_init (:111-184).
//
// Kernels
//  * der_lines_strided: one thread per pencil for the y and z axes; a warp
//    covers 32 consecutive x indices, so every step of the recurrence is a
//    coalesced 256-byte access.  The forward-elimination values are parked
//    in the output array and re-read by the back substitution.
//  * der_lines_contig: x axis.  A warp stages 32 pencils in shared memory
//    with coalesced loads, solves them in place (thread per pencil, odd row
//    pitch so the per-thread walks are bank-conflict free), and writes them
//    back coalesced.
// On GB300 the FP64 pipe (~1.2 TFLOP/s measured) rather than HBM bounds
// these kernels: ~10 DFMA per point and pass against 16 bytes of traffic,
// ~7 with the tridiagonal row tables used for schemes of order <= 6.
#include <algorithm>
#include <cstring>

#include "mf_internal.h"
#include "mf_line.cuh"
#include "mf_setup.h"

namespace mf {

// Line kind for solver-type coefficients (class_field.f90:648-671).
__device__ __forceinline__ int line_kind(int mode, int a, int na, int b, int nb) {
  if (mode == 1) return 0;  // all plain
  if (mode == 2) return 1;  // all _s
  if (mode == 0) return 0;  // field, plain coefficients
  const bool ea = (a == 0 || a == na - 1), eb = (b == 0 || b == nb - 1);
  if (ea && eb) return 2;   // edge line: left at zero
  return (ea || eb) ? 1 : 0;
}

// Row tables of the tridiagonal fast path (null when the scheme is not
// tridiagonal): plain lines and der_s / dder_s lines.
struct TriSets {
  const DerTriRow* plain;
  const DerTriRow* sub;
};

__device__ __forceinline__ void process_line(int kind, LineSet plain, LineSet sub, TriSets tri,
                                             const double* in, double* out, long long s) {
  if (kind == 0) {
    if (tri.plain)
      solve_line_tri_d(tri.plain, plain.n, in, out, s);
    else
      solve_line(plain.c, plain.n, in, out, s, LineBC(), StorePlain());
  } else if (kind == 1) {
    const int n = plain.n;
    if (tri.sub)
      solve_line_tri_d(tri.sub, sub.n, in + s, out + s, s);
    else
      solve_line(sub.c, sub.n, in + s, out + s, s, LineBC(), StorePlain());
    out[0] = 0.0;
    out[(long long)(n - 1) * s] = 0.0;
  } else {
    for (int i = 0; i < plain.n; ++i) out[(long long)i * s] = 0.0;
  }
}

// y (stride nx) or z (stride nx*ny) pencils; thread t -> (a = t % na, b = t / na).
__global__ void der_lines_strided(LineSet plain, LineSet sub, TriSets tri, int mode, const double* f,
                                  double* df, int na, int nb, long long sa,
                                  long long sb, long long s) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int a = (int)(t % na), b = (int)(t / na);
  const long long base = a * sa + b * sb;
  process_line(line_kind(mode, a, na, b, nb), plain, sub, tri, f + base, df + base, s);
}

// x pencils: 32 per warp, staged through shared memory.
constexpr int kLinesPerBlock = 32;
__global__ void __launch_bounds__(32) der_lines_contig(LineSet plain, LineSet sub, TriSets tri, int mode,
                                                       const double* __restrict__ f,
                                                       double* __restrict__ df, int n, int na,
                                                       int nb, int pitch) {
  extern __shared__ double tile[];
  const int lane = threadIdx.x;
  const long long nlines = (long long)na * nb;
  const long long l0 = (long long)blockIdx.x * kLinesPerBlock;
  const int nl = (int)min((long long)kLinesPerBlock, nlines - l0);
  for (int l = 0; l < nl; ++l) {
    const double* src = f + (l0 + l) * n;
    for (int i = lane; i < n; i += 32) tile[l * pitch + i] = src[i];
  }
  __syncwarp();
  if (lane < nl) {
    const long long line = l0 + lane;
    const int a = (int)(line % na), b = (int)(line / na);
    double* row = tile + lane * pitch;
    process_line(line_kind(mode, a, na, b, nb), plain, sub, tri, row, row, 1);
  }
  __syncwarp();
  for (int l = 0; l < nl; ++l) {
    double* dst = df + (l0 + l) * n;
    for (int i = lane; i < n; i += 32) dst[i] = tile[l * pitch + i];
  }
}

}  // namespace mf

using namespace mf;

struct mf_der {
  int n = 0, so = 6, solver = 0;
  double* dev = nullptr;  // packed sets: der(n), dder(n), der_s(n-2), dder_s(n-2)
  size_t off[4] = {0, 0, 0, 0};
  DevBuf tri;             // DerTriRow tables of the same sets (tridiagonal schemes)
  size_t tri_off[4] = {0, 0, 0, 0};
  bool tri_ok = false;
  DevBuf stage_in_buf, stage_out_buf;
};

// DerTriRow table of one set from its packed rows p, f, 1/c, d, e, r0..r6;
// false when the factored implicit part is not tridiagonal.
static bool tri_rows(const std::vector<double>& rows, int n, std::vector<DerTriRow>& out) {
  for (int i = 0; i < n; ++i)
    if (rows[(size_t)kRow * i + 0] != 0.0 || rows[(size_t)kRow * i + 4] != 0.0) return false;
  out.resize(n);
  for (int i = 0; i < n; ++i) {
    const double* r = &rows[(size_t)kRow * i];
    const double inv_c = r[2];
    DerTriRow& t = out[i];
    for (int m = 0; m < 7; ++m) t.w[m] = r[5 + m] * inv_c;
    t.ft = i > 0 ? r[1] * inv_c / rows[(size_t)kRow * (i - 1) + 2] : 0.0;
    t.dt = i < n - 1 ? r[3] * inv_c : 0.0;
  }
  return true;
}

static void pack_rows(const std::vector<double>& dl_lu, const std::vector<double>& dr, int n,
                      std::vector<double>& out) {
  for (int i = 0; i < n; ++i) {
    double* r = &out[(size_t)kRow * i];
    r[0] = dl_lu[5 * i + 0];
    r[1] = dl_lu[5 * i + 1];
    r[2] = 1.0 / dl_lu[5 * i + 2];
    r[3] = dl_lu[5 * i + 3];
    r[4] = dl_lu[5 * i + 4];
    for (int m = 0; m < 7; ++m) r[5 + m] = dr[7 * i + m];
  }
}

extern "C" {

int mf_der_coeffs_init(const double* grid, int n, int solver_type, int so, mf_der_t** out) {
  if (!grid || !out) return set_error(MF_ERR_ARG, "mf_der_coeffs_init: null argument");
  *out = nullptr;
  if (so != 2 && so != 4 && so != 6 && so != 8)
    return set_error(MF_ERR_ARG, "mf_der_coeffs_init: so must be 2, 4, 6 or 8");
  if (n < 7 || (solver_type && n < 9))
    return set_error(MF_ERR_ARG, "mf_der_coeffs_init: n=%d too small (needs >= 7, 9 with solver type)", n);
  const int nsets = solver_type ? 4 : 2;
  std::vector<double> packed;
  size_t off[4] = {0, 0, 0, 0};
  std::vector<DerTriRow> tri_all;
  size_t tri_off[4] = {0, 0, 0, 0};
  bool tri_ok = true;
  for (int set = 0; set < nsets; ++set) {
    const int der = (set % 2) + 1;
    const bool sub = set >= 2;
    const int m = sub ? n - 2 : n;
    std::vector<double> dl(5 * m), dr(7 * m);
    if (!der_line_coeffs(grid + (sub ? 1 : 0), m, der, so, dl.data(), dr.data()))
      return set_error(MF_ERR_SINGULAR, "mf_der_coeffs_init: singular Taylor system");
    pentalu(m, dl.data());
    off[set] = packed.size();
    packed.resize(packed.size() + (size_t)kRow * m);
    std::vector<double> rows((size_t)kRow * m);
    pack_rows(dl, dr, m, rows);
    std::copy(rows.begin(), rows.end(), packed.begin() + off[set]);
    std::vector<DerTriRow> tr;
    if (tri_ok && tri_rows(rows, m, tr)) {
      tri_off[set] = tri_all.size();
      tri_all.insert(tri_all.end(), tr.begin(), tr.end());
    } else {
      tri_ok = false;
    }
  }
  mf_der* dc = new mf_der();
  dc->n = n;
  dc->so = so;
  dc->solver = solver_type ? 1 : 0;
  for (int s = 0; s < 4; ++s) {
    dc->off[s] = off[s];
    dc->tri_off[s] = tri_off[s];
  }
  if (tri_ok) {
    int rc = dc->tri.ensure(tri_all.size() * sizeof(DerTriRow));
    if (!rc && cudaMemcpy(dc->tri.ptr, tri_all.data(), tri_all.size() * sizeof(DerTriRow),
                          cudaMemcpyHostToDevice) != cudaSuccess)
      rc = set_error(MF_ERR_CUDA, "mf_der_coeffs_init: upload of the row tables failed");
    if (rc) {
      dc->tri.release();
      delete dc;
      return rc;
    }
    dc->tri_ok = true;
  }
  cudaError_t e = cudaMalloc(&dc->dev, packed.size() * sizeof(double));
  if (e != cudaSuccess) {
    delete dc;
    return cuda_error(e, "cudaMalloc(derivative coefficients)");
  }
  e = cudaMemcpy(dc->dev, packed.data(), packed.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dc->dev);
    delete dc;
    return cuda_error(e, "cudaMemcpy(derivative coefficients)");
  }
  // the uploads complete before the handle is used on any stream
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
    mf_der_destroy(dc);
    return cuda_error(e, "cudaDeviceSynchronize(derivative coefficients)");
  }
  *out = dc;
  return MF_OK;
}

int mf_der_destroy(mf_der_t* dc) {
  if (!dc) return MF_OK;
  if (dc->dev) cudaFree(dc->dev);
  dc->stage_in_buf.release();
  dc->stage_out_buf.release();
  dc->tri.release();
  delete dc;
  return MF_OK;
}

int mf_dertype(const mf_der_t* dc, int* solver_type) {
  if (!dc || !solver_type) return set_error(MF_ERR_ARG, "mf_dertype: null argument");
  *solver_type = dc->solver;
  return MF_OK;
}

}  // extern "C"

namespace mf {

// Launches the pencil solves of one axis on device arrays.
int der_launch(const mf_der_t* dc, int axis, int order, int mode, const double* f, double* df,
               int nx, int ny, int nz, cudaStream_t st) {
  const int set = order - 1;
  LineSet plain{dc->dev + dc->off[set], dc->n};
  LineSet sub{dc->solver ? dc->dev + dc->off[set + 2] : dc->dev + dc->off[set], dc->n - 2};
  TriSets tri{nullptr, nullptr};
  if (dc->tri_ok) {
    const DerTriRow* t = dc->tri.as<DerTriRow>();
    tri.plain = t + dc->tri_off[set];
    tri.sub = dc->solver ? t + dc->tri_off[set + 2] : nullptr;
  }
  if (axis == 0) {
    const int na = ny, nb = nz;
    const int pitch = nx | 1;
    const size_t smem = (size_t)kLinesPerBlock * pitch * sizeof(double);
    const long long nlines = (long long)na * nb;
    // Staging 32 lines per one-warp block pays while the tile is small (up to
    // 48 KB, nx <= 191); for long lines it leaves too few warps per SM and the
    // thread-per-line walk (lines cached in L1 as each thread consumes them)
    // is faster.
    auto run = [&](int staged) -> int {
      if (staged) {
        static bool attr_set = false;
        if (!attr_set) {
          if (cudaFuncSetAttribute(der_lines_contig, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
              cudaSuccess)
            return 1;
          attr_set = true;
        }
        const unsigned grid = (unsigned)((nlines + kLinesPerBlock - 1) / kLinesPerBlock);
        der_lines_contig<<<grid, 32, smem, st>>>(plain, sub, tri, mode, f, df, nx, na, nb, pitch);
      } else {
        const unsigned grid = (unsigned)((nlines + 127) / 128);
        der_lines_strided<<<grid, 128, 0, st>>>(plain, sub, tri, mode, f, df, na, nb, (long long)nx,
                                                (long long)nx * ny, 1);
      }
      return cudaGetLastError() == cudaSuccess ? 0 : 1;
    };
    // measured on GB300: staged is faster at nx = 129 (33 KB tile, 0.064 vs
    // 0.080 ms per sweep of 129^3) and slower at nx = 257 (66 KB tile)
    int staged = smem <= 48 * 1024 ? 1 : 0;
    // measured choice (autotuner): only when the staged tile fits and the
    // call is not in place (a timed repeat must read the same input)
    if (tune_mode() == 1 && smem <= 200 * 1024) {
      int c = tune_lookup(kTuneDerX, nx, nlines, order, 0);
      if (c < 0 && f != df && !stream_capturing(st)) {
        c = tune_measure(st, 2, run);
        if (c >= 0) tune_store(kTuneDerX, nx, nlines, order, 0, c);
      }
      if (c >= 0) staged = c;
    }
    if (run(staged)) return set_error(MF_ERR_CUDA, "derivative x-line launch failed");
  } else if (axis == 1) {
    const int na = nx, nb = nz;
    const unsigned grid = (unsigned)(((long long)na * nb + 127) / 128);
    der_lines_strided<<<grid, 128, 0, st>>>(plain, sub, tri, mode, f, df, na, nb, 1,
                                            (long long)nx * ny, (long long)nx);
  } else {
    const int na = nx, nb = ny;
    const unsigned grid = (unsigned)(((long long)na * nb + 127) / 128);
    der_lines_strided<<<grid, 128, 0, st>>>(plain, sub, tri, mode, f, df, na, nb, 1, (long long)nx,
                                            (long long)nx * ny);
  }
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

// Several sweeps in one launch: up to kMaxDerJobs (field, axis) jobs of one
// field shape, one thread per line, every job's lines starting on a warp
// boundary so that no warp mixes jobs.  Small fields give a single sweep too
// few lines to fill the GPU (128 x 129 x 128: 16,512 lines, 3.4 warps per
// SM); the jobs of independent sweeps together do.
constexpr int kMaxDerJobs = 9;
struct DerJob {
  LineSet plain, sub;
  TriSets tri;
  const double* f;
  double* df;
  int na, nb, mode;
  long long sa, sb, s;
};
struct DerJobs {
  DerJob j[kMaxDerJobs];
  long long start[kMaxDerJobs + 1];
  int count;
};

__global__ void __launch_bounds__(128) der_lines_multi(DerJobs J) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= J.start[J.count]) return;
  int q = 0;
  while (q + 1 < J.count && t >= J.start[q + 1]) ++q;
  const DerJob& d = J.j[q];
  const long long u = t - J.start[q];
  if (u >= (long long)d.na * d.nb) return;
  const int a = (int)(u % d.na), b = (int)(u / d.na);
  const long long base = a * d.sa + b * d.sb;
  process_line(line_kind(d.mode, a, d.na, b, d.nb), d.plain, d.sub, d.tri, d.f + base, d.df + base, d.s);
}

}  // namespace mf

extern "C" {

int mf_der_apply_many(int count, const mf_der_t* const* dc, const int* axis, const int* order,
                      const double* const* f, double* const* df, int nx, int ny, int nz, void* stream) {
  if (count < 1 || count > kMaxDerJobs || !dc || !axis || !order || !f || !df)
    return set_error(MF_ERR_ARG, "mf_der_apply_many: 1..%d jobs with non-null arrays", kMaxDerJobs);
  if (nx < 2 || ny < 2 || nz < 2) return set_error(MF_ERR_ARG, "mf_der_apply_many: field too small");
  DerJobs J{};
  J.count = count;
  J.start[0] = 0;
  for (int q = 0; q < count; ++q) {
    const mf_der_t* d = dc[q];
    const int ax = axis[q], ord = order[q];
    if (!d || !f[q] || !df[q] || ax < 0 || ax > 2 || (ord != 1 && ord != 2))
      return set_error(MF_ERR_ARG, "mf_der_apply_many: bad job %d", q);
    const int nline = ax == 0 ? nx : ax == 1 ? ny : nz;
    if (nline != d->n)
      return set_error(MF_ERR_ARG, "mf_der_apply_many: job %d pencil length %d differs from n=%d", q, nline, d->n);
    if (!is_device_ptr(f[q]) || !is_device_ptr(df[q]))
      return set_error(MF_ERR_ARG, "mf_der_apply_many: device fields required");
    const int set = ord - 1;
    DerJob& j = J.j[q];
    j.plain = LineSet{d->dev + d->off[set], d->n};
    j.sub = LineSet{d->solver ? d->dev + d->off[set + 2] : d->dev + d->off[set], d->n - 2};
    j.tri = TriSets{nullptr, nullptr};
    if (d->tri_ok) {
      const DerTriRow* t = d->tri.as<DerTriRow>();
      j.tri.plain = t + d->tri_off[set];
      j.tri.sub = d->solver ? t + d->tri_off[set + 2] : nullptr;
    }
    j.f = f[q];
    j.df = df[q];
    j.mode = d->solver ? 3 : 0;
    if (ax == 0) {
      j.na = ny; j.nb = nz; j.sa = nx; j.sb = (long long)nx * ny; j.s = 1;
    } else if (ax == 1) {
      j.na = nx; j.nb = nz; j.sa = 1; j.sb = (long long)nx * ny; j.s = nx;
    } else {
      j.na = nx; j.nb = ny; j.sa = 1; j.sb = nx; j.s = (long long)nx * ny;
    }
    const long long lines = (long long)j.na * j.nb;
    J.start[q + 1] = J.start[q] + (lines + 31) / 32 * 32;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned grid = (unsigned)((J.start[count] + 127) / 128);
  der_lines_multi<<<grid, 128, 0, st>>>(J);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}


int mf_der_apply(const mf_der_t* dc_c, int axis, int order, const double* f, double* df, int nx,
                 int ny, int nz, void* stream) {
  mf_der_t* dc = const_cast<mf_der_t*>(dc_c);
  if (!dc || !f || !df) return set_error(MF_ERR_ARG, "mf_der_apply: null argument");
  if (axis < 0 || axis > 2 || (order != 1 && order != 2))
    return set_error(MF_ERR_ARG, "mf_der_apply: axis must be 0..2 and order 1 or 2");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(MF_ERR_ARG, "mf_der_apply: empty field");
  const int nline = axis == 0 ? nx : axis == 1 ? ny : nz;
  if (nline != dc->n)
    return set_error(MF_ERR_ARG, "mf_der_apply: pencil length %d differs from coefficients n=%d",
                     nline, dc->n);
  if (dc->solver && ((axis != 0 && nx < 2) || (axis != 1 && ny < 2) || (axis != 2 && nz < 2)))
    return set_error(MF_ERR_ARG, "mf_der_apply: solver-type derivative needs >= 2 points on the other axes");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int mode = dc->solver ? 3 : 0;
  const size_t bytes = (size_t)nx * ny * nz * sizeof(double);
  const bool dev_in = is_device_ptr(f), dev_out = is_device_ptr(df);
  if (dev_in && dev_out) return der_launch(dc, axis, order, mode, f, df, nx, ny, nz, st);
  // host pointers: stage through the handle's buffers
  const double* fin = f;
  int rc;
  HostCopyWait wait(st);
  wait.armed = true;
  if (!dev_in) {
    if ((rc = stage_in(dc->stage_in_buf, f, bytes, st))) return rc;
    fin = dc->stage_in_buf.as<double>();
  }
  double* dout = df;
  if (!dev_out) {
    if ((rc = dc->stage_out_buf.ensure(bytes))) return rc;
    dout = dc->stage_out_buf.as<double>();
  }
  if ((rc = der_launch(dc, axis, order, mode, fin, dout, nx, ny, nz, st))) return rc;
  if (!dev_out) MF_CUDA(cudaMemcpyAsync(df, dout, bytes, cudaMemcpyDeviceToHost, st));
  MF_CUDA(cudaStreamSynchronize(st));
  return MF_OK;
}

int mf_derx(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 0, 1, f, df, nx, ny, nz, s);
}
int mf_dery(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 1, 1, f, df, nx, ny, nz, s);
}
int mf_derz(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 2, 1, f, df, nx, ny, nz, s);
}
int mf_dderx(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 0, 2, f, df, nx, ny, nz, s);
}
int mf_ddery(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 1, 2, f, df, nx, ny, nz, s);
}
int mf_dderz(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* s) {
  return mf_der_apply(dc, 2, 2, f, df, nx, ny, nz, s);
}

int mf_der_lines(const mf_der_t* dc_c, int order, int solver_variant, const double* x, double* dx,
                 int count, void* stream) {
  mf_der_t* dc = const_cast<mf_der_t*>(dc_c);
  if (!dc || !x || !dx || count < 1 || (order != 1 && order != 2))
    return set_error(MF_ERR_ARG, "mf_der_lines: bad arguments");
  if (solver_variant && !dc->solver)
    return set_error(MF_ERR_ARG, "mf_der_lines: der_s/dder_s need solver-type coefficients");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = dc->n;
  const size_t bytes = (size_t)n * count * sizeof(double);
  const bool dev_in = is_device_ptr(x), dev_out = is_device_ptr(dx);
  const double* fin = x;
  double* dout = dx;
  int rc;
  HostCopyWait wait(st);
  wait.armed = !dev_in || !dev_out;
  if (!dev_in) {
    if ((rc = stage_in(dc->stage_in_buf, x, bytes, st))) return rc;
    fin = dc->stage_in_buf.as<double>();
  }
  if (!dev_out) {
    if ((rc = dc->stage_out_buf.ensure(bytes))) return rc;
    dout = dc->stage_out_buf.as<double>();
  }
  if ((rc = der_launch(dc, 0, order, solver_variant ? 2 : 1, fin, dout, n, count, 1, st))) return rc;
  if (!dev_out) {
    MF_CUDA(cudaMemcpyAsync(dx, dout, bytes, cudaMemcpyDeviceToHost, st));
  }
  if (!dev_out || !dev_in) MF_CUDA(cudaStreamSynchronize(st));
  return MF_OK;
}

}  // extern "C"
