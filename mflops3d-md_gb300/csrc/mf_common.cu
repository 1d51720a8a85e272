// Error reporting, pointer classification and device buffers.
#include <cstdio>
#include <cstring>

#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "mf_internal.h"

#include <cmath>
#include "mf_setup.h"

namespace mf {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 152;
    cached[dev] = sms;
  }
  return cached[dev];
}

namespace {
using TuneKey = std::tuple<int, long long, long long, long long, long long>;
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
int g_tune_mode = 0;
}  // namespace

int tune_mode() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune_mode;
}

int tune_lookup(int kind, long long a, long long b, long long c, long long d) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(TuneKey(kind, a, b, c, d));
  return it == g_tune.end() ? -1 : it->second;
}

void tune_store(int kind, long long a, long long b, long long c, long long d, int choice) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[TuneKey(kind, a, b, c, d)] = choice;
}

bool stream_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
    cudaGetLastError();
    return true;  // be safe: no timing when the state is unknown
  }
  return cs != cudaStreamCaptureStatusNone;
}

int cuda_error(cudaError_t e, const char* what) {
  return set_error(e == cudaErrorMemoryAllocation ? MF_ERR_ALLOC : MF_ERR_CUDA,
                   "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
  if (p == nullptr) return false;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

int DevBuf::ensure(size_t nbytes) {
  if (nbytes <= bytes) return MF_OK;
  release();
  cudaError_t e = cudaMalloc(&ptr, nbytes);
  if (e != cudaSuccess) {
    ptr = nullptr;
    bytes = 0;
    return cuda_error(e, "cudaMalloc");
  }
  bytes = nbytes;
  return MF_OK;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

int stage_in(DevBuf& buf, const void* host, size_t bytes, cudaStream_t s) {
  int rc = buf.ensure(bytes);
  if (rc) return rc;
  MF_CUDA(cudaMemcpyAsync(buf.ptr, host, bytes, cudaMemcpyHostToDevice, s));
  return MF_OK;
}

void StageProfiler::begin(int kind, cudaStream_t st, int count) {
  if (!on) return;
  Rec r{kind, nullptr, nullptr, count};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, st);
  pending.push_back(r);
}

void StageProfiler::end(cudaStream_t st) {
  if (!on || pending.empty()) return;
  cudaEventRecord(pending.back().b, st);
}

void StageProfiler::collect() {
  for (Rec& r : pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      total_ms[r.kind] += ms;
      launches[r.kind] += r.count;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  pending.clear();
  cudaGetLastError();
}

void StageProfiler::reset() {
  collect();
  for (int k = 0; k < kKinds; ++k) {
    total_ms[k] = 0.0;
    launches[k] = 0;
  }
}

}  // namespace mf

using namespace mf;

extern "C" {

const char* mf_last_error(void) { return g_last_error.c_str(); }

int mf_version(void) { return 1; }

int mf_device_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

int mf_der_coeffs_generic(const double h0[7], int cl, int der, int so, double coef_imp[5],
                          double coef_exp[7]) {
  if (cl < 1 || cl > 3 || (der != 1 && der != 2) || (so != 2 && so != 4 && so != 6 && so != 8))
    return set_error(MF_ERR_ARG, "mf_der_coeffs_generic: bad cl/der/so (%d,%d,%d)", cl, der, so);
  if (!der_coeffs_generic(h0, cl, der, so, coef_imp, coef_exp))
    return set_error(MF_ERR_SINGULAR, "mf_der_coeffs_generic: singular Taylor system");
  return MF_OK;
}

int mf_der_line_coeffs(const double* grid, int n, int der, int so, double* dl, double* dr) {
  if (n < 7 || !grid || !dl || !dr || (der != 1 && der != 2) ||
      (so != 2 && so != 4 && so != 6 && so != 8))
    return set_error(MF_ERR_ARG, "mf_der_line_coeffs: bad arguments (n=%d der=%d so=%d)", n, der, so);
  std::vector<double> l(5 * n), r(7 * n);
  if (!der_line_coeffs(grid, n, der, so, l.data(), r.data()))
    return set_error(MF_ERR_SINGULAR, "mf_der_line_coeffs: singular Taylor system");
  for (int i = 0; i < n; ++i) {
    for (int m = 0; m < 5; ++m) dl[i + n * m] = l[5 * i + m];
    for (int m = 0; m < 7; ++m) dr[i + n * m] = r[7 * i + m];
  }
  return MF_OK;
}

int mf_pentalu(int n, double* dl) {
  if (n < 7 || !dl) return set_error(MF_ERR_ARG, "mf_pentalu: n must be >= 7");
  std::vector<double> l(5 * n);
  for (int i = 0; i < n; ++i)
    for (int m = 0; m < 5; ++m) l[5 * i + m] = dl[i + n * m];
  pentalu(n, l.data());
  for (int i = 0; i < n; ++i)
    for (int m = 0; m < 5; ++m) dl[i + n * m] = l[5 * i + m];
  return MF_OK;
}

int mf_grid1d(int kind, int n, double xa, double xb, double param, double* grid) {
  if (n < 2 || !grid || !(xb > xa) || kind < MF_GRID_UNIFORM || kind > MF_GRID_TANH)
    return set_error(MF_ERR_ARG, "mf_grid1d: bad arguments (kind=%d n=%d [%g,%g])", kind, n, xa, xb);
  const double pas = (xb - xa) / double(n - 1);
  const double pi = 4.0 * std::atan(1.0);
  if (kind == MF_GRID_ARCSIN) {
    const double alpha = 1.0 - param / double(n * n);
    if (!(std::fabs(alpha) < 1.0) || alpha == 0.0)
      return set_error(MF_ERR_ARG, "mf_grid1d: arcsin parameter beta=%g gives alpha=%g outside (0,1)", param, alpha);
    const double asa = std::asin(alpha);
    for (int i = 0; i < n; ++i) {
      const double xi = xa + double(i) * pas;
      grid[i] = xa + (xb - xa) * (std::asin(-alpha * std::cos(pi * (xi - xa) / (xb - xa))) / asa + 1.0) * 0.5;
    }
  } else if (kind == MF_GRID_TANH && param != 0.0) {
    const double ta = std::tanh(param);
    for (int i = 0; i < n; ++i) {
      const double xi = xa + double(i) * pas;
      grid[i] = xa + (xb - xa) * (1.0 + std::tanh(param * (2.0 * (xi - xa) / (xb - xa) - 1.0)) / ta) / 2.0;
    }
  } else {
    for (int i = 0; i < n; ++i) grid[i] = xa + double(i) * pas;
  }
  return MF_OK;
}

int mf_grid_spacing(int n, const double* grid, double* dgrid) {
  if (n < 2 || !grid || !dgrid) return set_error(MF_ERR_ARG, "mf_grid_spacing: n must be >= 2");
  dgrid[0] = grid[1] - grid[0];
  dgrid[n - 1] = grid[n - 1] - grid[n - 2];
  for (int i = 1; i < n - 1; ++i) dgrid[i] = (grid[i + 1] - grid[i - 1]) * 0.5;
  return MF_OK;
}

int mf_mesh_grid_init(char choice, int n, int dom_coord, int ndomains, int kind, double param,
                      double* grid1d, double* dgrid1d) {
  if (choice != 'x' && choice != 'y' && choice != 'z')
    return set_error(MF_ERR_ARG, "mf_mesh_grid_init: choice must be 'x', 'y' or 'z'");
  if (ndomains < 1 || dom_coord < 0 || dom_coord >= ndomains)
    return set_error(MF_ERR_ARG, "mf_mesh_grid_init: subdomain %d of %d", dom_coord, ndomains);
  const double aux = 0.5;
  double xa = -aux, xb = aux;
  if (choice == 'z') { xa = -aux * 0.5; xb = aux * 0.5; }
  if (ndomains > 1) {
    const double size_dom = (xb - xa) / double(ndomains);
    xa = xa + double(dom_coord) * size_dom;
    xb = xa + size_dom;
  }
  int rc = mf_grid1d(kind, n, xa, xb, param, grid1d);
  if (rc) return rc;
  return dgrid1d ? mf_grid_spacing(n, grid1d, dgrid1d) : MF_OK;
}

int mf_solver_axis_setup(const double* grid, int nall, const int bct[2], int so, double* ddl,
                         double* ddr, double* inv_lhs, double* eigen, double* vect,
                         double* inv_vect, double* neum) {
  if (!grid || !bct) return set_error(MF_ERR_ARG, "mf_solver_axis_setup: null grid/bct");
  SolverAxisHost ax;
  std::string msg;
  int rc = solver_axis_setup(grid, nall, bct, so, ax, msg);
  if (rc) return set_error(rc, "mf_solver_axis_setup: %s", msg.c_str());
  const int n = ax.n;
  if (ddl)
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < 5; ++m) ddl[i + n * m] = ax.ddl[5 * i + m];
  if (ddr)
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < 8; ++m) ddr[i + n * m] = ax.ddr[8 * i + m];
  auto colmajor = [&](const std::vector<double>& src, double* dst) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) dst[i + (size_t)n * j] = src[(size_t)i * n + j];
  };
  if (inv_lhs) colmajor(ax.inv_lhs, inv_lhs);
  if (eigen)
    for (int i = 0; i < n; ++i) eigen[i] = ax.eigen[i];
  if (vect) colmajor(ax.vect, vect);
  if (inv_vect) colmajor(ax.inv_vect, inv_vect);
  if (neum)
    for (int s = 0; s < 2; ++s)
      for (int m = 0; m < 7; ++m) neum[s + 2 * m] = ax.neum[7 * s + m];
  return MF_OK;
}

int mf_tune_set(int mode) {
  if (mode != 0 && mode != 1) return set_error(MF_ERR_ARG, "mf_tune_set: mode must be 0 or 1");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_mode = mode;
  return MF_OK;
}

int mf_tune_get(void) { return tune_mode(); }

int mf_tune_entries(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return (int)g_tune.size();
}

int mf_tune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return MF_OK;
}

int mf_tune_save(const char* path) {
  if (!path) return set_error(MF_ERR_ARG, "mf_tune_save: null path");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  FILE* f = std::fopen(path, "w");
  if (!f) return set_error(MF_ERR_ARG, "mf_tune_save: cannot open %s", path);
  std::fprintf(f, "# mflops_gb300 launch-shape decisions: kind a b c d choice\n");
  for (const auto& kv : g_tune)
    std::fprintf(f, "%d %lld %lld %lld %lld %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
                 std::get<2>(kv.first), std::get<3>(kv.first), std::get<4>(kv.first), kv.second);
  std::fclose(f);
  return MF_OK;
}

int mf_tune_load(const char* path) {
  if (!path) return set_error(MF_ERR_ARG, "mf_tune_load: null path");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_error(MF_ERR_ARG, "mf_tune_load: cannot open %s", path);
  char line[256];
  int n = 0;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    int kind, choice;
    long long a, b, c, d;
    if (std::sscanf(line, "%d %lld %lld %lld %lld %d", &kind, &a, &b, &c, &d, &choice) == 6) {
      g_tune[TuneKey(kind, a, b, c, d)] = choice;
      ++n;
    }
  }
  std::fclose(f);
  return MF_OK;
}

}  // extern "C"
