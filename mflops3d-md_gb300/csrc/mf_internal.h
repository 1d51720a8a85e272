// Internal helpers shared by the translation units of libmflops_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "mflops_gb300.h"

namespace mf {

// Records a thread-local error message and returns `code`.
int set_error(int code, const char* fmt, ...);
// Turns a CUDA error into MF_ERR_CUDA with the call site in the message.
int cuda_error(cudaError_t e, const char* what);

#define MF_CUDA(call)                                         \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::mf::cuda_error(e_, #call); \
  } while (0)

// True when p points to device (or managed) memory.
bool is_device_ptr(const void* p);

// SM count of the current device (152 on GB300), cached per device.
int num_sms();

// Launch-shape autotuner (mf_tune_*).  Decisions are keyed by a kind and four
// shape numbers; mode 0 uses the built-in heuristics, mode 1 times the
// candidates on first use of a shape (CUDA events on the caller's stream,
// never while the stream is being captured) and keeps the fastest.
enum TuneKind { kTuneGemm64 = 0, kTuneDerX = 1, kTuneTcTf32 = 2 };
int tune_mode();
int tune_lookup(int kind, long long a, long long b, long long c, long long d);
void tune_store(int kind, long long a, long long b, long long c, long long d, int choice);
bool stream_capturing(cudaStream_t st);
// Times run(c) for c = 0..n-1 (one warm-up and three timed runs each) and
// returns the fastest choice, or -1 when timing failed.
template <class Run>
int tune_measure(cudaStream_t st, int n, Run run) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1;
  }
  int best = -1;
  float best_ms = 0.f;
  for (int c = 0; c < n; ++c) {
    if (run(c)) continue;
    cudaEventRecord(e0, st);
    bool ok = true;
    for (int r = 0; r < 3 && ok; ++r) ok = run(c) == 0;
    cudaEventRecord(e1, st);
    float ms = 0.f;
    if (!ok || cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      continue;
    if (best < 0 || ms < best_ms) {
      best = c;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

// Growable device buffer owned by a handle.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t nbytes);
  void release();
  template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// Read-only view of one axis of a solver's set-up (device arrays): n
// interior points, eigenvectors V (row-major n x n, V[i n + p]) and their
// inverse, eigenvalues, the four fold columns of inv_lhs (invl4[c n + i],
// c = 0..3 for the columns 1, 2, n-1, n) with their ddr factors bcc, the
// boundary types of the two ends and the Neumann extrapolation weights
// (neum[0..6] left, neum[7..13] right).
struct SolverAxisView {
  int n;
  const double *V, *Vinv, *eig, *invl4;
  double bcc[4];
  int bc[2];
  double neum[14];
};
int solver_axis_view(const ::mf_solver3d* sc, int axis, SolverAxisView* out);

// Copies host -> device buffer (growing it) on stream; returns MF_OK or error.
int stage_in(DevBuf& buf, const void* host, size_t bytes, cudaStream_t s);

// Waits on a stream when it goes out of scope armed: an entry point that
// has queued copies from or to the caller's host arrays returns, on an
// error too, only after they are done.
struct HostCopyWait {
  cudaStream_t st;
  bool armed = false;
  explicit HostCopyWait(cudaStream_t s) : st(s) {}
  ~HostCopyWait() {
    if (armed) cudaStreamSynchronize(st);
  }
};

// Optional per-kernel CUDA-event timers of a handle.  When enabled, every
// launch of the handle (or a short group of launches of one stage, whose
// count begin() is given) is bracketed by an event pair on its stream;
// collect() synchronises on the recorded events and accumulates per-kind
// totals of time and launches.
struct StageProfiler {
  static constexpr int kKinds = 12;
  bool on = false;
  struct Rec {
    int kind;
    cudaEvent_t a, b;
    int count;  // kernel launches between a and b
  };
  std::vector<Rec> pending;
  double total_ms[kKinds] = {0};
  long long launches[kKinds] = {0};
  void begin(int kind, cudaStream_t st, int count = 1);
  void end(cudaStream_t st);
  void collect();
  void reset();
};

}  // namespace mf
