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

// Growable device buffer owned by a handle.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t nbytes);
  void release();
  template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// Copies host -> device buffer (growing it) on stream; returns MF_OK or error.
int stage_in(DevBuf& buf, const void* host, size_t bytes, cudaStream_t s);

// Optional per-kernel CUDA-event timers of a handle.  When enabled, every
// launch of the handle is bracketed by an event pair on its stream; read()
// synchronises on the recorded events and accumulates per-kind totals.
struct StageProfiler {
  static constexpr int kKinds = 12;
  bool on = false;
  struct Rec {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  double total_ms[kKinds] = {0};
  long long launches[kKinds] = {0};
  void begin(int kind, cudaStream_t st);
  void end(cudaStream_t st);
  void collect();
  void reset();
};

}  // namespace mf
