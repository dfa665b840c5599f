// handles.h -- the library's handle types and error helpers (internal).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fields.h"

struct mr_bathymetry {
  mr::BathyDev dev{};
  int device = 0;
  bool one_point_axis = false;  // the reference panics on its first lookup
  std::vector<void *> mem;      // device allocations owned by the handle
};

struct mr_current {
  mr::CurrentDev dev{};
  int device = 0;
  bool one_point_axis = false;
  std::vector<void *> mem;
};

namespace mr {

extern thread_local std::string g_last_error;

// Records a formatted message for mr_last_error() and returns `code`.
int fail(int code, const char *fmt, ...);
// MR_ERR_CUDA / MR_ERR_OUT_OF_MEMORY with the CUDA error's name.
int cuda_fail(cudaError_t e, const char *what);

// Makes `device` current for the lifetime of the guard.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    ok_ = cudaGetDevice(&prev_) == cudaSuccess;
    if (ok_ && prev_ != device) ok_ = cudaSetDevice(device) == cudaSuccess;
    switched_ = ok_ && prev_ != device;
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  bool ok() const { return ok_; }

 private:
  int prev_ = 0;
  bool ok_ = false;
  bool switched_ = false;
};

}  // namespace mr

#define MR_CUDA(call)                                           \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return mr::cuda_fail(e_, #call);     \
  } while (0)
