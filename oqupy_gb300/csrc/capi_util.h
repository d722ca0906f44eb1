// Small host helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <utility>

#include "../../include/oqupy_gb300.h"

namespace otb {

otb_status set_error(otb_status code, const std::string& msg);
bool check_cuda(cudaError_t e, const char* what);

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  bool alloc(size_t b) {
    release();
    if (b == 0) b = 16;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(OTB_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
      cudaGetLastError();
      return false;
    }
    bytes = b;
    return true;
  }
};

}  // namespace otb
