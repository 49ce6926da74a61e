// Error text, version and the device-memory helpers of the sl3dgpu C ABI.
#include <string>

#include "common.cuh"

namespace sl3dgpu {

namespace {
thread_local std::string lastError;
}

void SetError(const std::string& text) { lastError = text; }

}  // namespace sl3dgpu

extern "C" const char* sl3dgpu_last_error(void) { return sl3dgpu::lastError.c_str(); }

extern "C" const char* sl3dgpu_version(void) { return "sl3dgpu 0.1 (sm_103a)"; }

extern "C" int sl3dgpu_device_alloc(long long bytes, void** out) {
  if (out == nullptr || bytes < 0) {
    sl3dgpu::SetError("device_alloc: an output pointer and bytes >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  *out = nullptr;
  if (bytes == 0) return SL3DGPU_OK;
  SL3D_CUDA(cudaMalloc(out, static_cast<size_t>(bytes)));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_device_free(void* p) {
  if (p != nullptr) SL3D_CUDA(cudaFree(p));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_device_copy(void* dst, const void* src, long long bytes) {
  if (bytes < 0 || (bytes > 0 && (dst == nullptr || src == nullptr))) {
    sl3dgpu::SetError("device_copy: two pointers and bytes >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (bytes > 0) SL3D_CUDA(cudaMemcpy(dst, src, static_cast<size_t>(bytes), cudaMemcpyDefault));
  return SL3DGPU_OK;
}
