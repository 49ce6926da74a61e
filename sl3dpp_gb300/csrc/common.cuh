// Shared helpers of the sl3dgpu CUDA library: status codes, the thread-local
// error text behind sl3dgpu_last_error(), and checked CUDA calls.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/sl3dgpu.h"

namespace sl3dgpu {

void SetError(const std::string& text);

#define SL3D_CUDA(call)                                                        \
  do {                                                                         \
    const cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) {                                                   \
      ::sl3dgpu::SetError(std::string(#call) + ": " + cudaGetErrorString(_e)); \
      return SL3DGPU_ERR_CUDA;                                                 \
    }                                                                          \
  } while (0)

#define SL3D_CHECK_LAUNCH()                                                          \
  do {                                                                               \
    const cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) {                                                         \
      ::sl3dgpu::SetError(std::string("kernel launch: ") + cudaGetErrorString(_e)); \
      return SL3DGPU_ERR_CUDA;                                                       \
    }                                                                                \
  } while (0)

inline cudaStream_t AsStream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// A host-to-device copy whose bytes are in device memory when it returns.
// cudaMemcpy from pageable host memory returns once the data is staged; the
// DMA to the destination may still be running on the legacy stream, and the
// operators' streams are created non-blocking, so they do not wait for it: a
// kernel launched on one of them right after could read the buffer before it
// is written (under a busy GPU, with many operators' streams in flight, it
// did). Every upload of setup data goes through here; waiting for the legacy
// stream puts the DMA behind us.
inline cudaError_t CopyIn(void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  if (const cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice); e != cudaSuccess) return e;
  return cudaStreamSynchronize(cudaStreamLegacy);
}

// A device memset that has landed when it returns (cudaMemset is
// asynchronous on the legacy stream, which non-blocking streams do not wait
// for).
inline cudaError_t ZeroIn(void* dst, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  if (const cudaError_t e = cudaMemset(dst, 0, bytes); e != cudaSuccess) return e;
  return cudaStreamSynchronize(cudaStreamLegacy);
}

// Allow a kernel all the dynamic shared memory the device's opt-in limit
// leaves beside its static shared memory. The attribute is global to the
// function, so it takes one value for every caller: host threads driving
// problems of different sizes would otherwise race between setting it and
// launching. Occupancy follows each launch's actual dynamic size.
template <class F>
inline cudaError_t AllowDynamicSmem(F* kernel) {
  static const int optin = [] {
    int device = 0, bytes = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&bytes, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    return bytes;
  }();
  cudaFuncAttributes a{};
  if (const cudaError_t e = cudaFuncGetAttributes(&a, kernel); e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - static_cast<int>(a.sharedSizeBytes));
}

constexpr int kWarp = 32;

}  // namespace sl3dgpu
