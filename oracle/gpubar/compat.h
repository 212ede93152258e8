// ORACLE / MEASUREMENT INFRASTRUCTURE -- pre-included (nvcc -include) when the
// reference's own CUDA program, SYCL-CUDA-GPU/mainBuilder.cu (owm-cuda), is
// compiled unmodified for sm_103a.  It only bridges the toolkit version: the
// reference was written for CUDA 11-12, and CUDA 13 changed one call it makes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// CUDA 13's cudaMemPrefetchAsync takes a cudaMemLocation and flags; the
// reference passes a device ordinal or cudaCpuDeviceId (the CUDA 12 form).
inline cudaError_t cudaMemPrefetchAsync(const void* ptr, size_t count, int device, cudaStream_t stream = 0) {
  cudaMemLocation loc;
  loc.type = device == cudaCpuDeviceId ? cudaMemLocationTypeHost : cudaMemLocationTypeDevice;
  loc.id = device == cudaCpuDeviceId ? 0 : device;
  return cudaMemPrefetchAsync(ptr, count, loc, 0u, stream);
}
