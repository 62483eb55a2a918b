// Force-included (nvcc -include) before the reference's driver headers.
// CUDA 13 removed cudaDeviceProp::clockRate and ::memoryClockRate, which the
// drivers' GPUinfo() prints (e.g. include/bfs_vertex_cuda.h:62-72).  This
// header supplies a property type that carries both fields and fills them from
// cudaDeviceGetAttribute, so the reference headers compile unmodified.
#pragma once
#include <cuda_runtime.h>

struct ig_compat_device_prop : public cudaDeviceProp {
  int clockRate;        // kHz
  int memoryClockRate;  // kHz
};

static inline cudaError_t ig_compat_get_device_properties(ig_compat_device_prop* p, int device) {
  cudaError_t e = cudaGetDeviceProperties(static_cast<cudaDeviceProp*>(p), device);
  if (e != cudaSuccess) return e;
  cudaDeviceGetAttribute(&p->clockRate, cudaDevAttrClockRate, device);
  cudaDeviceGetAttribute(&p->memoryClockRate, cudaDevAttrMemoryClockRate, device);
  return cudaSuccess;
}

#define cudaDeviceProp ig_compat_device_prop
#undef cudaGetDeviceProperties
#define cudaGetDeviceProperties ig_compat_get_device_properties
