// Shared device/host helpers for the meshtryoshka_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/meshtryoshka_gb300.h"

#define MT_CHECK_LAUNCH()                                   \
  do {                                                      \
    cudaError_t _e = cudaGetLastError();                    \
    if (_e != cudaSuccess) return MT_ERR_CUDA;              \
  } while (0)

#define MT_REQUIRE(cond)                                    \
  do {                                                      \
    if (!(cond)) return MT_ERR_INVALID_ARGUMENT;            \
  } while (0)

namespace mt {

constexpr int kSmCount = 152;  // GB300: 2 dies x 76 SMs.

inline unsigned grid_1d(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// Grid-stride launch size: enough CTAs to fill every SM several times over,
// capped so that tiny problems do not launch idle CTAs.
inline unsigned grid_stride_blocks(int64_t n, int block, int ctas_per_sm = 8) {
  int64_t need = (n + block - 1) / block;
  int64_t cap = (int64_t)kSmCount * ctas_per_sm;
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

inline cudaStream_t as_stream(mt_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Saturating float -> int32 conversion with truncation toward zero; NaN maps
// to 0. This is what `int(x)` compiles to on the GPU (cvt.rzi.s32.f32).
__device__ __forceinline__ int f2i_rz(float x) { return __float2int_rz(x); }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Record the first device-side error code in a status word (0 = ok).
__device__ __forceinline__ void set_device_error(int* status, int code) {
  if (status != nullptr) atomicCAS(status, 0, code);
}

// Raises a kernel's dynamic shared-memory limit once per device and size, so
// repeated launches (and launches under stream capture) make no attribute
// calls. The template argument is the kernel itself, so each kernel keeps its
// own record of the largest size set per device.
template <auto Kernel>
inline int set_smem(size_t bytes) {
  if (bytes <= 48 * 1024) return MT_OK;
  static std::atomic<size_t> granted[64];
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MT_ERR_CUDA;
  if (granted[device].load(std::memory_order_acquire) >= bytes) return MT_OK;
  if (cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return MT_ERR_CUDA;
  size_t prev = granted[device].load(std::memory_order_relaxed);
  while (prev < bytes && !granted[device].compare_exchange_weak(prev, bytes)) {
  }
  return MT_OK;
}

}  // namespace mt
