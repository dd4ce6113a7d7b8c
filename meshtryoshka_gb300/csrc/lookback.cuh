// Decoupled look-back (Merrill & Garland, 2016) of the single-pass scans
// (scan.cu), and the warp sums they use (also used by the capacity-mode key
// kernels of raster_front.cu).
//
// Tiles are claimed in launch order through an atomic counter, so every
// predecessor of a tile has already started when the tile looks back and the
// look-back always terminates. The wait is still bounded: after kSpinLimit
// polls of one descriptor the tile records MT_ERR_DEVICE_TIMEOUT in the status
// word and treats the descriptor as an empty prefix.
//
// Descriptor = (inclusive-or-aggregate value << 2) | flag; zero = not ready.
#pragma once

#include "mt_common.cuh"

namespace mt {

constexpr uint64_t kFlagAggregate = 1;
constexpr uint64_t kFlagPrefix = 2;
constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t pack_desc(int64_t value, uint64_t flag) {
  return ((uint64_t)value << 2) | flag;
}

__device__ __forceinline__ int64_t desc_value(uint64_t d) { return (int64_t)d >> 2; }

template <typename T>
__device__ __forceinline__ T warp_inclusive_sum(T x) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) >= o) x += y;
  }
  return x;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Called by all 32 lanes of one warp of tile `tile` with the tile's total.
// Publishes the tile's aggregate, gathers the exclusive prefix of all earlier
// tiles, publishes the inclusive prefix and returns the exclusive prefix (in
// every lane). `spin_limit` bounds the polls of one descriptor.
template <typename T>
__device__ __forceinline__ T lookback_prefix(uint64_t* desc, int64_t tile, T block_total, int* status,
                                             int spin_limit = kSpinLimit) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_relaxed(&desc[0], pack_desc((int64_t)block_total, kFlagPrefix));
    return (T)0;
  }
  if (lane == 0) st_relaxed(&desc[tile], pack_desc((int64_t)block_total, kFlagAggregate));
  T prefix = 0;
  int64_t window = tile - 1;
  bool timed_out = false;
  while (true) {
    const int64_t pred = window - lane;
    uint64_t d = pack_desc(0, kFlagPrefix);  // virtual prefix before tile 0
    if (pred >= 0) {
      int spins = 0;
      d = ld_relaxed(&desc[pred]);
      while ((d & 3) == 0) {
        if (++spins > spin_limit) {
          timed_out = true;
          d = pack_desc(0, kFlagPrefix);
          break;
        }
        __nanosleep(32);
        d = ld_relaxed(&desc[pred]);
      }
    }
    const unsigned prefix_lanes = __ballot_sync(0xffffffffu, (d & 3) == kFlagPrefix);
    const int stop = prefix_lanes ? __ffs(prefix_lanes) - 1 : 31;
    const T contrib = (lane <= stop) ? (T)desc_value(d) : (T)0;
    prefix += warp_sum(contrib);
    if (prefix_lanes) break;
    window -= 32;
  }
  if (__any_sync(0xffffffffu, timed_out) && lane == 0) set_device_error(status, MT_ERR_DEVICE_TIMEOUT);
  if (lane == 0) st_relaxed(&desc[tile], pack_desc((int64_t)(prefix + block_total), kFlagPrefix));
  return prefix;
}

}  // namespace mt
