// Single-pass prefix sums with decoupled look-back (Merrill & Garland, 2016).
//
// Replaces the CUB DeviceScan::ExclusiveSum wrapper of the reference
// (triangle_extraction/compute_exclusive_cumsum.cu:8-39) and the int64
// torch.cumsum of triangle_rasterization/generate_keys.py:48.
//
// One kernel per scan: tiles of 256 threads x 16 items are claimed in launch
// order through an atomic counter, so every predecessor of a tile has already
// started when the tile looks back, and the look-back always terminates. The
// wait is still bounded: after kSpinLimit polls a tile records
// MT_ERR_DEVICE_TIMEOUT in the workspace status word and stops waiting.
//
// Workspace layout: [0,4) status, [4,8) tile counter, [256, 256+8*tiles)
// tile descriptors. Descriptor = (inclusive-or-aggregate value << 2) | flag.

#include <atomic>
#include <mutex>

#include "lookback.cuh"

namespace mt {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr size_t kScanHeader = 256;

// Loads kScanItems consecutive elements owned by this thread.
template <typename TI, typename TO, bool kVector>
__device__ __forceinline__ void load_items(const TI* in, int64_t first, int64_t n, TO (&x)[kScanItems]) {
  if (kVector && first + kScanItems <= n) {
    constexpr int kPer = 16 / sizeof(TI);
    const int4* p = reinterpret_cast<const int4*>(in + first);
#pragma unroll
    for (int v = 0; v < kScanItems / kPer; ++v) {
      int4 w = p[v];
      const TI* e = reinterpret_cast<const TI*>(&w);
#pragma unroll
      for (int k = 0; k < kPer; ++k) x[v * kPer + k] = (TO)e[k];
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) x[k] = (first + k < n) ? (TO)in[first + k] : (TO)0;
  }
}

template <typename TO, bool kVector>
__device__ __forceinline__ void store_items(TO* out, int64_t first, int64_t n, const TO (&x)[kScanItems]) {
  if (kVector && first + kScanItems <= n) {
    constexpr int kPer = 16 / sizeof(TO);
    int4* p = reinterpret_cast<int4*>(out + first);
#pragma unroll
    for (int v = 0; v < kScanItems / kPer; ++v) {
      int4 w;
      TO* e = reinterpret_cast<TO*>(&w);
#pragma unroll
      for (int k = 0; k < kPer; ++k) e[k] = x[v * kPer + k];
      p[v] = w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
      if (first + k < n) out[first + k] = x[k];
  }
}

template <typename TI, typename TO, bool kInclusive, bool kVector>
__global__ void __launch_bounds__(kScanThreads)
    scan_kernel(const TI* in, TO* out, int64_t n, uint32_t* counter, uint64_t* desc, int* status) {
  __shared__ uint32_t s_tile;
  __shared__ TO s_warp[kScanThreads / 32];
  __shared__ TO s_prefix;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t first = tile * kScanTile + (int64_t)tid * kScanItems;

  TO x[kScanItems];
  load_items<TI, TO, kVector>(in, first, n, x);

  // Thread-local inclusive scan.
#pragma unroll
  for (int k = 1; k < kScanItems; ++k) x[k] += x[k - 1];
  const TO thread_total = x[kScanItems - 1];

  // Block-wide scan of the thread totals.
  TO inc = warp_inclusive_sum(thread_total);
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    TO w = (lane < kScanThreads / 32) ? s_warp[lane] : (TO)0;
    TO wi = warp_inclusive_sum(w);
    if (lane < kScanThreads / 32) s_warp[lane] = wi - w;  // exclusive per warp
    const TO block_total = __shfl_sync(0xffffffffu, wi, kScanThreads / 32 - 1);

    const TO prefix = lookback_prefix<TO>(desc, tile, block_total, status);
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();

  const TO offset = s_prefix + s_warp[warp] + (inc - thread_total);
  if (kInclusive) {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) x[k] += offset;
  } else {
    TO prev = offset;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      TO cur = x[k] + offset;
      x[k] = prev;
      prev = cur;
    }
  }
  store_items<TO, kVector>(out, first, n, x);
}

template <typename TI, typename TO, bool kInclusive>
int launch_scan(const TI* in, TO* out, int64_t n, void* ws, size_t ws_bytes, cudaStream_t stream) {
  MT_REQUIRE(n >= 0);
  if (n == 0) return MT_OK;
  MT_REQUIRE(in != nullptr && out != nullptr && ws != nullptr);
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  MT_REQUIRE(tiles < (int64_t)0xffffffff);
  if (ws_bytes < mt_scan_workspace_bytes(n)) return MT_ERR_WORKSPACE_TOO_SMALL;
  char* base = static_cast<char*>(ws);
  // Status word is cumulative across calls sharing a workspace: only the
  // counter and descriptors are reset here.
  if (cudaMemsetAsync(base + 4, 0, 4, stream) != cudaSuccess) return MT_ERR_CUDA;
  if (cudaMemsetAsync(base + kScanHeader, 0, (size_t)tiles * 8, stream) != cudaSuccess) return MT_ERR_CUDA;
  uint32_t* counter = reinterpret_cast<uint32_t*>(base + 4);
  uint64_t* desc = reinterpret_cast<uint64_t*>(base + kScanHeader);
  int* status = reinterpret_cast<int*>(base);
  const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  if (aligned)
    scan_kernel<TI, TO, kInclusive, true><<<(unsigned)tiles, kScanThreads, 0, stream>>>(in, out, n, counter, desc, status);
  else
    scan_kernel<TI, TO, kInclusive, false><<<(unsigned)tiles, kScanThreads, 0, stream>>>(in, out, n, counter, desc, status);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // namespace

int scan_exclusive_i32(int32_t* data, int64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
  return launch_scan<int32_t, int32_t, false>(data, data, n, ws, ws_bytes, s);
}

}  // namespace mt

extern "C" {

size_t mt_scan_workspace_bytes(int64_t n) {
  if (n < 0) n = 0;
  const int64_t tiles = (n + mt::kScanTile - 1) / mt::kScanTile;
  return mt::kScanHeader + (size_t)(tiles > 0 ? tiles : 1) * 8;
}

int mt_exclusive_scan_i32(int32_t* data, int64_t n, void* ws, size_t ws_bytes, mt_stream_t stream) {
  return mt::launch_scan<int32_t, int32_t, false>(data, data, n, ws, ws_bytes, mt::as_stream(stream));
}

int mt_exclusive_scan_i64(int64_t* data, int64_t n, void* ws, size_t ws_bytes, mt_stream_t stream) {
  return mt::launch_scan<int64_t, int64_t, false>(data, data, n, ws, ws_bytes, mt::as_stream(stream));
}

int mt_inclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, void* ws, size_t ws_bytes,
                                 mt_stream_t stream) {
  return mt::launch_scan<int32_t, int64_t, true>(in, out, n, ws, ws_bytes, mt::as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free exclusive scan.
//
// Some callers cannot allocate device memory for the scan's scratch: a plain
// C or C++ host that links this library without any device allocator of its
// own, or code running under a host framework whose memory policy forbids
// new device allocations (or where a cudaMalloc would synchronise the device
// in the middle of its work). For them, this variant keeps its scratch in a
// file-scope __device__ array of fixed size, so a call needs nothing but the
// data pointer and a stream.
//
// Limits and sharing rules:
//   * at most kStaticScanMaxElements (2^26 = 67,108,864) elements per call;
//     larger sizes are rejected with MT_ERR_TOO_LARGE before any work;
//   * the array (131,328 bytes) is resident on every GPU that loads this
//     library, until the process exits;
//   * every call on a device shares the same array and re-initialises the
//     parts that must start at zero, so calls whose work overlaps on the GPU
//     (two streams at once) race and must not be issued;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress, with that device current, and caches it; make
//     that first call before any stream capture on that device.
// ---------------------------------------------------------------------------
namespace mt {
namespace {

constexpr int64_t kStaticScanMaxElements = (int64_t)1 << 26;
constexpr size_t kStaticScanBytes =
    kScanHeader + (size_t)((kStaticScanMaxElements + kScanTile - 1) / kScanTile) * 8;
constexpr int kStaticScanMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scan_scratch[kStaticScanBytes];

// Host-side cache of each device's address of the array above. The symbol
// itself is only a host-side stand-in and must never be passed to a kernel.
std::atomic<void*> g_static_scan_address[kStaticScanMaxDevices];
std::mutex g_static_scan_setup;

int static_scan_scratch(void** out) {
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return MT_ERR_CUDA;
  if (device < 0 || device >= kStaticScanMaxDevices) return MT_ERR_INVALID_ARGUMENT;
  void* p = g_static_scan_address[device].load(std::memory_order_acquire);
  if (p == nullptr) {
    std::lock_guard<std::mutex> lock(g_static_scan_setup);
    p = g_static_scan_address[device].load(std::memory_order_relaxed);
    if (p == nullptr) {
      if (cudaGetSymbolAddress(&p, g_static_scan_scratch) != cudaSuccess || p == nullptr) return MT_ERR_CUDA;
      g_static_scan_address[device].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return MT_OK;
}

}  // namespace
}  // namespace mt

extern "C" {

int64_t mt_exclusive_scan_i32_static_max_elements(void) { return mt::kStaticScanMaxElements; }

int mt_exclusive_scan_i32_static(int32_t* data, int64_t n, mt_stream_t stream) {
  MT_REQUIRE(n >= 0);
  if (n > mt::kStaticScanMaxElements) return MT_ERR_TOO_LARGE;
  if (n == 0) return MT_OK;
  MT_REQUIRE(data != nullptr);
  void* scratch = nullptr;
  const int rc = mt::static_scan_scratch(&scratch);
  if (rc != MT_OK) return rc;
  // The status word is cleared too: calls share the array.
  if (cudaMemsetAsync(scratch, 0, 4, mt::as_stream(stream)) != cudaSuccess) return MT_ERR_CUDA;
  return mt::launch_scan<int32_t, int32_t, false>(data, data, n, scratch, mt::kStaticScanBytes,
                                                  mt::as_stream(stream));
}

}  // extern "C"
