// Single-pass prefix sums with decoupled look-back (Merrill & Garland, 2016).
//
// Replaces the CUB DeviceScan::ExclusiveSum wrapper of the reference
// (triangle_extraction/compute_exclusive_cumsum.cu:8-39) and the int64
// torch.cumsum of triangle_rasterization/generate_keys.py:48.
//
// One kernel per scan. Tiles of 256 threads x 48 elements (24 for 64-bit
// results) are claimed in launch order through an atomic counter, so every
// predecessor of a tile has already started when the tile looks back, and
// the look-back always terminates. The wait is still bounded: after
// kSpinLimit polls a tile records MT_ERR_DEVICE_TIMEOUT in the workspace
// status word and stops waiting.
//
// Each warp owns a run of consecutive elements of its tile and moves them
// with 16-byte vector accesses in warp-contiguous rounds (round r, lane l:
// the vector at 16 (32 r + l) bytes of the run), so every load and store
// instruction of the warp covers one contiguous 512-byte span, with
// streaming cache hints (the data is touched once). The scan runs in that
// striped order: within each vector, across the lanes of a round (warp
// shuffles), across the rounds, across the CTA's warps, then across tiles
// (look-back by one warp).
//
// Workspace layout: [0,4) status, [4,8) tile counter, [256, 256+8*tiles)
// tile descriptors. Descriptor = (inclusive-or-aggregate value << 2) | flag.

#include <atomic>
#include <mutex>

#include "lookback.cuh"

namespace mt {
namespace {

constexpr int kScanThreads = 256;
constexpr size_t kScanHeader = 256;

// Elements per thread: 48, or 24 when the results are 64-bit (registers).
template <typename TO>
constexpr int scan_items() {
  return sizeof(TO) == 4 ? 48 : 24;
}

// The smallest tile of any scan here: workspaces are sized by it.
constexpr int kScanTileMin = kScanThreads * 24;

template <typename TI, typename TO, bool kInclusive, bool kVector>
__global__ void __launch_bounds__(kScanThreads)
    scan_kernel(const TI* in, TO* out, int64_t n, uint32_t* counter, uint64_t* desc, int* status) {
  constexpr int kItems = scan_items<TO>();
  constexpr int V = 16 / (int)sizeof(TI);  // elements per 16-byte vector
  constexpr int R = kItems / V;            // vectors per thread
  constexpr int kWarps = kScanThreads / 32;
  __shared__ uint32_t s_tile;
  __shared__ TO s_warp[kWarps];
  __shared__ TO s_prefix;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t seg = tile * (kScanThreads * kItems) + (int64_t)warp * (32 * kItems);
  const bool full = kVector && seg + 32 * kItems <= n;
  TO x[R][V];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int64_t first = seg + (int64_t)(32 * r + lane) * V;
    if (full) {
      const int4 w = __ldcs(reinterpret_cast<const int4*>(in + first));
      const TI* e = reinterpret_cast<const TI*>(&w);
#pragma unroll
      for (int v = 0; v < V; ++v) x[r][v] = (TO)e[v];
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) x[r][v] = (first + v < n) ? (TO)in[first + v] : (TO)0;
    }
  }

  // Within each vector, then across the lanes of each round, then across
  // the rounds.
  TO lane_excl[R];
  TO warp_total = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int v = 1; v < V; ++v) x[r][v] += x[r][v - 1];
    const TO inc = warp_inclusive_sum(x[r][V - 1]);
    lane_excl[r] = inc - x[r][V - 1] + warp_total;
    warp_total += __shfl_sync(0xffffffffu, inc, 31);
  }
  if (lane == 0) s_warp[warp] = warp_total;
  __syncthreads();
  if (warp == 0) {
    const TO w = lane < kWarps ? s_warp[lane] : (TO)0;
    const TO wi = warp_inclusive_sum(w);
    if (lane < kWarps) s_warp[lane] = wi - w;  // exclusive per warp
    const TO block_total = __shfl_sync(0xffffffffu, wi, kWarps - 1);
    const TO prefix = lookback_prefix<TO>(desc, tile, block_total, status);
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  const TO offset = s_prefix + s_warp[warp];

#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int64_t first = seg + (int64_t)(32 * r + lane) * V;
    const TO base = lane_excl[r] + offset;
    TO y[V];
#pragma unroll
    for (int v = 0; v < V; ++v) y[v] = kInclusive ? base + x[r][v] : (v == 0 ? base : base + x[r][v - 1]);
    if (full) {
      constexpr int kOut = 16 / (int)sizeof(TO);  // results per 16-byte store
#pragma unroll
      for (int v = 0; v < V; v += kOut) {
        int4 w;
        TO* e = reinterpret_cast<TO*>(&w);
#pragma unroll
        for (int k = 0; k < kOut; ++k) e[k] = y[v + k];
        __stcs(reinterpret_cast<int4*>(out + first + v), w);
      }
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v)
        if (first + v < n) out[first + v] = y[v];
    }
  }
}

template <typename TI, typename TO, bool kInclusive>
int launch_scan(const TI* in, TO* out, int64_t n, void* ws, size_t ws_bytes, cudaStream_t stream) {
  MT_REQUIRE(n >= 0);
  if (n == 0) return MT_OK;
  MT_REQUIRE(in != nullptr && out != nullptr && ws != nullptr);
  constexpr int64_t kTile = (int64_t)kScanThreads * scan_items<TO>();
  const int64_t tiles = (n + kTile - 1) / kTile;
  MT_REQUIRE(tiles < (int64_t)0x7fffffff);
  if (ws_bytes < mt_scan_workspace_bytes(n)) return MT_ERR_WORKSPACE_TOO_SMALL;
  char* base = static_cast<char*>(ws);
  // Status word is cumulative across calls sharing a workspace: only the
  // counter and the descriptors are reset here, in one fill (with the unused
  // header bytes between them).
  if (cudaMemsetAsync(base + 4, 0, kScanHeader - 4 + (size_t)tiles * 8, stream) != cudaSuccess) return MT_ERR_CUDA;
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

// One warp looks back from tile 1 over a descriptor array whose tile 0 never
// publishes: the wait gives up after `spin_limit` polls, records
// MT_ERR_DEVICE_TIMEOUT in the status word and treats the missing tile as an
// empty prefix; out[0] receives the prefix the look-back returned.
__global__ void lookback_timeout_kernel(uint64_t* desc, int* status, int spin_limit, int64_t* out) {
  const int64_t prefix = lookback_prefix<int64_t>(desc, 1, (int64_t)5, status, spin_limit);
  if (threadIdx.x == 0) out[0] = prefix;
}

}  // namespace

int scan_exclusive_i32(int32_t* data, int64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
  return launch_scan<int32_t, int32_t, false>(data, data, n, ws, ws_bytes, s);
}

}  // namespace mt

extern "C" {

size_t mt_scan_workspace_bytes(int64_t n) {
  if (n < 0) n = 0;
  const int64_t tiles = (n + mt::kScanTileMin - 1) / mt::kScanTileMin;
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

int mt_test_lookback_timeout(int32_t spin_limit, int64_t* prefix_out, void* ws, size_t ws_bytes,
                             mt_stream_t stream) {
  MT_REQUIRE(spin_limit >= 1 && spin_limit <= (1 << 20) && prefix_out != nullptr && ws != nullptr);
  if (ws_bytes < mt::kScanHeader + 16) return MT_ERR_WORKSPACE_TOO_SMALL;
  char* base = static_cast<char*>(ws);
  cudaStream_t s = mt::as_stream(stream);
  // Tile 0's descriptor stays zero ("not ready"): nothing ever publishes it.
  if (cudaMemsetAsync(base + mt::kScanHeader, 0, 16, s) != cudaSuccess) return MT_ERR_CUDA;
  mt::lookback_timeout_kernel<<<1, 32, 0, s>>>(reinterpret_cast<uint64_t*>(base + mt::kScanHeader),
                                               reinterpret_cast<int*>(base), spin_limit, prefix_out);
  MT_CHECK_LAUNCH();
  return MT_OK;
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
//   * the array (87,640 bytes) is resident on every GPU that loads this
//     library, until the process exits;
//   * every call on a device shares the same array and re-initialises the
//     parts that must start at zero, so calls whose work overlaps on the GPU
//     (two streams at once) race and must not be issued;
//   * the first call in a CUDA context (with that context current) looks up
//     the array's device address with cudaGetSymbolAddress and caches it
//     under the context's unique id, so a device reset (which destroys the
//     primary context) or a driver-API context of the caller's own gets its
//     own lookup; make the first call in a context before any stream capture
//     in it;
//   * a look-back that gave up waiting (MT_ERR_DEVICE_TIMEOUT) leaves its
//     code in the array's status word, which the next call clears;
//     mt_exclusive_scan_i32_static_status copies that word out.
// ---------------------------------------------------------------------------
namespace mt {
namespace {

constexpr int64_t kStaticScanMaxElements = (int64_t)1 << 26;
constexpr size_t kStaticScanBytes =
    kScanHeader + (size_t)((kStaticScanMaxElements + kScanTileMin - 1) / kScanTileMin) * 8;
constexpr int kStaticScanMaxContexts = 64;

static __device__ __align__(256) unsigned char g_static_scan_scratch[kStaticScanBytes];

// Host-side cache of the array's device address per CUDA context (keyed by
// the driver's context id, which is never reused within a process). The
// symbol itself is only a host-side stand-in and must never be passed to a
// kernel.
struct StaticScanEntry {
  unsigned long long context_id;
  void* address;
};
StaticScanEntry g_static_scan_cache[kStaticScanMaxContexts];
int g_static_scan_entries = 0;
std::mutex g_static_scan_setup;

using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

// The current context's id through the driver entry points the runtime
// hands out (this library links only the runtime). *none is set when no
// context is current on this thread yet.
int current_context_id(unsigned long long* id, bool* none) {
  static std::atomic<CtxGetCurrentFn> get_current{nullptr};
  static std::atomic<CtxGetIdFn> get_id{nullptr};
  *none = false;
  CtxGetCurrentFn fc = get_current.load(std::memory_order_acquire);
  CtxGetIdFn fi = get_id.load(std::memory_order_acquire);
  if (fc == nullptr || fi == nullptr) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || a == nullptr)
      return MT_ERR_CUDA;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qb != cudaDriverEntryPointSuccess || b == nullptr)
      return MT_ERR_CUDA;
    fc = reinterpret_cast<CtxGetCurrentFn>(a);
    fi = reinterpret_cast<CtxGetIdFn>(b);
    get_current.store(fc, std::memory_order_release);
    get_id.store(fi, std::memory_order_release);
  }
  void* ctx = nullptr;
  if (fc(&ctx) != 0) return MT_ERR_CUDA;
  if (ctx == nullptr) {
    *none = true;
    return MT_OK;
  }
  if (fi(ctx, id) != 0) return MT_ERR_CUDA;
  return MT_OK;
}

int static_scan_scratch(void** out) {
  unsigned long long id = 0;
  bool none = false;
  int rc = current_context_id(&id, &none);
  if (rc != MT_OK) return rc;
  std::lock_guard<std::mutex> lock(g_static_scan_setup);
  if (!none) {
    for (int i = 0; i < g_static_scan_entries; ++i) {
      if (g_static_scan_cache[i].context_id == id) {
        *out = g_static_scan_cache[i].address;
        return MT_OK;
      }
    }
  }
  // Set-up for this context (with no context current yet, this binds the
  // runtime to the current device's primary context first).
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_static_scan_scratch) != cudaSuccess || p == nullptr) return MT_ERR_CUDA;
  if (none) {
    rc = current_context_id(&id, &none);
    if (rc != MT_OK || none) return MT_ERR_CUDA;
  }
  // A full table forgets its oldest context (contexts that old are long gone
  // in every realistic process).
  if (g_static_scan_entries == kStaticScanMaxContexts) {
    for (int i = 1; i < kStaticScanMaxContexts; ++i) g_static_scan_cache[i - 1] = g_static_scan_cache[i];
    --g_static_scan_entries;
  }
  g_static_scan_cache[g_static_scan_entries++] = StaticScanEntry{id, p};
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

int mt_exclusive_scan_i32_static_status(int32_t* status_out, mt_stream_t stream) {
  MT_REQUIRE(status_out != nullptr);
  void* scratch = nullptr;
  const int rc = mt::static_scan_scratch(&scratch);
  if (rc != MT_OK) return rc;
  if (cudaMemcpyAsync(status_out, scratch, 4, cudaMemcpyDefault, mt::as_stream(stream)) != cudaSuccess)
    return MT_ERR_CUDA;
  return MT_OK;
}

}  // extern "C"
