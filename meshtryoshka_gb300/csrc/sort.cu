// Stable LSD radix sort of (int64 key, int32 value) pairs in signed-key
// order: the onesweep scheme (Adinets & Merrill, 2022) on sm_103a.
//
// Replaces cub::DeviceRadixSort::SortPairs over bits [0, 64) of signed int64
// keys (triangle_rasterization/sort_keys.cu:215-270). Signed order is the
// unsigned order of key ^ 2^63, so digits are taken from the flipped key and
// the original key is written out.
//
// Kernels per sort, all enqueued without host synchronisation:
//   1. histogram: one read of the keys builds the digit histogram of every
//      pass;
//   2. plan: per pass, exclusive digit offsets; a pass whose digit is the same
//      for every key is an identity permutation and is skipped; the active
//      passes are chained in->(alt|out)->...->out so the last lands in `out`;
//   3. one onesweep kernel per pass: tiles are claimed in launch order, each
//      ranks its keys stably with warp match/ballot multisplit, publishes its
//      per-digit counts, looks back over predecessor tiles (bounded spin),
//      and scatters through shared memory so global writes are digit runs;
//   4. copy: in->out when every pass was skipped.
//
// The pair count may live on the device (the output of a preceding scan):
// every kernel then reads it and sorts min(count, capacity) pairs, so the
// sort needs no host synchronisation and can be captured in a graph. Tiles
// past the count return right after claiming their index; no live tile ever
// looks back at them.

#include "mt_common.cuh"

namespace mt {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 12;
constexpr int kSortTile = kSortThreads * kSortItems;  // 3072 keys
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;
constexpr uint64_t kSignFlip = 0x8000000000000000ull;
constexpr int kSpinLimit = 1 << 22;

constexpr uint64_t kLbAggregate = 1;
constexpr uint64_t kLbPrefix = 2;

struct SortPass {
  int active;
  int shift;
  uint32_t mask;
  int pad;
  const uint64_t* ksrc;
  const int32_t* vsrc;
  uint64_t* kdst;
  int32_t* vdst;
};

struct SortPlan {
  SortPass pass[kMaxPasses];
  int copy_needed;
};

// Workspace layout (bytes).
constexpr size_t kOffStatus = 0;
constexpr size_t kOffCounters = 64;                    // kMaxPasses x u32
constexpr size_t kOffHist = 128;                       // kMaxPasses x 256 x u32
constexpr size_t kOffPlan = kOffHist + kMaxPasses * kRadix * 4;
constexpr size_t kOffLookback = (kOffPlan + sizeof(SortPlan) + 255) / 256 * 256;

inline size_t lookback_bytes(int64_t n) {
  const int64_t tiles = (n + kSortTile - 1) / kSortTile;
  return (size_t)(tiles > 0 ? tiles : 1) * kRadix * 8;
}

inline size_t alt_offset(int64_t n) { return (kOffLookback + lookback_bytes(n) + 255) / 256 * 256; }

__device__ __forceinline__ int64_t live_count(int64_t capacity, const int64_t* count) {
  return count ? min(max(*count, (int64_t)0), capacity) : capacity;
}

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Look-back word: [63:60] pass tag (pass + 1), [59:58] flag, [57:0] value.
__device__ __forceinline__ uint64_t lb_pack(int pass, uint64_t flag, uint64_t value) {
  return ((uint64_t)(pass + 1) << 60) | (flag << 58) | (value & ((1ull << 58) - 1));
}

__global__ void __launch_bounds__(256) sort_histogram_kernel(const uint64_t* __restrict__ keys, int64_t capacity,
                                                             const int64_t* __restrict__ count, int num_passes,
                                                             int begin_bit, int end_bit,
                                                             uint32_t* __restrict__ hist) {
  const int64_t n = live_count(capacity, count);
  __shared__ uint32_t s_hist[kMaxPasses][kRadix];
  for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&s_hist[0][0])[i] = 0;
  __syncthreads();
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[idx] ^ kSignFlip;
    for (int p = 0; p < num_passes; ++p) {
      const int shift = begin_bit + 8 * p;
      const int bits = min(8, end_bit - shift);
      const uint32_t d = (uint32_t)(k >> shift) & ((1u << bits) - 1u);
      atomicAdd(&s_hist[p][d], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < num_passes * kRadix; i += blockDim.x) {
    const uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(hist + i, c);
  }
}

__global__ void __launch_bounds__(kRadix) sort_plan_kernel(const uint64_t* keys_in, const int32_t* vals_in,
                                                           uint64_t* keys_out, int32_t* vals_out, uint64_t* keys_alt,
                                                           int32_t* vals_alt, int64_t capacity,
                                                           const int64_t* count, int num_passes, int begin_bit,
                                                           int end_bit, uint32_t* hist, SortPlan* plan) {
  const int64_t n = live_count(capacity, count);
  __shared__ int s_active[kMaxPasses];
  __shared__ uint32_t s_warp[kRadix / 32];
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  for (int p = 0; p < num_passes; ++p) {
    const uint32_t c = hist[p * kRadix + d];
    const int full = __syncthreads_or((int64_t)c == n);
    // Block exclusive scan of the 256 counts.
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += s_warp[w];
    hist[p * kRadix + d] = before + x - c;
    if (d == 0) s_active[p] = !full;
    __syncthreads();
  }
  if (d == 0) {
    int m = 0;
    for (int p = 0; p < num_passes; ++p) m += s_active[p];
    const uint64_t* ks = keys_in;
    const int32_t* vs = vals_in;
    int i = 0;
    for (int p = 0; p < kMaxPasses; ++p) {
      SortPass sp{};
      sp.active = (p < num_passes) ? s_active[p] : 0;
      sp.shift = begin_bit + 8 * p;
      const int bits = (p < num_passes) ? min(8, end_bit - sp.shift) : 8;
      sp.mask = (1u << bits) - 1u;
      if (sp.active) {
        const bool to_out = ((m - 1 - i) % 2) == 0;
        sp.ksrc = ks;
        sp.vsrc = vs;
        sp.kdst = to_out ? keys_out : keys_alt;
        sp.vdst = to_out ? vals_out : vals_alt;
        ks = sp.kdst;
        vs = sp.vdst;
        ++i;
      }
      plan->pass[p] = sp;
    }
    plan->copy_needed = (m == 0);
  }
}

__global__ void __launch_bounds__(kSortThreads) sort_pass_kernel(const SortPlan* __restrict__ plan, int p,
                                                                 const uint32_t* __restrict__ hist,
                                                                 uint32_t* __restrict__ counter,
                                                                 uint64_t* __restrict__ lookback,
                                                                 int64_t capacity, const int64_t* __restrict__ live,
                                                                 int* __restrict__ status) {
  const SortPass ps = plan->pass[p];
  if (!ps.active) return;
  const int64_t n = live_count(capacity, live);

  __shared__ uint32_t s_warp_hist[kSortWarps][kRadix];
  __shared__ uint32_t s_digit_start[kRadix];
  __shared__ int64_t s_global[kRadix];
  __shared__ uint64_t s_keys[kSortTile];
  __shared__ int32_t s_vals[kSortTile];
  __shared__ uint32_t s_scan[kSortWarps];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(counter + p, 1u);
  for (int i = lane; i < kRadix; i += 32) s_warp_hist[warp][i] = 0;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t tile_base = tile * kSortTile;
  if (tile_base >= n) return;  // past the live pairs: nothing to publish

  // Warp-striped load: warp w owns [w * 32 * items, (w + 1) * 32 * items) of
  // the tile; item i of lane l sits at i * 32 + l, so (item, lane) order is
  // the input order.
  uint64_t key[kSortItems];
  int32_t val[kSortItems];
  uint32_t dig[kSortItems];
  uint32_t rank[kSortItems];
  const int64_t warp_base = tile_base + (int64_t)warp * 32 * kSortItems;
#pragma unroll
  for (int i = 0; i < kSortItems; ++i) {
    const int64_t idx = warp_base + i * 32 + lane;
    const bool valid = idx < n;
    key[i] = valid ? ps.ksrc[idx] : 0ull;
    val[i] = valid ? ps.vsrc[idx] : 0;
    dig[i] = valid ? ((uint32_t)((key[i] ^ kSignFlip) >> ps.shift) & ps.mask) : (uint32_t)kRadix;
  }

  // Stable warp-level multisplit: lanes with the same digit in the same item
  // are ranked by lane; items are processed in order.
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int i = 0; i < kSortItems; ++i) {
    const uint32_t peers = __match_any_sync(0xffffffffu, dig[i]);
    const bool valid = dig[i] < (uint32_t)kRadix;
    const uint32_t base = valid ? s_warp_hist[warp][dig[i]] : 0u;
    __syncwarp();
    rank[i] = base + __popc(peers & lt);
    if (valid && (peers & lt) == 0) s_warp_hist[warp][dig[i]] = base + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Thread d owns digit d: per-warp exclusive offsets and the tile's count.
  const int d = tid;
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    const uint32_t c = s_warp_hist[w][d];
    s_warp_hist[w][d] = count;
    count += c;
  }
  // Exclusive scan of counts over digits -> block-local digit starts.
  {
    uint32_t x = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_scan[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += s_scan[w];
    s_digit_start[d] = before + x - count;
  }

  // Decoupled look-back for digit d across tiles.
  uint64_t prefix = 0;
  uint64_t* my = lookback + tile * kRadix + d;
  if (tile == 0) {
    st_relaxed(my, lb_pack(p, kLbPrefix, count));
  } else {
    st_relaxed(my, lb_pack(p, kLbAggregate, count));
    int64_t t = tile - 1;
    int spins = 0;
    while (t >= 0) {
      const uint64_t w = ld_relaxed(lookback + t * kRadix + d);
      const int tag = (int)(w >> 60);
      const uint64_t flag = (w >> 58) & 3u;
      if (tag != p + 1 || flag == 0) {
        if (++spins > kSpinLimit) {
          set_device_error(status, MT_ERR_DEVICE_TIMEOUT);
          break;
        }
        __nanosleep(20);
        continue;
      }
      prefix += w & ((1ull << 58) - 1);
      if (flag == kLbPrefix) break;
      --t;
    }
    st_relaxed(my, lb_pack(p, kLbPrefix, prefix + count));
  }
  s_global[d] = (int64_t)hist[p * kRadix + d] + (int64_t)prefix - (int64_t)s_digit_start[d];
  __syncthreads();

  // Scatter into shared memory in (digit, stable rank) order.
#pragma unroll
  for (int i = 0; i < kSortItems; ++i) {
    if (dig[i] < (uint32_t)kRadix) {
      const uint32_t pos = s_digit_start[dig[i]] + s_warp_hist[warp][dig[i]] + rank[i];
      s_keys[pos] = key[i];
      s_vals[pos] = val[i];
    }
  }
  __syncthreads();

  // Write runs of equal digits to their global positions.
  const int64_t remaining = n - tile_base;
  const int tile_count = (int)(remaining < kSortTile ? remaining : kSortTile);
  for (int j = tid; j < tile_count; j += kSortThreads) {
    const uint64_t k = s_keys[j];
    const uint32_t dj = (uint32_t)((k ^ kSignFlip) >> ps.shift) & ps.mask;
    const int64_t g = s_global[dj] + j;
    ps.kdst[g] = k;
    ps.vdst[g] = s_vals[j];
  }
}

__global__ void sort_copy_kernel(const SortPlan* __restrict__ plan, const uint64_t* __restrict__ kin,
                                 const int32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                 int32_t* __restrict__ vout, int64_t capacity, const int64_t* __restrict__ count) {
  if (!plan->copy_needed) return;
  const int64_t n = live_count(capacity, count);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    kout[i] = kin[i];
    vout[i] = vin[i];
  }
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

size_t mt_sort_pairs_workspace_bytes(int64_t n) {
  if (n < 0) n = 0;
  return alt_offset(n) + (size_t)n * 8 + 256 + (size_t)n * 4;
}

int mt_sort_pairs_i64_i32(const int64_t* keys_in, const int32_t* values_in, int64_t* keys_out, int32_t* values_out,
                          int64_t n, const int64_t* count, int32_t begin_bit, int32_t end_bit, void* workspace,
                          size_t workspace_bytes, mt_stream_t stream) {
  MT_REQUIRE(n >= 0);
  MT_REQUIRE(begin_bit >= 0 && end_bit <= 64 && begin_bit < end_bit);
  if (n == 0) return MT_OK;
  MT_REQUIRE(n < ((int64_t)1 << 32));
  MT_REQUIRE(keys_in && values_in && keys_out && values_out && workspace);
  MT_REQUIRE((const void*)keys_in != (const void*)keys_out && (const void*)values_in != (const void*)values_out);
  if (workspace_bytes < mt_sort_pairs_workspace_bytes(n)) return MT_ERR_WORKSPACE_TOO_SMALL;
  cudaStream_t s = as_stream(stream);
  char* ws = static_cast<char*>(workspace);
  const int num_passes = (end_bit - begin_bit + 7) / 8;
  const int64_t tiles = (n + kSortTile - 1) / kSortTile;
  // Reset counters, histograms and look-back words (not the status word).
  if (cudaMemsetAsync(ws + kOffCounters, 0, kOffPlan - kOffCounters, s) != cudaSuccess) return MT_ERR_CUDA;
  if (cudaMemsetAsync(ws + kOffLookback, 0, lookback_bytes(n), s) != cudaSuccess) return MT_ERR_CUDA;
  int* status = reinterpret_cast<int*>(ws + kOffStatus);
  uint32_t* counters = reinterpret_cast<uint32_t*>(ws + kOffCounters);
  uint32_t* hist = reinterpret_cast<uint32_t*>(ws + kOffHist);
  SortPlan* plan = reinterpret_cast<SortPlan*>(ws + kOffPlan);
  uint64_t* lookback = reinterpret_cast<uint64_t*>(ws + kOffLookback);
  uint64_t* kalt = reinterpret_cast<uint64_t*>(ws + alt_offset(n));
  int32_t* valt = reinterpret_cast<int32_t*>(ws + (alt_offset(n) + (size_t)n * 8 + 255) / 256 * 256);
  const uint64_t* kin = reinterpret_cast<const uint64_t*>(keys_in);
  uint64_t* kout = reinterpret_cast<uint64_t*>(keys_out);

  sort_histogram_kernel<<<grid_stride_blocks(n, 256, 4), 256, 0, s>>>(kin, n, count, num_passes, begin_bit, end_bit,
                                                                      hist);
  MT_CHECK_LAUNCH();
  sort_plan_kernel<<<1, kRadix, 0, s>>>(kin, values_in, kout, values_out, kalt, valt, n, count, num_passes,
                                        begin_bit, end_bit, hist, plan);
  MT_CHECK_LAUNCH();
  for (int p = 0; p < num_passes; ++p) {
    sort_pass_kernel<<<(unsigned)tiles, kSortThreads, 0, s>>>(plan, p, hist, counters, lookback, n, count, status);
    MT_CHECK_LAUNCH();
  }
  sort_copy_kernel<<<grid_stride_blocks(n, 256, 2), 256, 0, s>>>(plan, kin, values_in, kout, values_out, n, count);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
