// Tile-bucketed sort of the rasterizer's (key, triangle) pairs for sm_103a:
// the result of a stable sort by signed 64-bit key (sort_keys.cu:241-267 of
// the reference) and the tile ranges of delineate_tiles.slang:14-58, in one
// pass over the keys instead of eight radix passes.
//
// The fields above the depth field (camera | tile, or camera | shell | tile)
// name a bin (one per tile range); the bits below them (depth, and in the
// fused layout the shell) order keys within a bin. So:
//   1. count the keys of every bin (warp-aggregated atomics);
//   2. exclusive-scan the counts: each bin's [start, end) is its tile range;
//   3. scatter every key into its bin as the 64-bit composite
//      (low bits << index bits) | original index;
//   4. sort each bin's composites: the original index breaks ties, so the
//      order is the stable sort's. Bins of up to 256 keys are sorted by one
//      warp, up to 512 by 64-thread CTAs, up to 1024 by 128-thread CTAs,
//      larger ones by 512-thread CTAs
//      (4096 keys in shared memory; beyond that, sorted 4096-key chunks
//      merged pairwise in global memory). In shared memory each thread sorts
//      8 values in registers, then sorted runs are merged (merge path);
//   5. write each sorted key and triangle, gathered by original index.
//
// Valid only when the bin order equals the signed key order (the camera
// field's top bit is clear for every camera) and the composite fits in 63
// bits; the caller checks both and otherwise uses the radix sort.
//
// The three bin sorts touch disjoint bins, so the large-bin sort (whose
// longest bins set the tail) runs on a helper stream forked from the caller's
// stream and joined back with events; the tiny and small sorts fill the SMs
// beside it. Fork and join are ordinary stream dependencies, so the call
// stays capturable in a CUDA graph.

#include <map>
#include <mutex>
#include <utility>

#include "mt_common.cuh"

namespace mt {
namespace {

struct BinMap {
  int cam_off, cam_len, shell_off, shell_len, tile_off, tile_len;
  int separate, B, Sd;
  int64_t T;
};

__device__ __forceinline__ uint64_t low_mask(int bits) { return bits >= 64 ? ~0ull : ((1ull << bits) - 1ull); }

__device__ __forceinline__ int64_t bin_of(const BinMap& m, uint64_t key) {
  const int64_t cam = (int64_t)((key >> m.cam_off) & low_mask(m.cam_len));
  const int64_t sh = m.separate ? (int64_t)((key >> m.shell_off) & low_mask(m.shell_len)) : 0;
  const int64_t tile = (int64_t)((key >> m.tile_off) & low_mask(m.tile_len));
  if (cam >= m.B || sh >= m.Sd || tile >= m.T) return -1;
  return (cam * m.Sd + sh) * m.T + tile;
}

__device__ __forceinline__ int64_t live_keys(int64_t capacity, const int64_t* count) {
  return count ? min(max(*count, (int64_t)0), capacity) : capacity;
}

constexpr int kThreads = 256;       // counting, scatter and tile-range kernels
constexpr int kTinyCap = 256;       // keys per bin sorted by one warp
constexpr int kMediumThreads = 64;
constexpr int kMediumCap = 512;     // keys per bin sorted by a 64-thread CTA
constexpr int kSmallThreads = 128;
constexpr int kSmallCap = 1024;     // keys per bin sorted by a 128-thread CTA
constexpr int kTiers = 4;           // tiny, medium, small, large
constexpr int kLargeThreads = 512;
constexpr int kChunk = 4096;        // keys per shared-memory sort of a 512-thread CTA

// 1. Per-bin counts. Lanes with the same bin add once (their leader).
__global__ void bin_count_kernel(const uint64_t* __restrict__ keys, int64_t Kcap, const int64_t* __restrict__ num_keys,
                                 BinMap m, int32_t* __restrict__ counts, int* __restrict__ status) {
  const int64_t K = live_keys(Kcap, num_keys);
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < K; base += stride) {
    const int64_t i = base + threadIdx.x;
    int64_t b = -2;  // -2: no key in this lane
    if (i < K) {
      b = bin_of(m, keys[i]);
      if (b < 0) set_device_error(status, MT_ERR_INVALID_ARGUMENT);
    }
    const unsigned group = __match_any_sync(0xffffffffu, b);
    if (b >= 0 && lane == __ffs(group) - 1) atomicAdd(counts + b, __popc(group));
  }
}

// 2b. Tile ranges: [start, end) of every non-empty bin, (0, 0) for empty
// bins (delineate_tiles zero-fills its output). Non-empty bins are listed
// for the sorting kernels, small and large ones apart.
__global__ void bin_bounds_kernel(const int32_t* __restrict__ offsets, int64_t nbins, int64_t* __restrict__ bounds,
                                  int2* __restrict__ lists, int32_t* __restrict__ list_sizes) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins; b += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = offsets[b], e = offsets[b + 1];
    bounds[2 * b] = e > s ? s : 0;
    bounds[2 * b + 1] = e > s ? e : 0;
    if (e > s) {
      const int n = e - s;
      const int which = n <= kTinyCap ? 0 : n <= kMediumCap ? 1 : n <= kSmallCap ? 2 : 3;
      lists[which * nbins + atomicAdd(list_sizes + which, 1)] = make_int2(s, n);
    }
  }
}

// 3. Scatter composites into their bins (order inside a bin is arbitrary;
// the composite carries the original index).
__global__ void bin_scatter_kernel(const uint64_t* __restrict__ keys, int64_t Kcap,
                                   const int64_t* __restrict__ num_keys, BinMap m,
                                   const int32_t* __restrict__ offsets, int32_t* __restrict__ cursors, int idx_bits,
                                   uint64_t low_bits_mask, uint64_t* __restrict__ tmp) {
  const int64_t K = live_keys(Kcap, num_keys);
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < K; base += stride) {
    const int64_t i = base + threadIdx.x;
    int64_t b = -2;
    uint64_t key = 0;
    if (i < K) {
      key = keys[i];
      b = bin_of(m, key);
    }
    const unsigned group = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(group) - 1;
    int first = 0;
    if (b >= 0 && lane == leader) first = atomicAdd(cursors + b, __popc(group));
    first = __shfl_sync(0xffffffffu, first, leader);
    if (b >= 0) {
      const int64_t pos = (int64_t)offsets[b] + first + __popc(group & lanemask_lt());
      tmp[pos] = ((key & low_bits_mask) << idx_bits) | (uint64_t)i;
    }
  }
}

// ---------------------------------------------------------------------------
// Block merge sort of up to kT * 8 composites in shared memory: every thread
// sorts 8 values in registers (a 19-comparator network), then sorted runs
// are merged pairwise (merge path) between two shared buffers, so each round
// moves every value once. Padding values are ~0 (composites stay below
// 2^63, so they sort last).
// ---------------------------------------------------------------------------
constexpr int kPerThread = 8;

__device__ __forceinline__ void cmp_swap(uint64_t& a, uint64_t& b) {
  const uint64_t lo = a < b ? a : b, hi = a < b ? b : a;
  a = lo;
  b = hi;
}

__device__ __forceinline__ void sort8(uint64_t (&v)[kPerThread]) {
  cmp_swap(v[0], v[2]); cmp_swap(v[1], v[3]); cmp_swap(v[4], v[6]); cmp_swap(v[5], v[7]);
  cmp_swap(v[0], v[4]); cmp_swap(v[1], v[5]); cmp_swap(v[2], v[6]); cmp_swap(v[3], v[7]);
  cmp_swap(v[0], v[1]); cmp_swap(v[2], v[3]); cmp_swap(v[4], v[5]); cmp_swap(v[6], v[7]);
  cmp_swap(v[2], v[4]); cmp_swap(v[3], v[5]);
  cmp_swap(v[1], v[4]); cmp_swap(v[3], v[6]);
  cmp_swap(v[1], v[2]); cmp_swap(v[3], v[4]); cmp_swap(v[5], v[6]);
}

// Barrier of the threads that sort together: the CTA, or one warp.
template <bool kWarp>
__device__ __forceinline__ void group_sync() {
  if (kWarp) __syncwarp();
  else __syncthreads();
}

// Shared-memory position of logical element i: XOR-swizzled within each run
// of 16 values (one 128-byte bank row of 64-bit words) by the row number, so
// that the 8 consecutive values of neighbouring threads fall on different
// banks.
__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 4) & 15); }

// Sorts src[0, n) (global, n <= kT * 8) in shared memory with the kT
// threads of the group (t = 0 .. kT-1: a CTA, or a warp when kWarp); returns
// the buffer (s or s2, each kT * 8 long, swizzled by swz) that holds the
// sorted values.
template <int kT, bool kWarp = false>
__device__ __forceinline__ const uint64_t* block_merge_sort(const uint64_t* __restrict__ src, int n, uint64_t* s,
                                                            uint64_t* s2, int t) {
  const int runs = (n + kPerThread - 1) / kPerThread;  // threads with a run
  const int total = runs * kPerThread;
  if (t < runs) {
    uint64_t v[kPerThread];
#pragma unroll
    for (int e = 0; e < kPerThread; ++e) {
      const int i = t * kPerThread + e;
      v[e] = i < n ? __ldg(src + i) : ~0ull;
    }
    sort8(v);
#pragma unroll
    for (int e = 0; e < kPerThread; ++e) s[swz(t * kPerThread + e)] = v[e];
  }
  group_sync<kWarp>();
  uint64_t* in = s;
  uint64_t* out = s2;
  for (int len = kPerThread; len < total; len <<= 1) {
    if (t < runs) {
      const int p = t * kPerThread;
      const int ps = (p / (2 * len)) * (2 * len);
      const int na = min(len, total - ps);
      const int nb = max(0, min(len, total - ps - len));
      const int d = p - ps;
      // Elements of a = [ps, ps + na) among the first d outputs.
      int lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (in[swz(ps + mid)] < in[swz(ps + na + d - mid - 1)]) lo = mid + 1;
        else hi = mid;
      }
      int i = lo, j = d - lo;
      uint64_t av = i < na ? in[swz(ps + i)] : ~0ull;
      uint64_t bv = j < nb ? in[swz(ps + na + j)] : ~0ull;
#pragma unroll
      for (int e = 0; e < kPerThread; ++e) {
        const bool take_a = av < bv;
        out[swz(p + e)] = take_a ? av : bv;
        if (take_a) {
          ++i;
          av = i < na ? in[swz(ps + i)] : ~0ull;
        } else {
          ++j;
          bv = j < nb ? in[swz(ps + na + j)] : ~0ull;
        }
      }
    }
    group_sync<kWarp>();
    uint64_t* x = in;
    in = out;
    out = x;
  }
  return in;
}

// 5. Sorted composites -> keys and triangles (gathered by original index),
// four per thread in flight.
template <int kCtaThreads, bool kSwizzled>
__device__ __forceinline__ void write_sorted(const uint64_t* sorted, int64_t n, int64_t start, uint64_t idx_mask,
                                             const uint64_t* __restrict__ keys_in,
                                             const int32_t* __restrict__ tri_in, uint64_t* __restrict__ keys_out,
                                             int32_t* __restrict__ tri_out, int t) {
  constexpr int kUnroll = 4;
  for (int64_t p0 = t; p0 < n; p0 += kUnroll * kCtaThreads) {
    int64_t idx[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const int64_t p = p0 + u * kCtaThreads;
      idx[u] = p < n ? (int64_t)(sorted[kSwizzled ? swz((int)p) : p] & idx_mask) : -1;
    }
    uint64_t k[kUnroll];
    int32_t t[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      if (idx[u] >= 0) {
        k[u] = __ldg(keys_in + idx[u]);
        t[u] = __ldg(tri_in + idx[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      if (idx[u] >= 0) {
        keys_out[start + p0 + u * kCtaThreads] = k[u];
        tri_out[start + p0 + u * kCtaThreads] = t[u];
      }
    }
  }
}

// 4 + 5 for the listed bins of at most kTinyCap keys: one warp per bin.
constexpr int kTinyWarps = 8;

__global__ void __launch_bounds__(32 * kTinyWarps)
    bin_sort_tiny_kernel(const uint64_t* __restrict__ tmp, const int2* __restrict__ list,
                         const int32_t* __restrict__ list_size, uint64_t idx_mask,
                         const uint64_t* __restrict__ keys_in, const int32_t* __restrict__ tri_in,
                         uint64_t* __restrict__ keys_out, int32_t* __restrict__ tri_out) {
  __shared__ uint64_t s[kTinyWarps][2][kTinyCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int count = *list_size;
  for (int l = blockIdx.x * kTinyWarps + warp; l < count; l += gridDim.x * kTinyWarps) {
    const int2 e = list[l];
    const uint64_t* sorted = block_merge_sort<32, true>(tmp + e.x, e.y, s[warp][0], s[warp][1], lane);
    write_sorted<32, true>(sorted, e.y, e.x, idx_mask, keys_in, tri_in, keys_out, tri_out, lane);
    __syncwarp();
  }
}

// 4 + 5 for the listed bins of at most kCtaThreads * 8 keys (and more than
// the tier below): one CTA per bin. Instantiated for the medium (64 threads,
// <= 512 keys) and small (128 threads, <= 1024 keys) tiers, so that a bin's
// idle threads stay few.
template <int kCtaThreads>
__global__ void __launch_bounds__(kCtaThreads)
    bin_sort_cta_kernel(const uint64_t* __restrict__ tmp, const int2* __restrict__ list,
                        const int32_t* __restrict__ list_size, uint64_t idx_mask,
                        const uint64_t* __restrict__ keys_in, const int32_t* __restrict__ tri_in,
                        uint64_t* __restrict__ keys_out, int32_t* __restrict__ tri_out) {
  __shared__ uint64_t s[kCtaThreads * kPerThread], s2[kCtaThreads * kPerThread];
  const int count = *list_size;
  for (int l = blockIdx.x; l < count; l += gridDim.x) {
    const int2 e = list[l];
    const uint64_t* sorted = block_merge_sort<kCtaThreads>(tmp + e.x, e.y, s, s2, threadIdx.x);
    write_sorted<kCtaThreads, true>(sorted, e.y, e.x, idx_mask, keys_in, tri_in, keys_out, tri_out, threadIdx.x);
    __syncthreads();
  }
}

// Merges the sorted runs a = src[0, na) and b = src[na, na + nb) into
// dst[0, na + nb); composites are distinct, so the order is unambiguous.
// Each thread finds where its output range starts on the merge path, then
// merges sequentially.
__device__ __forceinline__ void merge_runs(const uint64_t* __restrict__ src, int64_t na, int64_t nb,
                                           uint64_t* __restrict__ dst) {
  const uint64_t* A = src;
  const uint64_t* Bv = src + na;
  const int64_t m = na + nb;
  const int64_t per = (m + kLargeThreads - 1) / kLargeThreads;
  const int64_t d0 = (int64_t)threadIdx.x * per;
  if (d0 >= m) return;
  const int64_t d1 = min(d0 + per, m);
  // i = number of A elements among the first d0 outputs.
  int64_t lo = max((int64_t)0, d0 - nb), hi = min(d0, na);
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (A[mid] < Bv[d0 - mid - 1]) lo = mid + 1;
    else hi = mid;
  }
  int64_t i = lo, j = d0 - lo;
  for (int64_t d = d0; d < d1; ++d) {
    if (j >= nb || (i < na && A[i] < Bv[j])) dst[d] = A[i++];
    else dst[d] = Bv[j++];
  }
}

// 4 + 5 for the listed bins of more than kSmallCap keys.
__global__ void __launch_bounds__(kLargeThreads)
    bin_sort_large_kernel(uint64_t* __restrict__ tmp, uint64_t* __restrict__ alt, const int2* __restrict__ list,
                          const int32_t* __restrict__ list_size, uint64_t idx_mask,
                          const uint64_t* __restrict__ keys_in, const int32_t* __restrict__ tri_in,
                          uint64_t* __restrict__ keys_out, int32_t* __restrict__ tri_out) {
  extern __shared__ uint64_t smem[];  // two buffers of kChunk entries
  uint64_t* s = smem;
  uint64_t* s2 = smem + kChunk;
  const int count = *list_size;
  for (int l = blockIdx.x; l < count; l += gridDim.x) {
    const int2 e = list[l];
    const int64_t start = e.x;
    const int64_t n = e.y;
    if (n <= kChunk) {
      const uint64_t* sorted = block_merge_sort<kLargeThreads>(tmp + start, (int)n, s, s2, threadIdx.x);
      write_sorted<kLargeThreads, true>(sorted, n, start, idx_mask, keys_in, tri_in, keys_out, tri_out, threadIdx.x);
      __syncthreads();
      continue;
    }
    uint64_t* src = tmp + start;
    uint64_t* dst = alt + start;
    for (int64_t c0 = 0; c0 < n; c0 += kChunk) {
      const int len = (int)min((int64_t)kChunk, n - c0);
      const uint64_t* sorted = block_merge_sort<kLargeThreads>(src + c0, len, s, s2, threadIdx.x);
      for (int i = threadIdx.x; i < len; i += kLargeThreads) src[c0 + i] = sorted[swz(i)];
      __syncthreads();
    }
    for (int64_t run = kChunk; run < n; run <<= 1) {
      for (int64_t p0 = 0; p0 < n; p0 += 2 * run) {
        const int64_t na = min(run, n - p0);
        const int64_t nb = min(run, n - p0 - na);
        merge_runs(src + p0, na, nb, dst + p0);
      }
      __syncthreads();
      uint64_t* t = src;
      src = dst;
      dst = t;
    }
    write_sorted<kLargeThreads, false>(src, n, start, idx_mask, keys_in, tri_in, keys_out, tri_out, threadIdx.x);
    __syncthreads();
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct TileSortWorkspace {
  int32_t* counts;   // nbins + 1 (scanned in place into offsets)
  int32_t* cursors;  // nbins
  int2* lists;       // kTiers x nbins (start, count): tiny, medium, small and large non-empty bins
  int32_t* list_sizes;  // kTiers
  uint64_t* tmp;     // K
  uint64_t* alt;     // K
  void* scan_ws;
  size_t scan_bytes;
};

size_t tile_sort_bytes(int64_t K, int64_t nbins, TileSortWorkspace* w, char* base) {
  size_t off = 256;  // bytes [0, 256): the workspace's status word (not touched but for errors)
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  char* counts = take((size_t)(nbins + 1) * sizeof(int32_t));
  char* cursors = take((size_t)nbins * sizeof(int32_t));
  char* lists = take((size_t)kTiers * nbins * sizeof(int2));
  char* list_sizes = take(kTiers * sizeof(int32_t));
  char* tmp = take((size_t)K * sizeof(uint64_t));
  char* alt = take((size_t)K * sizeof(uint64_t));
  const size_t scan_bytes = mt_scan_workspace_bytes(nbins + 1);
  char* scan = take(scan_bytes);
  if (w) {
    w->counts = reinterpret_cast<int32_t*>(counts);
    w->cursors = reinterpret_cast<int32_t*>(cursors);
    w->lists = reinterpret_cast<int2*>(lists);
    w->list_sizes = reinterpret_cast<int32_t*>(list_sizes);
    w->tmp = reinterpret_cast<uint64_t*>(tmp);
    w->alt = reinterpret_cast<uint64_t*>(alt);
    w->scan_ws = scan;
    w->scan_bytes = scan_bytes;
  }
  return off;
}

int bit_length(uint64_t x) {
  int n = 0;
  while (x) {
    ++n;
    x >>= 1;
  }
  return n;
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

size_t mt_sort_keys_by_tile_workspace_bytes(int64_t K, int64_t num_bins) {
  if (K < 0 || num_bins < 0) return 0;
  return tile_sort_bytes(K, num_bins, nullptr, nullptr);
}

int mt_sort_keys_by_tile_supported(const int32_t* layout, int32_t separate_shells, int32_t B, int64_t K) {
  if (!layout || B < 0 || K < 0) return 0;
  const int cam_off = layout[0], cam_len = layout[1], shell_off = layout[2], shell_len = layout[3];
  const int tile_off = layout[4], tile_len = layout[5], depth_off = layout[6];
  if (cam_len < 1 || cam_len > 31 || tile_len < 1 || tile_len > 31 || shell_len < 1 || shell_len > 31) return 0;
  if (cam_off + cam_len != 64) return 0;
  if (B > (1 << (cam_len - 1))) return 0;  // a set top camera bit would sort first (signed order)
  if (separate_shells) {
    // camera | shell | tile | depth
    if (depth_off != 0 || tile_off != 32 || shell_off != tile_off + tile_len || cam_off != shell_off + shell_len)
      return 0;
  } else {
    // camera | tile | depth | shell
    if (shell_off != 0 || depth_off != shell_len || tile_off != depth_off + 32 || cam_off != tile_off + tile_len)
      return 0;
  }
  const int low_bits = depth_off + 32;
  const int idx_bits = K > 1 ? bit_length((uint64_t)(K - 1)) : 1;
  return low_bits + idx_bits <= 63 ? 1 : 0;
}

}  // extern "C"

namespace {

// Helper streams and fork / join events of one (device, caller stream),
// created on first use and kept for the process: the bin tiers other than
// the tiny one sort on helper streams, concurrently with it.
struct ForkJoin {
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[3] = {nullptr, nullptr, nullptr};
};

int fork_join_for(cudaStream_t caller, ForkJoin& out) {
  static std::mutex mu;
  static std::map<std::pair<int, cudaStream_t>, ForkJoin> table;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return MT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  auto it = table.find({device, caller});
  if (it == table.end()) {
    ForkJoin f;
    if (cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming) != cudaSuccess) return MT_ERR_CUDA;
    for (int i = 0; i < 3; ++i)
      if (cudaStreamCreateWithFlags(&f.side[i], cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&f.join[i], cudaEventDisableTiming) != cudaSuccess)
        return MT_ERR_CUDA;
    it = table.emplace(std::make_pair(device, caller), f).first;
  }
  out = it->second;
  return MT_OK;
}

}  // namespace

extern "C" {

int mt_sort_keys_by_tile(const int64_t* keys, const int32_t* triangles, int64_t K, const int64_t* num_keys,
                         const int32_t* layout, int32_t separate_shells, int32_t B, int32_t shell_dim,
                         int64_t num_tiles, int64_t* sorted_keys, int32_t* sorted_triangles, int64_t* boundaries,
                         void* workspace, size_t workspace_bytes, mt_stream_t stream) {
  MT_REQUIRE(K >= 0 && B >= 0 && shell_dim >= 1 && num_tiles >= 0 && layout);
  MT_REQUIRE(mt_sort_keys_by_tile_supported(layout, separate_shells, B, K));
  MT_REQUIRE(separate_shells || shell_dim == 1);
  const int64_t nbins = (int64_t)B * shell_dim * num_tiles;
  MT_REQUIRE(nbins < (int64_t)0x7fffffff && K < (int64_t)0x7fffffff);
  cudaStream_t s = as_stream(stream);
  if (nbins > 0) {
    MT_REQUIRE(boundaries);
    if (cudaMemsetAsync(boundaries, 0, (size_t)nbins * 2 * sizeof(int64_t), s) != cudaSuccess) return MT_ERR_CUDA;
  }
  if (K == 0 || nbins == 0) return MT_OK;
  MT_REQUIRE(keys && triangles && sorted_keys && sorted_triangles && workspace);
  TileSortWorkspace w;
  MT_REQUIRE(tile_sort_bytes(K, nbins, &w, static_cast<char*>(workspace)) <= workspace_bytes);
  BinMap m{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], separate_shells ? 1 : 0, B,
           shell_dim, num_tiles};
  const int low_bits = layout[6] + 32;
  const int idx_bits = K > 1 ? bit_length((uint64_t)(K - 1)) : 1;
  const uint64_t low_mask_host = (1ull << low_bits) - 1ull;
  const uint64_t idx_mask = (1ull << idx_bits) - 1ull;
  if (cudaMemsetAsync(w.counts, 0, (size_t)(nbins + 1) * sizeof(int32_t), s) != cudaSuccess) return MT_ERR_CUDA;
  if (cudaMemsetAsync(w.cursors, 0, (size_t)nbins * sizeof(int32_t), s) != cudaSuccess) return MT_ERR_CUDA;
  if (cudaMemsetAsync(w.list_sizes, 0, kTiers * sizeof(int32_t), s) != cudaSuccess) return MT_ERR_CUDA;
  const uint64_t* k64 = reinterpret_cast<const uint64_t*>(keys);
  // A key outside every bin (never made by mt_generate_keys) is recorded in
  // the workspace status word; it is left out of the output.
  int* status = static_cast<int*>(workspace);
  bin_count_kernel<<<grid_stride_blocks(K, kThreads), kThreads, 0, s>>>(k64, K, num_keys, m, w.counts, status);
  MT_CHECK_LAUNCH();
  const int rc = mt_exclusive_scan_i32(w.counts, nbins + 1, w.scan_ws, w.scan_bytes, stream);
  if (rc != MT_OK) return rc;
  bin_bounds_kernel<<<grid_stride_blocks(nbins, kThreads), kThreads, 0, s>>>(w.counts, nbins, boundaries, w.lists,
                                                                           w.list_sizes);
  MT_CHECK_LAUNCH();
  bin_scatter_kernel<<<grid_stride_blocks(K, kThreads), kThreads, 0, s>>>(k64, K, num_keys, m, w.counts, w.cursors,
                                                                        idx_bits, low_mask_host, w.tmp);
  MT_CHECK_LAUNCH();
  // The four tiers sort concurrently (large, medium and small bins on the
  // helper streams, tiny ones on the caller's); as many CTAs as are resident
  // at once per tier, each taking listed bins in turn.
  const size_t large_smem = 2 * (size_t)kChunk * sizeof(uint64_t);
  if (set_smem<bin_sort_large_kernel>(large_smem) != MT_OK) return MT_ERR_CUDA;
  ForkJoin fj;
  if (fork_join_for(s, fj) != MT_OK) return MT_ERR_CUDA;
  if (cudaEventRecord(fj.fork, s) != cudaSuccess) return MT_ERR_CUDA;
  for (int i = 0; i < 3; ++i)
    if (cudaStreamWaitEvent(fj.side[i], fj.fork, 0) != cudaSuccess) return MT_ERR_CUDA;
  const unsigned large_ctas = (unsigned)(nbins < (int64_t)kSmCount * 2 ? nbins : (int64_t)kSmCount * 2);
  bin_sort_large_kernel<<<large_ctas, kLargeThreads, large_smem, fj.side[0]>>>(
      w.tmp, w.alt, w.lists + 3 * nbins, w.list_sizes + 3, idx_mask, k64, triangles,
      reinterpret_cast<uint64_t*>(sorted_keys), sorted_triangles);
  MT_CHECK_LAUNCH();
  const unsigned tiny_ctas = (unsigned)(nbins < (int64_t)kSmCount * 5 ? nbins : (int64_t)kSmCount * 5);
  bin_sort_tiny_kernel<<<tiny_ctas, 32 * kTinyWarps, 0, s>>>(w.tmp, w.lists, w.list_sizes, idx_mask, k64, triangles,
                                                             reinterpret_cast<uint64_t*>(sorted_keys),
                                                             sorted_triangles);
  MT_CHECK_LAUNCH();
  const unsigned medium_ctas = (unsigned)(nbins < (int64_t)kSmCount * 22 ? nbins : (int64_t)kSmCount * 22);
  bin_sort_cta_kernel<kMediumThreads><<<medium_ctas, kMediumThreads, 0, fj.side[1]>>>(
      w.tmp, w.lists + nbins, w.list_sizes + 1, idx_mask, k64, triangles, reinterpret_cast<uint64_t*>(sorted_keys),
      sorted_triangles);
  MT_CHECK_LAUNCH();
  const unsigned small_ctas = (unsigned)(nbins < (int64_t)kSmCount * 11 ? nbins : (int64_t)kSmCount * 11);
  bin_sort_cta_kernel<kSmallThreads><<<small_ctas, kSmallThreads, 0, fj.side[2]>>>(
      w.tmp, w.lists + 2 * nbins, w.list_sizes + 2, idx_mask, k64, triangles,
      reinterpret_cast<uint64_t*>(sorted_keys), sorted_triangles);
  MT_CHECK_LAUNCH();
  for (int i = 0; i < 3; ++i)
    if (cudaEventRecord(fj.join[i], fj.side[i]) != cudaSuccess || cudaStreamWaitEvent(s, fj.join[i], 0) != cudaSuccess)
      return MT_ERR_CUDA;
  return MT_OK;
}

}  // extern "C"
