// Fused multi-shell intersect + composite, forward and backward, for sm_103a.
//
// Follows triangle_rasterization/intersect_and_composite.slang:1-564. One
// thread per pixel, as in the reference, but warps are independent: persistent
// warps pull (camera, tile, warp-in-tile) work items from a device counter and
// never wait for each other:
//
//   * a pre-pass (warp_mask_kernel) gives every sorted key a bitmask of the
//     warps of its tile whose pixels the triangle can cover. Warps own compact
//     8x4 pixel blocks, and the bit is set unless the triangle's conservative
//     accept box (bary.cuh: cull_box) misses the block or one barycentric
//     numerator is provably below the fast-reject threshold at every pixel
//     centre of the block (edge exclusion), so culling changes no hit
//     decision;
//   * each warp walks its tile's key list on its own: it scans 32 masks per
//     step (one coalesced load + ballot), queues the keys that concern it,
//     and whenever 32 are queued its lanes gather those triangles (one each)
//     into the warp's private shared memory, computing the triangle-only part
//     of the barycentric solve with the same operations the per-pixel formula
//     uses (bit-identical results), then composites them in depth order;
//   * a warp stops as soon as all its pixels are done, without any CTA-wide
//     barrier.
//
// Per pixel, the three barycentric numerators reject most triangles before
// any division (bary.cuh: hit_test).
//
// The forward stores each lane's hit bits (optional hit-bit store): every
// work item counts the keys its warp will walk, reserves exactly that many
// batches (a bump allocator) and writes one 32-word line per batch while the
// store's capacity lasts; the backward re-walks the same way, reads those
// bits instead of testing again (gathering only the triangles some pixel
// hits), re-solves each hit's barycentrics and applies the suffix trick of
// the reference. Batches past the capacity are tested again. Per-triangle gradient sums live in a per-warp ring
// of 64 shared-memory slots (the current and the previous batch); a slot is
// flushed to global memory with one atomic per non-zero scalar when its batch
// retires, and gradients for older triangles go to global memory directly.
// Two routings:
//   reference (exact_adjoint = 0): the deferred gradient of the previous
//     (outer) hit is scattered to the previous triangle's vertices with the
//     *current* hit's barycentric weights (intersect_and_composite.slang:
//     487-509), as the reference does;
//   exact (exact_adjoint = 1): with the previous hit's own weights.
// The sharpness gradient is warp-reduced before one global atomic per warp.

#include <atomic>
#include <type_traits>

#include "bary.cuh"
#include "mt_common.cuh"

namespace mt {
namespace {

constexpr int kBatch = 32;   // triangles gathered per warp batch
constexpr int kQueue = 64;   // queued key offsets per warp
constexpr int kRing = 64;    // gradient slots per warp (two batches)
constexpr int kSavedFwd = 2;  // hits per pixel per batch whose samples the test phase keeps (forward)
constexpr int kSavedBwd = 3;  // same, backward (its shared memory is tighter)
// Hit-bit store (bytes): [0, 8) batch allocator, [8, 8 + 4 items) first
// stored batch of each work item (int32, -1 = none), then from a 128-byte
// boundary `capacity` batches of 32 words (one per lane).
struct HitStore {
  unsigned long long* next;
  int32_t* item_base;
  uint32_t* batches;  // NULL: no store
  int64_t capacity;
};

__host__ __device__ constexpr size_t hit_store_header(int64_t items) {
  return ((size_t)(8 + 4 * items) + 127) / 128 * 128;
}

// The (u, v, w) of the first K hits each lane finds in a batch, so that the
// hit phase does not solve them again (later hits are re-solved).
template <int K>
struct SavedHits {
  float u[K][32], v[K][32], w[K][32];
};

struct alignas(16) TriAttr {
  float ca[3], cb[3], cc[3];
  float sa, sb, sc;
};

// The samples of up to K hits per pixel of a batch (the interpolated
// signed distance's CDF and the interpolated colour), tagged with their
// triangle: the forward's test phase solves pairs in dealt order, so a
// pixel's hits arrive in no particular order. They depend on the hit alone,
// not on the pixel's compositing state, so the lanes that solve the hits
// compute them (all lanes busy) and the per-pixel compositing loop only
// blends them.
template <int K>
struct TaggedSamples {
  int tri[K][32];
  float cdf[K][32];
  float rgb[3][K][32];
};

// A (pixel, triangle) pair of the forward's test phase whose numerators
// passed the fast reject; its divisions and acceptance test are pending.
struct alignas(16) Candidate {
  int id;  // pixel lane | triangle << 5
  float un, vn, wn;
};
constexpr int kCandRing = 64;  // ring of pending candidates per warp (solved 32 at a time)

struct CompositeArgs {
  const float* xy;      // [B, V, 2]
  const float* colors;  // [B, V, 3]
  const float* sdf;     // [V]
  int64_t V;
  const int32_t* faces;  // [F, 3]
  const float* sharpness;
  const uint64_t* keys;   // sorted keys
  const int32_t* tri;     // sorted triangle indices
  const int64_t* bounds;  // [B, rows * cols, 2]
  int B, S, rows, cols, tile_h, tile_w, H, W;
  int shell_off, shell_len, cam_off, cam_len, tile_off, tile_len;
  const float* out;  // forward output (input to backward)
  // Ragged cameras: NULL (every camera rows x cols tiles, H x W pixels, output
  // [B, 4, H, W]) or a device table [B, 6] = (rows, cols, height, width,
  // first tile, first output element): each camera's output is [4, h, w] at
  // its first output element and its tiles follow its first tile in the work
  // order. rows / cols / H / W are then the maxima over cameras.
  const int64_t* cameras;
  int64_t total_tiles;  // tiles over all cameras
  // Optional MSE epilogue (target NULL: none). The image is
  // clip(rgb + T * background, 0, 1) as the render entry points form it; the
  // target holds each camera's [3, h, w] at 3/4 of its first output element;
  // the loss is loss_scale x the sum of squared errors.
  const float* target;
  const float* background;
  float loss_scale;
  // SSAA factor of the epilogue's backward (1: none). With ssaa > 1 the
  // backward's `target` is the per-output-pixel factor written by
  // ssaa_loss_kernel, [B, 3, H / ssaa, W / ssaa].
  int ssaa;
};

struct CompositeGrads {
  const float* grad_loss;  // with the epilogue: d L / d loss (device scalar)
  const float* grad_out;  // [B, 4, H, W]
  float* grad_colors;     // [B, V, 3]
  float* grad_sdf;        // [V]
  float* grad_sharpness;  // [1]
  int exact;
};

// ---------------------------------------------------------------------------
// Bulk-copy staging of the backward's triangles. Each (camera, vertex) is one
// 32-byte record (x, y, r, g, b, signed distance, 0, 0) in a packed array;
// while a warp composites one batch, the three records of every triangle of
// its next batch are on their way into the warp's shared memory through
// cp.async.bulk (one 32-byte copy per vertex), completing on the warp's
// mbarrier. The waits are bounded: a wait that gives up records
// MT_ERR_DEVICE_TIMEOUT and the warp stops.
// ---------------------------------------------------------------------------
struct alignas(16) VertexRecord {
  float x, y, r, g, b, sdf, pad0, pad1;
};
constexpr int kWaitPolls = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test_wait(unsigned long long* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of parity `parity`; false when it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
  for (int i = 0; i < kWaitPolls; ++i) {
    if (mbar_test_wait(bar, parity)) return true;
    __nanosleep(20);
  }
  return false;
}

__device__ __forceinline__ void bulk_copy_to_shared(void* dst, const void* src, uint32_t bytes,
                                                    unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Per-warp shared-memory region.
struct WarpForward {
  TriGeom geo[kBatch];
  TriAttr attr[kBatch];
  TaggedSamples<kSavedFwd> saved;
  Candidate cand[kCandRing];
  uint32_t hitw[32];  // per pixel: bit i = triangle i of the batch is a hit
  int nsaved[32];     // per pixel: hits solved in the batch (the first kSavedFwd are kept)
  int queue[kQueue];
  uint8_t owner[32];  // test phase: triangle whose pairs start at each position of the current 32
};

struct WarpBackward {
  TriGeom geo[kBatch];
  TriAttr attr[kBatch];
  SavedHits<kSavedBwd> saved;
  int3 vids[kRing];
  float gslot[kRing][13];  // 12 used; stride 13 keeps lanes on distinct banks
  int queue[kQueue];
};

// The staged backward's region: the same, plus the next batch's vertex
// records and their mbarrier.
struct WarpBackwardStaged : WarpBackward {
  VertexRecord stage[kBatch][3];
  unsigned long long bar;
  unsigned long long pad;
};

struct Staging {
  const VertexRecord* records;  // [B, V] (NULL: no staging)
  int* status;                  // device status word
};

__device__ __forceinline__ uint64_t field(uint64_t key, int off, int len) {
  return (key >> off) & (uint64_t)((1u << len) - 1u);
}

// Pixel rectangle (pixel centres) of warp `w` inside tile (tx, ty); matches
// tile_pixel().
__device__ __forceinline__ void warp_block_rect(int w, int tile_w, int tile_h, int tx, int ty, float& x0, float& x1,
                                                float& y0, float& y1) {
  int lx0, lx1, ly0, ly1;
  if ((tile_w & 7) == 0 && (tile_h & 3) == 0) {
    const int per_row = tile_w >> 3;
    lx0 = (w % per_row) * 8;
    lx1 = lx0 + 7;
    ly0 = (w / per_row) * 4;
    ly1 = ly0 + 3;
  } else {
    const int numel = tile_w * tile_h;
    const int t0 = 32 * w, t1 = min(32 * w + 31, numel - 1);
    ly0 = t0 / tile_w;
    ly1 = t1 / tile_w;
    if (ly0 == ly1) {
      lx0 = t0 % tile_w;
      lx1 = t1 % tile_w;
    } else {
      lx0 = 0;
      lx1 = tile_w - 1;
    }
  }
  x0 = (float)(tx * tile_w + lx0) + 0.5f;
  x1 = (float)(tx * tile_w + lx1) + 0.5f;
  y0 = (float)(ty * tile_h + ly0) + 0.5f;
  y1 = (float)(ty * tile_h + ly1) + 0.5f;
}

// Exact block exclusion by the barycentric numerators. hit_test computes
// each numerator N(p) = A (q . eX) - C (q . eY), q = p - P, in single
// precision and rejects p when N(p) < thr. The exact value is affine in p,
// N(p) = a qx + b qy with a = A eXx - C eYx, b = A eXy - C eYy, and the
// single-precision evaluation errs by at most 5 u S(p), u = 2^-24, with
// S(p) = |qx| sx + |qy| sy, sx = |A eXx| + |C eYx|, sy = |A eXy| + |C eYy|.
// Over the rectangle of pixel centres [x0, x1] x [y0, y1] the affine part and
// S are largest at corners and separate in x and y, so with E = 32 u (room
// for the rounding of a, b, sx, sy and of this evaluation, at most 10 u S):
//   max_x (a qx + E sx |qx|) + max_y (b qy + E sy |qy|) + E max S < thr
// means every pixel centre of the rectangle is rejected by hit_test.
// Non-finite values compare false: no exclusion.
struct EdgeBound {
  float a, b, sx, sy, px, py;
};

__device__ __forceinline__ EdgeBound edge_bound(float A, float C, float Px, float Py, float eXx, float eXy,
                                                float eYx, float eYy) {
  return EdgeBound{A * eXx - C * eYx, A * eXy - C * eYy, fabsf(A * eXx) + fabsf(C * eYx),
                   fabsf(A * eXy) + fabsf(C * eYy), Px, Py};
}

__device__ __forceinline__ bool edge_excludes(const EdgeBound& e, float thr, float x0, float x1, float y0,
                                              float y1) {
  constexpr float kErr = 0x1p-19f;  // 32 u
  const float qx0 = x0 - e.px, qx1 = x1 - e.px, qy0 = y0 - e.py, qy1 = y1 - e.py;
  const float tx = fmaxf(e.a * qx0 + kErr * e.sx * fabsf(qx0), e.a * qx1 + kErr * e.sx * fabsf(qx1));
  const float ty = fmaxf(e.b * qy0 + kErr * e.sy * fabsf(qy0), e.b * qy1 + kErr * e.sy * fabsf(qy1));
  const float bm = kErr * (e.sx * fmaxf(fabsf(qx0), fabsf(qx1)) + e.sy * fmaxf(fabsf(qy0), fabsf(qy1)));
  return tx + ty + bm < thr;
}

// The three numerator bounds of a staged triangle (vn and wn from corner 1,
// un from corner 2, as hit_test forms them).
struct TriangleBounds3 {
  EdgeBound v, w, u;
};

__device__ __forceinline__ TriangleBounds3 triangle_bounds(const TriGeom& g) {
  return TriangleBounds3{edge_bound(g.d1313, g.d1213, g.p1x, g.p1y, g.e12x, g.e12y, g.e13x, g.e13y),
                         edge_bound(g.d1212, g.d1213, g.p1x, g.p1y, g.e13x, g.e13y, g.e12x, g.e12y),
                         edge_bound(g.d1223, g.d1323, g.p2x, g.p2y, g.e13x, g.e13y, g.e12x, g.e12y)};
}

// The warp blocks of its tile that a key's triangle (corners pa, pb, pc) may
// cover: bit w = warp w.
__device__ __forceinline__ uint32_t key_mask(const CompositeArgs& a, int warps, int tile, int cols_b, float2 pa,
                                             float2 pb, float2 pc) {
  TriGeom g;
  setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, g);
  const CullBox box = cull_box(g, pa.x, pa.y, pb.x, pb.y, pc.x, pc.y);
  const int tx = tile % cols_b, ty = tile / cols_b;
  // Exclusion needs the fast reject, finite coordinates and a
  // well-conditioned triangle: exactly the triangles with a finite box.
  const bool exact_cull = box.x0 > -__int_as_float(0x7f800000);
  const TriangleBounds3 tb = triangle_bounds(g);
  uint32_t m = 0;
  for (int w = 0; w < warps; ++w) {
    float x0, x1, y0, y1;
    warp_block_rect(w, a.tile_w, a.tile_h, tx, ty, x0, x1, y0, y1);
    if (!box_overlaps(box, x0, x1, y0, y1)) continue;
    if (exact_cull && (edge_excludes(tb.v, g.thr, x0, x1, y0, y1) || edge_excludes(tb.w, g.thr, x0, x1, y0, y1) ||
                       edge_excludes(tb.u, g.thr, x0, x1, y0, y1)))
      continue;
    m |= 1u << w;
  }
  return m;
}

// One mask per sorted key: bit w = warp w of the key's tile may be covered.
// Keys past num_keys (a device value; all K when NULL) get no mask: no tile
// range reaches them. Each thread takes two keys and issues their dependent
// loads (key and triangle, face, projected corners) side by side.
__global__ void warp_mask_kernel(CompositeArgs a, int64_t K_capacity, const int64_t* __restrict__ num_keys,
                                 uint32_t* __restrict__ masks) {
  const int warps = (a.tile_h * a.tile_w + 31) / 32;
  const int64_t K = num_keys ? min(max(*num_keys, (int64_t)0), K_capacity) : K_capacity;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k0 < K; k0 += 2 * stride) {
    const int64_t kk[2] = {k0, k0 + stride};
    int32_t f[2];
    int cam[2], tile[2], cols_b[2];
    bool ok[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const bool in = kk[j] < K;
      const uint64_t key = in ? __ldg(reinterpret_cast<const unsigned long long*>(a.keys) + kk[j]) : 0ull;
      f[j] = in ? __ldg(a.tri + kk[j]) : 0;
      cam[j] = (int)field(key, a.cam_off, a.cam_len);
      tile[j] = (int)field(key, a.tile_off, a.tile_len);
      cols_b[j] = (a.cameras && cam[j] < a.B) ? (int)__ldg(a.cameras + 6 * cam[j] + 1) : a.cols;
      const int rows_b = (a.cameras && cam[j] < a.B) ? (int)__ldg(a.cameras + 6 * cam[j]) : a.rows;
      ok[j] = in && cam[j] < a.B && tile[j] < rows_b * cols_b[j];
    }
    int32_t ids[2][3];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int q = 0; q < 3; ++q) ids[j][q] = ok[j] ? __ldg(a.faces + 3 * (int64_t)f[j] + q) : 0;
    float2 p[2][3];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float2* xy = reinterpret_cast<const float2*>(a.xy) + (int64_t)(ok[j] ? cam[j] : 0) * a.V;
#pragma unroll
      for (int q = 0; q < 3; ++q) p[j][q] = ok[j] ? __ldg(xy + ids[j][q]) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j)
      if (kk[j] < K) masks[kk[j]] = ok[j] ? key_mask(a, warps, tile[j], cols_b[j], p[j][0], p[j][1], p[j][2]) : 0u;
  }
}

// A sorted key's triangle: its vertex ids and its shell.
struct TriRef {
  int32_t ia, ib, ic;
  int shell;
};

// Sorted key k -> its face -> the face's vertex ids (two levels of dependent
// loads).
__device__ __forceinline__ TriRef locate(const CompositeArgs& a, int64_t k) {
  const int32_t f = __ldg(a.tri + k);
  const uint64_t key = __ldg(reinterpret_cast<const unsigned long long*>(a.keys) + k);
  return TriRef{__ldg(a.faces + 3 * (int64_t)f), __ldg(a.faces + 3 * (int64_t)f + 1),
                __ldg(a.faces + 3 * (int64_t)f + 2), (int)field(key, a.shell_off, a.shell_len)};
}

// Stages a located triangle into batch slot `slot` (its projected corners
// into `corners` when given): geometry and per-vertex colours and signed
// distances.
__device__ __forceinline__ void fetch(const CompositeArgs& a, int cam, const TriRef& r, TriGeom* geo, TriAttr* attr,
                                      int slot, float2* corners = nullptr) {
  const float2* xy = reinterpret_cast<const float2*>(a.xy) + (int64_t)cam * a.V;
  const float2 pa = __ldg(xy + r.ia), pb = __ldg(xy + r.ib), pc = __ldg(xy + r.ic);
  TriGeom g;
  setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, g);
  g.shell = r.shell;
  geo[slot] = g;
  if (corners) {
    corners[0] = pa;
    corners[1] = pb;
    corners[2] = pc;
  }
  const float* col = a.colors + (int64_t)cam * a.V * 3;
  TriAttr t;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    t.ca[c] = __ldg(col + 3 * (int64_t)r.ia + c);
    t.cb[c] = __ldg(col + 3 * (int64_t)r.ib + c);
    t.cc[c] = __ldg(col + 3 * (int64_t)r.ic + c);
  }
  t.sa = __ldg(a.sdf + r.ia);
  t.sb = __ldg(a.sdf + r.ib);
  t.sc = __ldg(a.sdf + r.ic);
  attr[slot] = t;
}

// Gathers triangle `k` of the sorted list into batch slot `slot`; returns its
// vertex ids.
__device__ __forceinline__ int3 gather(const CompositeArgs& a, int cam, int64_t k, TriGeom* geo, TriAttr* attr,
                                       int slot) {
  const int32_t f = __ldg(a.tri + k);
  const uint64_t key = __ldg(reinterpret_cast<const unsigned long long*>(a.keys) + k);
  const int32_t ia = __ldg(a.faces + 3 * (int64_t)f), ib = __ldg(a.faces + 3 * (int64_t)f + 1),
                ic = __ldg(a.faces + 3 * (int64_t)f + 2);
  const float2* xy = reinterpret_cast<const float2*>(a.xy) + (int64_t)cam * a.V;
  const float2 pa = __ldg(xy + ia), pb = __ldg(xy + ib), pc = __ldg(xy + ic);
  TriGeom g;
  setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, g);
  g.shell = (int)field(key, a.shell_off, a.shell_len);
  geo[slot] = g;
  const float* col = a.colors + (int64_t)cam * a.V * 3;
  TriAttr t;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    t.ca[c] = __ldg(col + 3 * (int64_t)ia + c);
    t.cb[c] = __ldg(col + 3 * (int64_t)ib + c);
    t.cc[c] = __ldg(col + 3 * (int64_t)ic + c);
  }
  t.sa = __ldg(a.sdf + ia);
  t.sb = __ldg(a.sdf + ib);
  t.sc = __ldg(a.sdf + ic);
  attr[slot] = t;
  return make_int3(ia, ib, ic);
}

// Fills the warp's queue with offsets (relative to `start`) of keys whose
// mask has this warp's bit, until 32 are queued or the list ends. Returns the
// number queued; `next` advances through the list 32 keys at a time.
__device__ __forceinline__ int refill(const uint32_t* __restrict__ masks, int64_t start, int64_t end, int64_t& next,
                                      int queued, int* queue, int warp, int lane) {
  const uint32_t lt = lanemask_lt();
  while (queued < kBatch && next < end) {
    const int64_t k = next + lane;
    const bool keep = k < end && ((__ldg(masks + k) >> warp) & 1u);
    const uint32_t sel = __ballot_sync(0xffffffffu, keep);
    if (keep) queue[queued + __popc(sel & lt)] = (int)(k - start);
    queued += __popc(sel);
    next += 32;
  }
  __syncwarp();
  return queued;
}

// Drops the first `nb` queue entries.
__device__ __forceinline__ void pop(int* queue, int queued, int nb, int lane) {
  const int rest = queued - nb;  // <= 31
  const int v = lane < rest ? queue[nb + lane] : 0;
  __syncwarp();
  if (lane < rest) queue[lane] = v;
  __syncwarp();
}

// Test phase of a batch: bit i = triangle i of the batch passes the exact
// hit test at this pixel. Triangles of shells the pixel has already passed
// are skipped (last_shell only grows, so they would be skipped later too).
// The costly per-hit work then runs in a separate loop over each pixel's own
// bits, so the warp executes it as often as its busiest pixel has hits, not
// once for every triangle that any of its pixels hits. The (u, v, w) of the
// lane's first K hits are kept for that loop.
template <int K>
__device__ __forceinline__ uint32_t batch_hits(const TriGeom* geo, int nb, float fx, float fy, int last_shell,
                                               SavedHits<K>& saved, int lane) {
  uint32_t hits = 0;
  int n = 0;
#pragma unroll 2  // two independent tests in flight
  for (int i = 0; i < nb; ++i) {
    const TriGeom& g = geo[i];
    if (g.shell <= last_shell) continue;
    float u, v, w;
    if (hit_test(g, fx, fy, u, v, w)) {
      hits |= 1u << i;
      if (n < K) {
        saved.u[n][lane] = u;
        saved.v[n][lane] = v;
        saved.w[n][lane] = w;
      }
      ++n;
    }
  }
  return hits;
}

// ---------------------------------------------------------------------------
// The forward's test phase, dealt over (pixel, triangle) pairs.
//
// A staged triangle can only be accepted at pixel centres inside its
// conservative accept box (bary.cuh: cull_box; outside it the fast reject
// fires). Its span is the set of the warp's pixels whose centres lie in that
// box that no barycentric numerator provably rejects (edge_span): with 8x4
// warp blocks, up to 4 rows of consecutive columns, one byte per row (first
// column | count << 3); for other tile shapes every pixel of the warp (4
// "rows" of 8 lanes). The pairs of all spans of a batch are numbered
// triangle by triangle and dealt 32 at a time, one per lane, so that the warp
// evaluates the barycentric numerators only where a hit is possible instead
// of every lane testing every staged triangle.
// ---------------------------------------------------------------------------
constexpr uint32_t kFullSpan = 0x40404040u;  // 4 rows, columns 0..7

__device__ __forceinline__ uint32_t span_row(uint32_t span, int r) { return (span >> (8 * r)) & 0xffu; }

__device__ __forceinline__ int span_count(uint32_t span) {
  return (int)(((span >> 3) & 15u) + ((span >> 11) & 15u) + ((span >> 19) & 15u) + ((span >> 27) & 15u));
}

// Span of a staged triangle over the 8x4 block whose first pixel centre is
// (bx, by), row by row: the columns of a row inside the accept box that none
// of the three barycentric numerators provably rejects. edge_excludes applied
// to a single pixel centre p says that numerator j rejects p when
//   a qx + b qy + 2E (sx |qx| + sy |qy|) < thr,  q = p - P_j.
// On a row (qy fixed) this reads g(qx) = a qx + 2E sx |qx| < R with
// R = thr - b qy - 2E sy |qy|. When |a| > 2E sx, g is monotonic, so the
// columns that survive form a ray bounded at the root of g(qx) = R (on the
// side of zero that the sign of R selects), which is widened here by a
// padding far above the rounding of this computation. Otherwise (an edge
// within a few ulps of horizontal) g <= 4E sx |qx|, and the edge removes the
// whole row when that bound stays below R at the row's farthest column.
// Triangles without an exact fast reject (open accept box) span every pixel.
__device__ __forceinline__ uint32_t edge_span(const TriGeom& g, const CullBox& box, float bx, float by) {
  if (!(box.x0 > -__int_as_float(0x7f800000))) return kFullSpan;
  constexpr float k2E = 0x1p-18f;  // 2 x 32 u, as in edge_excludes for one point
  const TriangleBounds3 tb = triangle_bounds(g);
  const EdgeBound eb[3] = {tb.v, tb.w, tb.u};
  float slack[3], inv_lo[3], inv_hi[3];  // 2E sx, 1 / (a - 2E sx), 1 / (a + 2E sx)
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    slack[j] = k2E * eb[j].sx;
    inv_lo[j] = __frcp_rn(eb[j].a - slack[j]);
    inv_hi[j] = __frcp_rn(eb[j].a + slack[j]);
  }
  uint32_t span = 0u;
#pragma unroll 1  // rolled: the unrolled rows cost more in instruction-cache misses than they save
  for (int r = 0; r < 4; ++r) {
    const float y = by + (float)r;
    if (!(y >= box.y0 && y <= box.y1)) continue;
    float xl = box.x0, xu = box.x1;
    bool empty = false;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const EdgeBound& e = eb[j];
      const float qy = y - e.py;
      const float R = g.thr - (e.b * qy + k2E * e.sy * fabsf(qy));
      if (e.a > slack[j]) {  // g increasing: columns at or right of the root survive
        const float q = R * (R <= 0.0f ? inv_lo[j] : inv_hi[j]);
        xl = fmaxf(xl, e.px + q - (0.0625f + 0x1p-16f * (fabsf(e.px) + fabsf(q))));
      } else if (e.a < -slack[j]) {  // g decreasing: columns at or left of the root survive
        const float q = R * (R <= 0.0f ? inv_hi[j] : inv_lo[j]);
        xu = fminf(xu, e.px + q + (0.0625f + 0x1p-16f * (fabsf(e.px) + fabsf(q))));
      } else {
        const float qf = fmaxf(fabsf(bx - e.px), fabsf(bx + 7.0f - e.px));
        empty = empty || 2.02f * slack[j] * qf < R;
      }
    }
    if (empty) continue;
    const int c0 = max((int)ceilf(fmaxf(xl - bx, -1.0f)), 0);
    const int c1 = min((int)floorf(fminf(xu - bx, 8.0f)), 7);
    if (c0 <= c1) span |= ((uint32_t)c0 | ((uint32_t)(c1 - c0 + 1) << 3)) << (8 * r);
  }
  return span;
}

// Pixel lane of pair k (< span_count) of a span.
__device__ __forceinline__ int span_pixel(uint32_t span, int k) {
  const int n0 = (int)((span >> 3) & 15u), n1 = (int)((span >> 11) & 15u), n2 = (int)((span >> 19) & 15u);
  const int t1 = n0, t2 = n0 + n1, t3 = n0 + n1 + n2;
  const int row = (k >= t1) + (k >= t2) + (k >= t3);
  const int before = row == 0 ? 0 : row == 1 ? t1 : row == 2 ? t2 : t3;
  return 8 * row + (int)(span_row(span, row) & 7u) + (k - before);
}

// Solves `count` (<= 32) pending candidates starting at ring position
// `head`, one per lane: the divisions and the acceptance test of hit_test. An
// accepted candidate sets its triangle's bit in its pixel's hit word and, if
// it is among the first kSavedFwd hits solved for that pixel, keeps its
// samples (sample_of) tagged with the triangle.
__device__ __forceinline__ void sample_of(const TriAttr& t, float u, float v, float w, float s, float& cdf,
                                          float (&rgb)[3]) {
  float e;
  cdf = sdf_to_cdf(interp(u, v, w, t.sa, t.sb, t.sc), s, e);
#pragma unroll
  for (int c = 0; c < 3; ++c) rgb[c] = interp(u, v, w, t.ca[c], t.cb[c], t.cc[c]);
}

__device__ __forceinline__ void solve_candidates(WarpForward& ws, int head, int count, float s, int lane) {
  if (lane < count) {
    const Candidate c = ws.cand[(head + lane) & (kCandRing - 1)];
    const int pl = c.id & 31, i = c.id >> 5;
    float u, v, w;
    if (solve_and_accept(c.un, c.vn, c.wn, ws.geo[i].dd, u, v, w)) {
      atomicOr(&ws.hitw[pl], 1u << i);
      const int n = atomicAdd(&ws.nsaved[pl], 1);
      if (n < kSavedFwd) {
        float cdf, rgb[3];
        sample_of(ws.attr[i], u, v, w, s, cdf, rgb);
        ws.saved.tri[n][pl] = i;
        ws.saved.cdf[n][pl] = cdf;
#pragma unroll
        for (int k = 0; k < 3; ++k) ws.saved.rgb[k][n][pl] = rgb[k];
      }
    }
  }
}

// Test phase of a batch. `span` is the span of the lane's staged triangle (0
// for lanes at or past the batch); `blocked`: 8x4 warp blocks, whose first
// pixel centre is (bx, by); s: the sharpness. Returns the pixel's hit bits: bit i = triangle i
// passes the exact hit test (hit_test's decision) and its shell is above
// `last_shell`; pixels that are not active have none.
__device__ __forceinline__ uint32_t span_batch_hits(WarpForward& ws, uint32_t span, bool blocked, float bx, float by,
                                                    float fx, float fy, int last_shell, bool active, float s,
                                                    int lane) {
  const uint32_t lt = lanemask_lt();
  ws.hitw[lane] = 0u;
  ws.nsaved[lane] = 0;
  // Pairs before this lane's triangle (exclusive scan of the span sizes);
  // lanes past the batch have no pairs, so their offset is the total.
  const int cnt = span_count(span);
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const int total = __shfl_sync(0xffffffffu, inc, 31);
  const int off = inc - cnt;
  const int ls = active ? last_shell : 0x7fffffff;  // an inactive pixel passes nothing
  int head = 0, tail = 0;
  for (int base = 0; base < total; base += 32) {
    // Each triangle with pairs among [base, base + 32) marks where its first
    // one there falls; the pair's triangle is the last mark at or before it.
    const bool here = cnt > 0 && off < base + 32 && off + cnt > base;
    const int first = max(off, base) - base;
    __syncwarp();
    if (here) ws.owner[first] = (uint8_t)lane;
    const uint32_t starts = __reduce_or_sync(0xffffffffu, here ? 1u << first : 0u);
    __syncwarp();
    const int i = ws.owner[31 - __clz(starts & (0xffffffffu >> (31 - lane)))];
    const int q = base + lane;
    const int p = span_pixel(__shfl_sync(0xffffffffu, span, i), q - __shfl_sync(0xffffffffu, off, i)) & 31;
    const float qx = __shfl_sync(0xffffffffu, fx, p), qy = __shfl_sync(0xffffffffu, fy, p);
    const float px = blocked ? bx + (float)(p & 7) : qx, py = blocked ? by + (float)(p >> 3) : qy;
    const int pls = __shfl_sync(0xffffffffu, ls, p);
    bool pass = false;
    float un = 0.f, vn = 0.f, wn = 0.f;
    if (q < total) {
      const TriGeom g = load_geom(&ws.geo[i]);
      numerators(g, px, py, un, vn, wn);
      pass = g.shell > pls && numerators_pass(g, un, vn, wn);
    }
    const uint32_t m = __ballot_sync(0xffffffffu, pass);
    if (pass) ws.cand[(tail + __popc(m & lt)) & (kCandRing - 1)] = Candidate{p | (i << 5), un, vn, wn};
    tail += __popc(m);
    if (tail - head >= 32) {  // at most 63 pending: one round empties below 32
      __syncwarp();
      solve_candidates(ws, head, 32, s, lane);
      head += 32;
      __syncwarp();
    }
  }
  if (tail > head) {
    __syncwarp();
    solve_candidates(ws, head, tail - head, s, lane);
  }
  __syncwarp();
  return ws.hitw[lane];
}

// Samples of the pixel's hit on triangle i (g) of the batch: kept by the
// forward's test phase (ns tagged entries), or formed again.
__device__ __forceinline__ void hit_samples(const WarpForward& ws, int ns, int i, int lane, const TriGeom& g,
                                            float fx, float fy, float s, float& cdf, float (&rgb)[3]) {
  int slot = -1;
#pragma unroll
  for (int n = 0; n < kSavedFwd; ++n)
    if (n < ns && ws.saved.tri[n][lane] == i) slot = n;
  if (slot >= 0) {
    cdf = ws.saved.cdf[slot][lane];
#pragma unroll
    for (int k = 0; k < 3; ++k) rgb[k] = ws.saved.rgb[k][slot][lane];
  } else {
    float u, v, w;
    hit_test(g, fx, fy, u, v, w);
    sample_of(ws.attr[i], u, v, w, s, cdf, rgb);
  }
}

// (u, v, w) of the lane's n-th hit in the batch (triangle g): kept by the
// backward's test phase, or solved again.
template <int K>
__device__ __forceinline__ void hit_weights(const SavedHits<K>& saved, int n, int lane, const TriGeom& g, float fx,
                                            float fy, float& u, float& v, float& w) {
  if (n < K) {
    u = saved.u[n][lane];
    v = saved.v[n][lane];
    w = saved.w[n][lane];
  } else {
    hit_test(g, fx, fy, u, v, w);
  }
}

struct Pixel {
  int cam;
  int64_t tile;     // tile inside its camera's grid
  int px, py;       // pixel inside its camera's image
  bool in_image;
  float fx, fy;
  int wt;           // warp index inside its tile
  int64_t out_base;  // first output element of the camera
  int64_t plane;     // pixels per output channel of the camera
  int width;         // image width of the camera
};

// Work is a list of (camera, tile, warp-in-tile) items, warp-in-tile
// fastest, cameras in order; warps are independent, so CTAs are containers of
// 4, 8 or 16 warps (the caller's choice: 128, 256 or 512 threads per CTA,
// where the reference runs one tile of TILE_H x TILE_W threads per CTA) that
// each pull items from a device counter until the list is exhausted
// (persistent warps: any camera sizes and tile loads in one launch).
constexpr int kDefaultWarpsPerCta = 8;

__device__ __forceinline__ int tile_warps(const CompositeArgs& a) { return (a.tile_h * a.tile_w + 31) / 32; }

__device__ __forceinline__ int64_t total_items(const CompositeArgs& a) { return a.total_tiles * tile_warps(a); }

__device__ __forceinline__ Pixel pixel_of(const CompositeArgs& a, int64_t item) {
  Pixel p;
  const int tw = tile_warps(a);
  const int64_t gt = item / tw;  // global tile
  p.wt = (int)(item - gt * tw);
  int rows_b = a.rows, cols_b = a.cols, h = a.H, w = a.W;
  if (a.cameras == nullptr) {
    const int64_t T = (int64_t)a.rows * a.cols;
    p.cam = (int)(gt / T);
    p.tile = gt - (int64_t)p.cam * T;
    p.plane = (int64_t)a.H * a.W;
    p.out_base = (int64_t)p.cam * 4 * p.plane;
  } else {
    int lo = 0, hi = a.B - 1;  // last camera whose first tile <= gt
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(a.cameras + 6 * mid + 4) <= gt) lo = mid; else hi = mid - 1;
    }
    const int64_t* c = a.cameras + 6 * lo;
    p.cam = lo;
    rows_b = (int)__ldg(c);
    cols_b = (int)__ldg(c + 1);
    h = (int)__ldg(c + 2);
    w = (int)__ldg(c + 3);
    p.tile = gt - __ldg(c + 4);
    p.plane = (int64_t)h * w;
    p.out_base = __ldg(c + 5);
  }
  (void)rows_b;
  p.width = w;
  const int tid = p.wt * 32 + (threadIdx.x & 31);  // thread index inside the tile
  int lx = 0, ly = 0;
  tile_pixel(tid, a.tile_w, a.tile_h, lx, ly);
  p.px = (int)(p.tile % cols_b) * a.tile_w + lx;
  p.py = (int)(p.tile / cols_b) * a.tile_h + ly;
  p.in_image = tid < a.tile_h * a.tile_w && p.px < w && p.py < h;
  p.fx = (float)p.px + 0.5f;
  p.fy = (float)p.py + 0.5f;
  return p;
}

// Next work item for the calling warp (lane 0 claims, the warp shares it).
__device__ __forceinline__ int64_t next_item(unsigned long long* counter, int lane) {
  unsigned long long item = 0;
  if (lane == 0) item = atomicAdd(counter, 1ull);
  return (int64_t)__shfl_sync(0xffffffffu, item, 0);
}

// ---------------------------------------------------------------------------
// Longest-first order of the work. A work item's cost grows with its tile's
// key count, and a few tiles (silhouettes, overlapping objects) hold many
// times the mean; handed out in launch order they start last and the launch
// waits on them. The tile order sorts the tiles (over all cameras) by
// descending key count, in buckets of 8 keys (a counting sort: histogram,
// then a scatter at each bucket's offset), and the persistent warps claim
// the tiles' items in that order (the warps of a tile consecutively). Only
// the processing order changes: every item computes what it computed before.
//
// Buffer (int32): [0, 256) bucket sizes, [256, 512) bucket cursors, then one
// global tile index per tile.
// ---------------------------------------------------------------------------
constexpr int kOrderBuckets = 256;
constexpr int kOrderHeader = 2 * kOrderBuckets;

__device__ __forceinline__ int order_bucket(const CompositeArgs& a, int64_t gt) {
  int64_t bi = gt;  // index of the tile's range in `bounds`
  if (a.cameras != nullptr) {
    int lo = 0, hi = a.B - 1;  // last camera whose first tile <= gt
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(a.cameras + 6 * mid + 4) <= gt) lo = mid; else hi = mid - 1;
    }
    bi = (int64_t)lo * a.rows * a.cols + (gt - __ldg(a.cameras + 6 * lo + 4));
  }
  const int64_t keys = __ldg(a.bounds + 2 * bi + 1) - __ldg(a.bounds + 2 * bi);
  if (keys <= 0) return kOrderBuckets - 1;  // the last bucket holds exactly the tiles without keys
  return kOrderBuckets - 2 - (int)min((keys - 1) >> 3, (int64_t)(kOrderBuckets - 2));
}

__global__ void order_histogram_kernel(CompositeArgs a, int32_t* __restrict__ order) {
  __shared__ int hist[kOrderBuckets];
  for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gt < a.total_tiles;
       gt += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[order_bucket(a, gt)], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x)
    if (hist[i]) atomicAdd(order + i, hist[i]);
}

__global__ void __launch_bounds__(kOrderBuckets) order_scatter_kernel(CompositeArgs a, int32_t* __restrict__ order) {
  // Bucket offsets: a CTA-wide exclusive scan of the bucket sizes (one per
  // thread; the kernel runs with kOrderBuckets threads).
  __shared__ int base[kOrderBuckets];
  __shared__ int warp_sums[kOrderBuckets / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int size = order[threadIdx.x];
  int inc = size;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += warp_sums[w];
  base[threadIdx.x] = before + inc - size;
  // Each round places the CTA's next kOrderBuckets tiles: ranks within the
  // CTA by shared-memory counters, then one global atomic per (CTA, bucket)
  // reserves the CTA's places (most tiles of a scene can share one bucket:
  // the empty ones).
  __shared__ int count[kOrderBuckets], first_slot[kOrderBuckets];
  for (int64_t first = blockIdx.x * (int64_t)blockDim.x; first < a.total_tiles;
       first += (int64_t)gridDim.x * blockDim.x) {
    count[threadIdx.x] = 0;
    __syncthreads();
    const int64_t gt = first + threadIdx.x;
    const int b = gt < a.total_tiles ? order_bucket(a, gt) : -1;
    const int rank = b >= 0 ? atomicAdd(&count[b], 1) : 0;
    __syncthreads();
    const int c = count[threadIdx.x];
    if (c > 0) first_slot[threadIdx.x] = atomicAdd(order + kOrderBuckets + threadIdx.x, c);
    __syncthreads();
    if (b >= 0) order[kOrderHeader + base[b] + first_slot[b] + rank] = (int32_t)gt;
    __syncthreads();  // count and first_slot are reset by the next round
  }
}

// The work item the claim `u` stands for (launch order without an order).
__device__ __forceinline__ int64_t ordered_item(const CompositeArgs& a, const int32_t* __restrict__ order,
                                                int64_t u) {
  if (order == nullptr) return u;
  const int tw = (a.tile_h * a.tile_w + 31) / 32;
  return (int64_t)__ldg(order + kOrderHeader + u / tw) * tw + u % tw;
}

// With a tile order, the claims past the tiles with keys (which come last in
// the order) stand for items without keys: cheap, so they are claimed
// kEmptyClaim at a time. Returns the first such claim (all items without an
// order).
constexpr int kEmptyClaim = 8;

__device__ __forceinline__ int64_t keyed_items(const CompositeArgs& a, const int32_t* __restrict__ order) {
  const int64_t items = total_items(a);
  if (order == nullptr) return items;
  const int tw = (a.tile_h * a.tile_w + 31) / 32;
  return items - (int64_t)__ldg(order + kOrderBuckets - 1) * tw;
}

// Background blend and clip of the render entry points (images[:, :3] +
// images[:, 3:4] * background, then clip to [0, 1]); `inside` is clip's
// pass-through test (inclusive, as torch's clamp backward).
__device__ __forceinline__ float blend_clip(float rgb, float T, float bg, bool& inside) {
  const float x = __fadd_rn(rgb, __fmul_rn(T, bg));
  inside = x >= 0.0f && x <= 1.0f;
  return fminf(fmaxf(x, 0.0f), 1.0f);
}

__device__ __forceinline__ const float* target_of(const CompositeArgs& a, const Pixel& px) {
  return a.target + px.out_base / 4 * 3 + (int64_t)px.py * px.width + px.px;
}

// Reserves the work item's batches in the hit-bit store, in batches of
// kBatch for a bound on the keys the warp walks (the walk forms at most that
// many batches): with at most two warps to a tile, the tile's key count, which
// needs no pass over the masks (a 256^3 scene at 8x8 tiles reserves 165,764
// batches for the 94,988 walked); with more warps to a tile, the keys whose
// mask has this warp's bit, counted. Returns the item's first stored batch,
// or -1 when nothing is stored; records it for the backward.
__device__ __forceinline__ int64_t reserve_hit_batches(const HitStore& hs, const uint32_t* __restrict__ masks,
                                                       int64_t start, int64_t end, int wt, int tile_warps,
                                                       int64_t item, int lane) {
  int keys = (int)(end - start);
  if (tile_warps > 2) {
    keys = 0;
    for (int64_t k0 = start; k0 < end; k0 += 32) {
      const int64_t k = k0 + lane;
      keys += __popc(__ballot_sync(0xffffffffu, k < end && ((__ldg(masks + k) >> wt) & 1u)));
    }
  }
  const unsigned long long batches = (unsigned long long)((keys + kBatch - 1) / kBatch);
  unsigned long long base = 0;
  if (lane == 0 && batches > 0) base = atomicAdd(hs.next, batches);
  base = __shfl_sync(0xffffffffu, base, 0);
  const int64_t first = (batches > 0 && base < (unsigned long long)hs.capacity) ? (int64_t)base : -1;
  if (lane == 0) hs.item_base[item] = (int32_t)first;
  return first;
}

// Returns the pixel's sum of squared errors when the epilogue is on.
// `keyless`: the item's tile has no keys (known from the tile order): only
// the empty composite is written (no tile range, no hit-bit reservation: the
// backward never takes such items).
__device__ __forceinline__ float forward_item(const CompositeArgs& a, const uint32_t* __restrict__ masks,
                                              float* __restrict__ out, WarpForward& ws, const Pixel& px, int lane,
                                              int64_t item, const HitStore& hs, bool keyless = false) {
  const int64_t T = (int64_t)a.rows * a.cols;
  const float s = *a.sharpness;

  float acc[3] = {0.f, 0.f, 0.f};
  float T_ = 1.0f;
  bool active = px.in_image;
  int last_shell = -1;
  float e_dummy;
  float outer_cdf = sdf_to_cdf(1e10f, s, e_dummy);  // dummy outer sample

  const int64_t start = keyless ? 0 : a.bounds[2 * ((int64_t)px.cam * T + px.tile)];
  const int64_t end = keyless ? 0 : a.bounds[2 * ((int64_t)px.cam * T + px.tile) + 1];
  int64_t next = start;
  int queued = 0;
  int batch = 0;
  const int64_t hit_base =
      hs.batches && !keyless
          ? reserve_hit_batches(hs, masks, start, end, px.wt, (a.tile_h * a.tile_w + 31) / 32, item, lane)
          : -1;
  // With 8x4 warp blocks a triangle's span is the part of its accept box on
  // the block (lane 0 holds the block's first pixel); otherwise every pixel.
  const bool blocked = (a.tile_w & 7) == 0 && (a.tile_h & 3) == 0;
  const float bx = __shfl_sync(0xffffffffu, px.fx, 0), by = __shfl_sync(0xffffffffu, px.fy, 0);
  // Each batch's triangles are located (sorted key -> face -> vertex ids)
  // one batch ahead, while the previous batch is tested and composited, so
  // that staging a batch waits on one level of dependent loads only.
  queued = refill(masks, start, end, next, queued, ws.queue, px.wt, lane);
  int nb = min(queued, kBatch);
  TriRef ref{0, 0, 0, 0};
  if (lane < nb) ref = locate(a, start + ws.queue[lane]);
  while (__any_sync(0xffffffffu, active)) {
    if (nb == 0) break;
    uint32_t span = 0u;
    if (lane < nb) {
      float2 c[3];
      fetch(a, px.cam, ref, ws.geo, ws.attr, lane, c);
      if (blocked) {
        const TriGeom& g = ws.geo[lane];
        span = edge_span(g, cull_box(g, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y), bx, by);
      } else {
        span = kFullSpan;
      }
    }
    pop(ws.queue, queued, nb, lane);
    queued -= nb;
    queued = refill(masks, start, end, next, queued, ws.queue, px.wt, lane);
    const int nb_next = min(queued, kBatch);
    if (lane < nb_next) ref = locate(a, start + ws.queue[lane]);
    uint32_t hits = span_batch_hits(ws, span, blocked, bx, by, px.fx, px.fy, last_shell, active, s, lane);
    if (hit_base >= 0 && hit_base + batch < hs.capacity) __stcs(hs.batches + (hit_base + batch) * 32 + lane, hits);
    ++batch;
    if (active) {
      const int ns = min(ws.nsaved[lane], kSavedFwd);
      while (hits) {
        const int i = __ffs(hits) - 1;
        hits &= hits - 1;
        const TriGeom& g = ws.geo[i];
        if (g.shell <= last_shell) continue;
        float inner_cdf, rgb[3];
        hit_samples(ws, ns, i, lane, g, px.fx, px.fy, s, inner_cdf, rgb);
        const float alpha = clamp01(alpha_raw(outer_cdf, inner_cdf));
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[c] = over(acc[c], rgb[c], T_, alpha);
        T_ = __fmul_rn(T_, __fsub_rn(1.0f, alpha));
        outer_cdf = inner_cdf;
        last_shell = g.shell;
        if (last_shell == a.S - 1) {
          active = false;
          break;
        }
      }
    }
    nb = nb_next;
    __syncwarp();
  }
  float sq = 0.0f;
  if (px.in_image) {
    float* o = out + px.out_base + (int64_t)px.py * px.width + px.px;
    o[0] = acc[0];
    o[px.plane] = acc[1];
    o[2 * px.plane] = acc[2];
    o[3 * px.plane] = T_;
    if (a.target) {
      const float* tg = target_of(a, px);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        bool inside;
        const float d = blend_clip(acc[c], T_, a.background[c], inside) - tg[c * px.plane];
        sq += d * d;
      }
    }
  }
  __syncwarp();
  return sq;
}

template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps, 32 / kWarps)
    composite_forward_kernel(CompositeArgs a, const uint32_t* __restrict__ masks, float* __restrict__ out,
                             unsigned long long* __restrict__ counter, float* __restrict__ loss_sum,
                             HitStore hs, const int32_t* __restrict__ order) {
  extern __shared__ float4 smem_f4[];
  const int lane = threadIdx.x & 31;
  WarpForward& ws = reinterpret_cast<WarpForward*>(smem_f4)[threadIdx.x >> 5];
  const int64_t items = total_items(a);
  float sq = 0.0f;
  // Claims of one item while they land on items with keys, then of
  // kEmptyClaim items: a claim covers [u, u + claimed).
  const int64_t keyed = keyed_items(a, order);
  int64_t claimed = 1;
  for (int64_t u = next_item(counter, lane); u < items;) {
    for (int64_t v = u; v < min(u + claimed, items); ++v) {
      const int64_t item = ordered_item(a, order, v);
      sq += forward_item(a, masks, out, ws, pixel_of(a, item), lane, item, hs, v >= keyed);
    }
    claimed = u + claimed >= keyed ? kEmptyClaim : 1;  // the next claim lands at or past u + claimed
    unsigned long long next = 0;
    if (lane == 0) next = atomicAdd(counter, (unsigned long long)claimed);
    u = (int64_t)__shfl_sync(0xffffffffu, next, 0);
  }
  if (a.target) {  // one atomic per warp for the whole launch
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0 && sq != 0.0f) atomicAdd(loss_sum, sq * a.loss_scale);
  }
}

__device__ __forceinline__ void scatter_global(const CompositeArgs& a, const CompositeGrads& gr, int cam, int3 vid,
                                               float u, float v, float w, const float (&drgb)[3], float dsdf) {
  float* gc = gr.grad_colors + (int64_t)cam * a.V * 3;
  const int id[3] = {vid.x, vid.y, vid.z};
  const float wt[3] = {u, v, w};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(gc + 3 * (int64_t)id[q] + c, wt[q] * drgb[c]);
    atomicAdd(gr.grad_sdf + id[q], wt[q] * dsdf);
  }
}

__device__ __forceinline__ void scatter_slot(float* slot, float u, float v, float w, const float (&drgb)[3],
                                             float dsdf) {
  const float wt[3] = {u, v, w};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(slot + 4 * q + c, wt[q] * drgb[c]);
    atomicAdd(slot + 4 * q + 3, wt[q] * dsdf);
  }
}

// Flushes and clears the 32 ring slots of batch parity `half` (lane i owns
// slot half * 32 + i).
__device__ __forceinline__ void flush_half(const CompositeArgs& a, const CompositeGrads& gr, int cam, WarpBackward& ws,
                                           int half, int lane) {
  const int slot = half * kBatch + lane;
  float* g = ws.gslot[slot];
  const int3 vid = ws.vids[slot];
  const int id[3] = {vid.x, vid.y, vid.z};
  float* gc = gr.grad_colors + (int64_t)cam * a.V * 3;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float x = g[4 * q + c];
      if (x != 0.f) atomicAdd(gc + 3 * (int64_t)id[q] + c, x);
      g[4 * q + c] = 0.f;
    }
    const float y = g[4 * q + 3];
    if (y != 0.f) atomicAdd(gr.grad_sdf + id[q], y);
    g[4 * q + 3] = 0.f;
  }
  __syncwarp();
}

// Returns false when a staged wait gave up (the warp then stops).
template <bool kStaged, typename WS>
__device__ __forceinline__ bool backward_item(const CompositeArgs& a, const uint32_t* __restrict__ masks,
                                              const CompositeGrads& gr, WS& ws, const Pixel& px, int lane,
                                              int64_t item, const HitStore& hs, const Staging& st,
                                              uint32_t& phase) {
  const int64_t T = (int64_t)a.rows * a.cols;
  // A tile without keys has no hits, so nothing flows back from its pixels
  // (most tiles of a scene: with the tile order they come last).
  const int64_t range = 2 * ((int64_t)px.cam * T + px.tile);
  if (__ldg(a.bounds + range) == __ldg(a.bounds + range + 1)) return true;
  const float s = *a.sharpness;
  const int cam = px.cam;

  float final_rgb[3] = {0.f, 0.f, 0.f}, dL_rgb[3] = {0.f, 0.f, 0.f};
  float final_T = 0.f, dL_T = 0.f;
  if (px.in_image) {
    const int64_t o = px.out_base + (int64_t)px.py * px.width + px.px;
#pragma unroll
    for (int c = 0; c < 3; ++c) final_rgb[c] = a.out[o + c * px.plane];
    final_T = a.out[o + 3 * px.plane];
    if (a.target && a.ssaa > 1) {
      // SSAA: every sub-pixel gets 1 / ssaa^2 of its output pixel's
      // d loss / d image, through the background blend.
      const int f = a.ssaa;
      const int64_t wo = px.width / f, plane_out = (int64_t)(px.plane / ((int64_t)f * f));
      const float* g = a.target + (int64_t)px.cam * 3 * plane_out + (int64_t)(px.py / f) * wo + px.px / f;
      const float gscale = a.loss_scale * *gr.grad_loss / (float)(f * f);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float x = gscale * g[c * plane_out];
        dL_rgb[c] = x;
        dL_T += x * a.background[c];
      }
    } else if (a.target) {
      // d loss / d image = 2 (image - target) loss_scale, through the clip
      // and the background blend.
      const float gscale = 2.0f * a.loss_scale * *gr.grad_loss;
      const float* tg = target_of(a, px);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        bool inside;
        const float img = blend_clip(final_rgb[c], final_T, a.background[c], inside);
        const float g = inside ? gscale * (img - tg[c * px.plane]) : 0.0f;
        dL_rgb[c] = g;
        dL_T += g * a.background[c];
      }
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) dL_rgb[c] = gr.grad_out[o + c * px.plane];
      dL_T = gr.grad_out[o + 3 * px.plane];
    }
  }
  for (int i = lane; i < kRing * 13; i += 32) (&ws.gslot[0][0])[i] = 0.f;
  ws.vids[lane] = make_int3(0, 0, 0);
  ws.vids[kBatch + lane] = make_int3(0, 0, 0);
  __syncwarp();

  float acc[3] = {0.f, 0.f, 0.f};
  float T_ = 1.0f;
  bool active = px.in_image;
  int last_shell = -1;
  float e_out;
  float outer_cdf = sdf_to_cdf(1e10f, s, e_out);
  float outer_sdf = 1e10f;
  float d_sharp = 0.f;
  float dp_rgb[3] = {0.f, 0.f, 0.f};
  float dp_sdf = 0.f;
  int prev_batch = -2, prev_slot = 0;  // ring slot of the previous hit (valid while its batch is live)
  int3 prev_vid = make_int3(0, 0, 0);
  float pu = 0.f, pv = 0.f, pw = 0.f;

  const int64_t start = a.bounds[2 * ((int64_t)cam * T + px.tile)];
  const int64_t end = a.bounds[2 * ((int64_t)cam * T + px.tile) + 1];
  int64_t next = start;
  int queued = 0;
  int batch = 0;
  const int64_t hit_base = hs.batches ? (int64_t)hs.item_base[item] : -1;
  // Staged form: the next batch is formed one step ahead and its vertex
  // records are in flight while the current batch composites.
  int nb_next = 0, shell_next = 0;
  bool stored_next = false;
  uint32_t hits_next = 0, needed_next = 0;
  int3 vid_next = make_int3(0, 0, 0);
  auto form_next = [&](int b) {
    queued = refill(masks, start, end, next, queued, ws.queue, px.wt, lane);
    nb_next = min(queued, kBatch);
    if (nb_next == 0) return;
    stored_next = hit_base >= 0 && hit_base + b < hs.capacity;
    hits_next = stored_next ? __ldcs(hs.batches + (hit_base + b) * 32 + lane) : 0u;
    needed_next = stored_next ? __reduce_or_sync(0xffffffffu, hits_next) : 0xffffffffu;
    const bool mine = lane < nb_next && ((needed_next >> lane) & 1u);
    if (mine) {
      const int64_t k = start + ws.queue[lane];
      const int32_t f = __ldg(a.tri + k);
      const uint64_t key = __ldg(reinterpret_cast<const unsigned long long*>(a.keys) + k);
      vid_next = make_int3(__ldg(a.faces + 3 * (int64_t)f), __ldg(a.faces + 3 * (int64_t)f + 1),
                           __ldg(a.faces + 3 * (int64_t)f + 2));
      shell_next = (int)field(key, a.shell_off, a.shell_len);
    }
    const uint32_t copies = __popc(__ballot_sync(0xffffffffu, mine));
    if constexpr (kStaged) {
      if (lane == 0) mbar_arrive_expect_tx(&ws.bar, copies * 3 * (uint32_t)sizeof(VertexRecord));
      __syncwarp();
      if (mine) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const VertexRecord* r = st.records + (int64_t)cam * a.V;
        bulk_copy_to_shared(&ws.stage[lane][0], r + vid_next.x, sizeof(VertexRecord), &ws.bar);
        bulk_copy_to_shared(&ws.stage[lane][1], r + vid_next.y, sizeof(VertexRecord), &ws.bar);
        bulk_copy_to_shared(&ws.stage[lane][2], r + vid_next.z, sizeof(VertexRecord), &ws.bar);
      }
    }
    pop(ws.queue, queued, nb_next, lane);
    queued -= nb_next;
  };
  if constexpr (kStaged) form_next(0);
  while (__any_sync(0xffffffffu, active)) {
    int nb;
    bool stored;
    uint32_t hits;
    const int half = batch & 1;
    if constexpr (kStaged) {
      nb = nb_next;
      if (nb == 0) break;
      stored = stored_next;
      hits = hits_next;
      const uint32_t needed = needed_next;
      if (!mbar_wait(&ws.bar, phase & 1u)) {
        if (lane == 0) set_device_error(st.status, MT_ERR_DEVICE_TIMEOUT);
        return false;
      }
      ++phase;
      if (batch >= 2) flush_half(a, gr, cam, ws, half, lane);
      if (lane < nb && ((needed >> lane) & 1u)) {
        const VertexRecord ra = ws.stage[lane][0], rb = ws.stage[lane][1], rc = ws.stage[lane][2];
        TriGeom g;
        setup_geometry(ra.x, ra.y, rb.x, rb.y, rc.x, rc.y, g);
        g.shell = shell_next;
        ws.geo[lane] = g;
        ws.attr[lane] = TriAttr{{ra.r, ra.g, ra.b}, {rb.r, rb.g, rb.b}, {rc.r, rc.g, rc.b}, ra.sdf, rb.sdf, rc.sdf};
        ws.vids[half * kBatch + lane] = vid_next;
      }
      __syncwarp();
      form_next(batch + 1);  // the next batch's copies overlap this batch's compositing
    } else {
      queued = refill(masks, start, end, next, queued, ws.queue, px.wt, lane);
      nb = min(queued, kBatch);
      if (nb == 0) break;
      // The half being overwritten held batch - 2: flush it first.
      if (batch >= 2) flush_half(a, gr, cam, ws, half, lane);
      // The forward's hit bits for this batch when it stored them (the same
      // walk, so the same bits); otherwise the test phase runs again. With
      // stored bits only the triangles that some pixel of the warp hits are
      // gathered (the other slots are never read).
      stored = hit_base >= 0 && hit_base + batch < hs.capacity;
      hits = stored ? __ldcs(hs.batches + (hit_base + batch) * 32 + lane) : 0u;
      const uint32_t needed = stored ? __reduce_or_sync(0xffffffffu, hits) : 0xffffffffu;
      if (lane < nb && ((needed >> lane) & 1u))
        ws.vids[half * kBatch + lane] = gather(a, cam, start + ws.queue[lane], ws.geo, ws.attr, lane);
      pop(ws.queue, queued, nb, lane);
      queued -= nb;
    }
    if (!stored && active) hits = batch_hits(ws.geo, nb, px.fx, px.fy, last_shell, ws.saved, lane);
    if (active) {
      int n = 0;
      while (hits) {
        const int i = __ffs(hits) - 1;
        hits &= hits - 1;
        const int k = n++;
        const TriGeom& g = ws.geo[i];
        if (g.shell <= last_shell) continue;
        float u, v, w;
        if (stored)
          hit_test(g, px.fx, px.fy, u, v, w);  // a hit: the solve gives the forward's (u, v, w)
        else
          hit_weights(ws.saved, k, lane, g, px.fx, px.fy, u, v, w);
        const TriAttr& t = ws.attr[i];
        const float sdf_in = interp(u, v, w, t.sa, t.sb, t.sc);
        float e_in;
        const float inner_cdf = sdf_to_cdf(sdf_in, s, e_in);
        const float raw = alpha_raw(outer_cdf, inner_cdf);
        const float alpha = clamp01(raw);

        // Suffix trick (intersect_and_composite.slang:458-473).
        const float weight = __fmul_rn(alpha, T_);
        const float inv = __fdiv_rn(1.0f, __fadd_rn(__fsub_rn(1.0f, alpha), 1e-6f));
        float d_color[3];
        float d_alpha = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float rgb = interp(u, v, w, t.ca[c], t.cb[c], t.cc[c]);
          acc[c] = __fadd_rn(acc[c], __fmul_rn(weight, rgb));
          const float suffix = final_rgb[c] - acc[c];
          d_color[c] = weight * dL_rgb[c];
          d_alpha += dL_rgb[c] * (T_ * rgb - suffix * inv);
        }
        d_alpha += -dL_T * final_T * inv;

        // compute_alpha backward; the clamp passes gradient strictly inside.
        const float d_raw = (raw > 0.0f && raw < 1.0f) ? d_alpha : 0.0f;
        const float den = outer_cdf + 1e-5f;
        const float num = (outer_cdf - inner_cdf) + 1e-5f;
        const float d_num = d_raw / den;
        const float d_den = -d_raw * num / (den * den);
        const float d_oc = d_num + d_den;
        const float d_ic = -d_num;
        // d cdf / d sdf = cdf^2 e s ; d cdf / d s = cdf^2 e sdf.
        const float ki = inner_cdf * inner_cdf * e_in;
        const float ko = outer_cdf * outer_cdf * e_out;
        d_sharp += d_ic * ki * sdf_in + d_oc * ko * outer_sdf;

        if (last_shell != -1) {
          dp_sdf += d_oc * ko * s;
          const float su = gr.exact ? pu : u, sv = gr.exact ? pv : v, sw = gr.exact ? pw : w;
          if (prev_batch >= batch - 1)
            scatter_slot(ws.gslot[prev_slot], su, sv, sw, dp_rgb, dp_sdf);
          else
            scatter_global(a, gr, cam, prev_vid, su, sv, sw, dp_rgb, dp_sdf);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) dp_rgb[c] = d_color[c];
        dp_sdf = d_ic * ki * s;
        prev_batch = batch;
        prev_slot = half * kBatch + i;
        prev_vid = ws.vids[prev_slot];
        pu = u;
        pv = v;
        pw = w;

        T_ = __fmul_rn(T_, __fsub_rn(1.0f, alpha));
        outer_cdf = inner_cdf;
        outer_sdf = sdf_in;
        e_out = e_in;
        last_shell = g.shell;
        if (last_shell == a.S - 1) {
          active = false;
          break;
        }
      }
    }
    __syncwarp();
    ++batch;
  }
  if constexpr (kStaged) {
    // A batch formed ahead whose copies are still in flight: let them land
    // before the stage is reused.
    if (nb_next > 0) {
      if (!mbar_wait(&ws.bar, phase & 1u)) {
        if (lane == 0) set_device_error(st.status, MT_ERR_DEVICE_TIMEOUT);
        return false;
      }
      ++phase;
    }
  }
  // The last hit's deferred gradient, with its own weights.
  if (px.in_image && last_shell != -1) {
    if (prev_batch >= batch - 2)
      scatter_slot(ws.gslot[prev_slot], pu, pv, pw, dp_rgb, dp_sdf);
    else
      scatter_global(a, gr, cam, prev_vid, pu, pv, pw, dp_rgb, dp_sdf);
  }
  __syncwarp();
  flush_half(a, gr, cam, ws, 0, lane);
  flush_half(a, gr, cam, ws, 1, lane);

  // Sharpness gradient: one atomic per warp.
  float x = px.in_image ? d_sharp : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if (lane == 0 && x != 0.f) atomicAdd(gr.grad_sharpness, x);
  __syncwarp();
  return true;
}

template <bool kStaged>
using WarpBackwardOf = typename std::conditional<kStaged, WarpBackwardStaged, WarpBackward>::type;

// The unstaged form keeps to 80 registers (24 warps per SM) at every CTA size.
template <bool kStaged, int kWarps>
__global__ void __launch_bounds__(32 * kWarps, kStaged ? 1 : (24 / kWarps > 0 ? 24 / kWarps : 1))
    composite_backward_kernel(CompositeArgs a, const uint32_t* __restrict__ masks, CompositeGrads gr,
                              unsigned long long* __restrict__ counter, HitStore hs, Staging st,
                              const int32_t* __restrict__ order) {
  extern __shared__ float4 smem_f4[];
  const int lane = threadIdx.x & 31;
  WarpBackwardOf<kStaged>& ws = reinterpret_cast<WarpBackwardOf<kStaged>*>(smem_f4)[threadIdx.x >> 5];
  uint32_t phase = 0;
  if constexpr (kStaged) {
    if (lane == 0) mbar_init(&ws.bar);
    __syncwarp();
  }
  // Items without keys pass no gradient: with a tile order they are all past
  // `keyed` and never claimed. The bound is read from shared memory at each
  // claim: held in registers across the loop it made the kernel spill.
  __shared__ int64_t s_keyed;
  if (threadIdx.x == 0) s_keyed = keyed_items(a, order);
  __syncthreads();
  for (int64_t u = next_item(counter, lane); u < *(volatile int64_t*)&s_keyed; u = next_item(counter, lane)) {
    const int64_t item = ordered_item(a, order, u);
    if (!backward_item<kStaged>(a, masks, gr, ws, pixel_of(a, item), lane, item, hs, st, phase)) return;
  }
}

// Packed (camera, vertex) records for the staged backward.
__global__ void pack_vertex_records_kernel(const float* __restrict__ xy, const float* __restrict__ colors,
                                           const float* __restrict__ sdf, int64_t V, int B,
                                           VertexRecord* __restrict__ out) {
  const int64_t n = (int64_t)B * V;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = o % V;
    const float2 p = reinterpret_cast<const float2*>(xy)[o];
    out[o] = VertexRecord{p.x, p.y, colors[3 * o], colors[3 * o + 1], colors[3 * o + 2], __ldg(sdf + v), 0.f, 0.f};
  }
}

// The MSE epilogue with SSAA (triangle_rasterization/__init__.py:274-287
// followed by the trainer's MSE): per output pixel, the mean over its
// ssaa x ssaa sub-pixels of rgb + T * background, clipped to [0, 1], against
// the target; loss += loss_scale x sum of squared errors (one atomic per CTA),
// and factor = 2 (image - target) where the clip passes the gradient, else 0
// (the backward scales it by loss_scale x d L / d loss / ssaa^2).
__global__ void ssaa_loss_kernel(const float* __restrict__ raw, int B, int H, int W, int f,
                                 const float* __restrict__ background, const float* __restrict__ target,
                                 float loss_scale, float* __restrict__ loss, float* __restrict__ factor) {
  const int ho = H / f, wo = W / f;
  const int64_t plane = (int64_t)H * W, plane_out = (int64_t)ho * wo;
  const int64_t n = (int64_t)B * plane_out;
  const float inv = 1.0f / (float)(f * f);
  float sq = 0.0f;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = o / plane_out, r = o - b * plane_out;
    const int y = (int)(r / wo), x = (int)(r - (int64_t)y * wo);
    const float* src = raw + b * 4 * plane;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float acc = 0.0f;
      for (int dy = 0; dy < f; ++dy) {
        const int64_t row = (int64_t)(y * f + dy) * W + (int64_t)x * f;
        for (int dx = 0; dx < f; ++dx)
          acc += __fadd_rn(src[c * plane + row + dx], __fmul_rn(src[3 * plane + row + dx], background[c]));
      }
      const float mean = acc * inv;
      const bool inside = mean >= 0.0f && mean <= 1.0f;
      const float d = fminf(fmaxf(mean, 0.0f), 1.0f) - target[(b * 3 + c) * plane_out + r];
      sq += d * d;
      factor[(b * 3 + c) * plane_out + r] = inside ? 2.0f * d : 0.0f;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  __shared__ float part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    if (t != 0.0f) atomicAdd(loss, t * loss_scale);
  }
}

int check_args(const CompositeArgs& a) {
  if (a.B < 0 || a.S < 1 || a.rows < 0 || a.cols < 0 || a.tile_h < 1 || a.tile_w < 1 || a.H < 0 || a.W < 0)
    return MT_ERR_INVALID_ARGUMENT;
  if ((int64_t)a.tile_h * a.tile_w > 1024) return MT_ERR_INVALID_ARGUMENT;
  if ((int64_t)a.rows * a.tile_h < a.H || (int64_t)a.cols * a.tile_w < a.W) return MT_ERR_INVALID_ARGUMENT;
  auto ok = [](int off, int len) { return off >= 0 && len >= 1 && len <= 31 && off + len <= 64; };
  if (!ok(a.shell_off, a.shell_len) || !ok(a.cam_off, a.cam_len) || !ok(a.tile_off, a.tile_len))
    return MT_ERR_INVALID_ARGUMENT;
  return MT_OK;
}

// Warps per CTA for a requested threads-per-CTA (128, 256 or 512; anything
// else, 0 included, gives the default 256).
int cta_warps(int32_t threads) {
  return threads == 128 ? 4 : threads == 512 ? 16 : kDefaultWarpsPerCta;
}

// Persistent grid: as many CTAs as fit on the device at once (queried once
// per kernel and device), but no more than there are work items for.
template <auto Kernel, int kWarps>
int persistent_ctas(const CompositeArgs& a, size_t smem, int64_t& ctas) {
  static std::atomic<int> resident[64];
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MT_ERR_CUDA;
  int r = resident[device].load(std::memory_order_acquire);
  if (r == 0) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MT_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kernel, 32 * kWarps, smem) != cudaSuccess)
      return MT_ERR_CUDA;
    r = max(1, sms * max(per_sm, 1));
    resident[device].store(r, std::memory_order_release);
  }
  const int64_t warps = a.total_tiles * ((a.tile_h * a.tile_w + 31) / 32);
  const int64_t needed = (warps + kWarps - 1) / kWarps;
  ctas = needed < (int64_t)r ? needed : (int64_t)r;
  return MT_OK;
}


// The hit-bit store of `bytes` bytes at `base` for the launch's work items
// (NULL base or too few bytes for one batch: no store).
int make_hit_store(const CompositeArgs& a, void* base, size_t bytes, HitStore& hs) {
  hs = HitStore{nullptr, nullptr, nullptr, 0};
  if (base == nullptr) return MT_OK;
  if ((reinterpret_cast<uintptr_t>(base) & 127) != 0) return MT_ERR_INVALID_ARGUMENT;
  const int64_t items = a.total_tiles * ((a.tile_h * a.tile_w + 31) / 32);
  const size_t header = hit_store_header(items);
  if (bytes < header + 128) return MT_OK;
  int64_t cap = (int64_t)((bytes - header) / 128);
  if (cap > 0x7fffffff) cap = 0x7fffffff;  // item bases are int32
  char* p = static_cast<char*>(base);
  hs = HitStore{reinterpret_cast<unsigned long long*>(p), reinterpret_cast<int32_t*>(p + 8),
                reinterpret_cast<uint32_t*>(p + header), cap};
  return MT_OK;
}

CompositeArgs make_args(const float* xy, const float* colors, const float* sdf, int64_t V, const int32_t* faces,
                        const float* sharpness, const int64_t* keys, const int32_t* tri, const int64_t* bounds,
                        int32_t B, int32_t S, int32_t rows, int32_t cols, int32_t tile_h, int32_t tile_w, int32_t H,
                        int32_t W, const int32_t* layout, const float* out, const int64_t* cameras,
                        int64_t camera_tiles) {
  CompositeArgs a{};
  a.ssaa = 1;
  a.target = nullptr;
  a.background = nullptr;
  a.loss_scale = 0.0f;
  a.cameras = cameras;
  a.total_tiles = cameras ? camera_tiles : (int64_t)B * rows * cols;
  a.xy = xy;
  a.colors = colors;
  a.sdf = sdf;
  a.V = V;
  a.faces = faces;
  a.sharpness = sharpness;
  a.keys = reinterpret_cast<const uint64_t*>(keys);
  a.tri = tri;
  a.bounds = bounds;
  a.B = B;
  a.S = S;
  a.rows = rows;
  a.cols = cols;
  a.tile_h = tile_h;
  a.tile_w = tile_w;
  a.H = H;
  a.W = W;
  a.cam_off = layout ? layout[0] : -1;
  a.cam_len = layout ? layout[1] : 0;
  a.shell_off = layout ? layout[2] : -1;
  a.shell_len = layout ? layout[3] : 0;
  a.tile_off = layout ? layout[4] : -1;
  a.tile_len = layout ? layout[5] : 0;
  a.out = out;
  return a;
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

size_t mt_composite_tile_order_bytes(int64_t camera_tiles) {
  if (camera_tiles < 0) camera_tiles = 0;
  return ((size_t)mt::kOrderHeader + (size_t)camera_tiles) * sizeof(int32_t);
}

size_t mt_composite_staging_bytes(int32_t B, int64_t V) {
  if (B <= 0 || V <= 0) return 0;
  return 128 + (size_t)B * (size_t)V * sizeof(VertexRecord);
}

size_t mt_composite_hit_bits_bytes(int64_t camera_tiles, int32_t tile_h, int32_t tile_w, int64_t batches) {
  if (camera_tiles <= 0 || tile_h <= 0 || tile_w <= 0 || batches <= 0) return 0;
  if (batches > 0x7fffffff) batches = 0x7fffffff;
  const int64_t items = camera_tiles * (((int64_t)tile_h * tile_w + 31) / 32);
  return hit_store_header(items) + (size_t)batches * 128;
}

int mt_intersect_and_composite_forward(const float* xy, const float* colors, const float* signed_distances,
                                       int64_t V, const int32_t* faces, const float* sharpness,
                                       const int64_t* sorted_keys, const int32_t* sorted_triangles, int64_t K,
                                       const int64_t* num_keys, const int64_t* tile_boundaries, int32_t B,
                                       int32_t num_shells, int32_t rows, int32_t cols, int32_t tile_h,
                                       int32_t tile_w, int32_t H, int32_t W, const int32_t* layout,
                                       const int64_t* cameras, int64_t camera_tiles, uint32_t* warp_masks,
                                       uint64_t* work_counter, float* out, const float* target,
                                       const float* background, float loss_scale, float* loss_sum,
                                       void* hit_bits, size_t hit_bits_bytes, int32_t* tile_order,
                                       size_t tile_order_bytes, int32_t cta_threads, mt_stream_t stream) {
  MT_REQUIRE(layout != nullptr && K >= 0 && camera_tiles >= 0);
  CompositeArgs a = make_args(xy, colors, signed_distances, V, faces, sharpness, sorted_keys, sorted_triangles,
                              tile_boundaries, B, num_shells, rows, cols, tile_h, tile_w, H, W, layout, nullptr,
                              cameras, camera_tiles);
  a.target = target;
  a.background = background;
  a.loss_scale = loss_scale;
  int rc = check_args(a);
  if (rc != MT_OK) return rc;
  MT_REQUIRE(target == nullptr || (background && loss_sum));
  cudaStream_t s = as_stream(stream);
  if (target && cudaMemsetAsync(loss_sum, 0, sizeof(float), s) != cudaSuccess) return MT_ERR_CUDA;
  if (a.total_tiles == 0 || H == 0 || W == 0) return MT_OK;
  MT_REQUIRE(xy && colors && signed_distances && faces && sharpness && tile_boundaries && out && work_counter);
  MT_REQUIRE(K == 0 || (sorted_keys && sorted_triangles && warp_masks));
  HitStore hs;
  rc = make_hit_store(a, hit_bits, hit_bits_bytes, hs);
  if (rc != MT_OK) return rc;
  if (hs.next && cudaMemsetAsync(hs.next, 0, 8, s) != cudaSuccess) return MT_ERR_CUDA;
  if (K > 0) {
    warp_mask_kernel<<<grid_stride_blocks(K, 256), 256, 0, s>>>(a, K, num_keys, warp_masks);
    MT_CHECK_LAUNCH();
  }
  if (cudaMemsetAsync(work_counter, 0, sizeof(uint64_t), s) != cudaSuccess) return MT_ERR_CUDA;
  if (tile_order) {
    MT_REQUIRE(tile_order_bytes >= mt_composite_tile_order_bytes(a.total_tiles));
    if (cudaMemsetAsync(tile_order, 0, kOrderHeader * sizeof(int32_t), s) != cudaSuccess) return MT_ERR_CUDA;
    const unsigned blocks = grid_stride_blocks(a.total_tiles, 256, 1);
    order_histogram_kernel<<<blocks, 256, 0, s>>>(a, tile_order);
    MT_CHECK_LAUNCH();
    order_scatter_kernel<<<blocks, kOrderBuckets, 0, s>>>(a, tile_order);
    MT_CHECK_LAUNCH();
  }
  auto launch = [&](auto warps) -> int {
    constexpr int kW = decltype(warps)::value;
    const size_t smem = sizeof(WarpForward) * kW;
    int r = set_smem<composite_forward_kernel<kW>>(smem);
    if (r != MT_OK) return r;
    int64_t ctas = 0;
    r = persistent_ctas<composite_forward_kernel<kW>, kW>(a, smem, ctas);
    if (r != MT_OK) return r;
    composite_forward_kernel<kW><<<(unsigned)ctas, 32 * kW, smem, s>>>(
        a, warp_masks, out, reinterpret_cast<unsigned long long*>(work_counter), loss_sum, hs, tile_order);
    MT_CHECK_LAUNCH();
    return MT_OK;
  };
  switch (cta_warps(cta_threads)) {
    case 4: return launch(std::integral_constant<int, 4>{});
    case 16: return launch(std::integral_constant<int, 16>{});
    default: return launch(std::integral_constant<int, 8>{});
  }
}

int mt_intersect_and_composite_backward(const float* xy, const float* colors, const float* signed_distances,
                                        int64_t V, const int32_t* faces, const float* sharpness,
                                        const int64_t* sorted_keys, const int32_t* sorted_triangles, int64_t K,
                                        const int64_t* tile_boundaries, int32_t B, int32_t num_shells,
                                        int32_t rows, int32_t cols, int32_t tile_h, int32_t tile_w, int32_t H,
                                        int32_t W, const int32_t* layout, const int64_t* cameras,
                                        int64_t camera_tiles, const uint32_t* warp_masks, uint64_t* work_counter,
                                        const float* out, const float* grad_out, const float* target,
                                        const float* background, float loss_scale, const float* grad_loss,
                                        int32_t ssaa, float* grad_colors, float* grad_signed_distances,
                                        float* grad_sharpness,
                                        int32_t exact_adjoint, const void* hit_bits, size_t hit_bits_bytes,
                                        void* staging, size_t staging_bytes, const int32_t* tile_order,
                                        size_t tile_order_bytes, int32_t cta_threads, mt_stream_t stream) {
  MT_REQUIRE(layout != nullptr && K >= 0 && camera_tiles >= 0);
  CompositeArgs a = make_args(xy, colors, signed_distances, V, faces, sharpness, sorted_keys, sorted_triangles,
                              tile_boundaries, B, num_shells, rows, cols, tile_h, tile_w, H, W, layout, out,
                              cameras, camera_tiles);
  a.target = target;
  a.background = background;
  a.loss_scale = loss_scale;
  a.ssaa = ssaa;
  int rc = check_args(a);
  if (rc != MT_OK) return rc;
  MT_REQUIRE(ssaa >= 1 && (ssaa == 1 || (target && !cameras && H % ssaa == 0 && W % ssaa == 0)));
  if (a.total_tiles == 0 || H == 0 || W == 0) return MT_OK;
  MT_REQUIRE(xy && colors && signed_distances && faces && sharpness && tile_boundaries && out);
  MT_REQUIRE(target ? (background && grad_loss) : grad_out != nullptr);
  MT_REQUIRE(grad_colors && grad_signed_distances && grad_sharpness && work_counter);
  MT_REQUIRE(K == 0 || (sorted_keys && sorted_triangles && warp_masks));
  CompositeGrads gr{grad_loss, grad_out, grad_colors, grad_signed_distances, grad_sharpness, exact_adjoint ? 1 : 0};
  HitStore hs;
  rc = make_hit_store(a, const_cast<void*>(hit_bits), hit_bits_bytes, hs);
  if (rc != MT_OK) return rc;
  cudaStream_t s = as_stream(stream);
  MT_REQUIRE(tile_order == nullptr || tile_order_bytes >= mt_composite_tile_order_bytes(a.total_tiles));
  if (cudaMemsetAsync(work_counter, 0, sizeof(uint64_t), s) != cudaSuccess) return MT_ERR_CUDA;
  const bool staged = staging != nullptr && staging_bytes >= mt_composite_staging_bytes(B, V);
  Staging st{nullptr, nullptr};
  if (staged) {
    MT_REQUIRE((reinterpret_cast<uintptr_t>(staging) & 127) == 0);
    st = Staging{reinterpret_cast<const VertexRecord*>(static_cast<char*>(staging) + 128),
                 static_cast<int*>(staging)};
    const int64_t n = (int64_t)B * V;
    if (n > 0) {
      pack_vertex_records_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(
          xy, colors, signed_distances, V, B, const_cast<VertexRecord*>(st.records));
      MT_CHECK_LAUNCH();
    }
  }
  auto launch = [&](auto staged_c, auto warps) -> int {
    constexpr bool kS = decltype(staged_c)::value;
    constexpr int kW = decltype(warps)::value;
    const size_t smem = sizeof(WarpBackwardOf<kS>) * kW;
    int r = set_smem<composite_backward_kernel<kS, kW>>(smem);
    if (r != MT_OK) return r;
    int64_t ctas = 0;
    r = persistent_ctas<composite_backward_kernel<kS, kW>, kW>(a, smem, ctas);
    if (r != MT_OK) return r;
    composite_backward_kernel<kS, kW><<<(unsigned)ctas, 32 * kW, smem, s>>>(
        a, warp_masks, gr, reinterpret_cast<unsigned long long*>(work_counter), hs, st, tile_order);
    MT_CHECK_LAUNCH();
    return MT_OK;
  };
  const int warps = cta_warps(cta_threads);
  if (staged) {
    if (warps == 4) return launch(std::true_type{}, std::integral_constant<int, 4>{});
    if (warps == 16) return launch(std::true_type{}, std::integral_constant<int, 16>{});
    return launch(std::true_type{}, std::integral_constant<int, 8>{});
  }
  if (warps == 4) return launch(std::false_type{}, std::integral_constant<int, 4>{});
  if (warps == 16) return launch(std::false_type{}, std::integral_constant<int, 16>{});
  return launch(std::false_type{}, std::integral_constant<int, 8>{});
}

int mt_ssaa_loss(const float* raw, int32_t B, int32_t H, int32_t W, int32_t ssaa, const float* background,
                 const float* target, float loss_scale, float* loss, float* factor, mt_stream_t stream) {
  MT_REQUIRE(B >= 0 && H >= 0 && W >= 0 && ssaa >= 1 && H % ssaa == 0 && W % ssaa == 0 && loss != nullptr);
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess) return MT_ERR_CUDA;
  const int64_t n = (int64_t)B * (H / ssaa) * (W / ssaa);
  if (n == 0) return MT_OK;
  MT_REQUIRE(raw && background && target && factor);
  ssaa_loss_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(raw, B, H, W, ssaa, background, target, loss_scale,
                                                              loss, factor);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
