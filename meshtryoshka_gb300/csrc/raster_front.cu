// Rasterization front end for sm_103a: camera centres, vertex projection,
// spherical-harmonic colours (forward / backward), triangle tile bounds, key
// generation and tile delineation.
//
// Follows triangle_rasterization/project_vertices.slang, bound_triangles.slang,
// generate_keys.slang + keys.slang, delineate_tiles.slang and
// evaluate_spherical_harmonics.slang. Arithmetic follows the reference
// source's operations in their order, without contraction (explicit
// __fmul_rn / __fadd_rn, never fused by nvcc), so projected positions, tile
// bounds, key depths and colours equal the reference kernels evaluated
// operation by operation in IEEE-754 single precision.

#include "lookback.cuh"  // warp_sum, warp_inclusive_sum
#include "sh.cuh"

namespace mt {
namespace {

// ---------------------------------------------------------------------------
// Camera centres: inverse(extrinsics)[:, :3, 3]
// (triangle_rasterization/evaluate_spherical_harmonics.py:38), in fp64.
// ---------------------------------------------------------------------------
// One warp per camera: column 3 of the inverse is C[3][r] / det with
// det = sum_c m[0][c] C[0][c], so only seven cofactors are needed; lanes
// 0-3 compute C[0][c], lanes 4-6 C[3][r] (one 3x3 minor each).
__global__ void camera_positions_kernel(const float* __restrict__ ext, int B, float* __restrict__ out) {
  const int cam = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (cam >= B) return;  // whole warps exit together
  const float* E = ext + 16 * cam;
  double cof = 0.0;
  if (lane < 7) {
    const int skip_r = lane < 4 ? 0 : 3, skip_c = lane < 4 ? lane : lane - 4;
    int rs[3], cs[3], ri = 0, ci = 0;
    for (int k = 0; k < 4; ++k) {
      if (k != skip_r) rs[ri++] = k;
      if (k != skip_c) cs[ci++] = k;
    }
    auto m = [&](int r, int c) { return (double)E[4 * r + c]; };
    const double minor =
        m(rs[0], cs[0]) * (m(rs[1], cs[1]) * m(rs[2], cs[2]) - m(rs[1], cs[2]) * m(rs[2], cs[1])) -
        m(rs[0], cs[1]) * (m(rs[1], cs[0]) * m(rs[2], cs[2]) - m(rs[1], cs[2]) * m(rs[2], cs[0])) +
        m(rs[0], cs[2]) * (m(rs[1], cs[0]) * m(rs[2], cs[1]) - m(rs[1], cs[1]) * m(rs[2], cs[0]));
    cof = ((skip_r + skip_c) & 1) ? -minor : minor;
  }
  double det = 0.0;
#pragma unroll
  for (int c = 0; c < 4; ++c) det += (double)E[c] * __shfl_sync(0xffffffffu, cof, c);
  if (lane >= 4 && lane < 7) out[3 * cam + (lane - 4)] = (float)(cof / det);
}

// ---------------------------------------------------------------------------
// project_vertices.slang:51-92. cam = W2C [v, 1]; xy = (K cam).xy / cam.z.
// ---------------------------------------------------------------------------
__global__ void project_kernel(const float* __restrict__ verts, int64_t V, const float* __restrict__ ext,
                               const float* __restrict__ intr, int B, float* __restrict__ out_xy,
                               float* __restrict__ out_depth) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float x = verts[3 * v], y = verts[3 * v + 1], z = verts[3 * v + 2];
    for (int b = 0; b < B; ++b) {
      const float* E = ext + 16 * b;
      const float* K = intr + 9 * b;
      // mul(W2C, float4(v, 1)) and mul(K, cam.xyz): row sums left to right.
      float cam[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float* row = E + 4 * r;
        cam[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(row[0], x), __fmul_rn(row[1], y)), __fmul_rn(row[2], z)),
                           __fmul_rn(row[3], 1.0f));
      }
      const float kx =
          __fadd_rn(__fadd_rn(__fmul_rn(K[0], cam[0]), __fmul_rn(K[1], cam[1])), __fmul_rn(K[2], cam[2]));
      const float ky =
          __fadd_rn(__fadd_rn(__fmul_rn(K[3], cam[0]), __fmul_rn(K[4], cam[1])), __fmul_rn(K[5], cam[2]));
      const int64_t o = (int64_t)b * V + v;
      out_xy[2 * o] = __fdiv_rn(kx, cam[2]);
      out_xy[2 * o + 1] = __fdiv_rn(ky, cam[2]);
      out_depth[o] = cam[2];
    }
  }
}

// The vertex's coefficients are read once into registers and serve every
// camera.
template <int kCoeff>
__device__ __forceinline__ void sh_forward_vertex(const float* __restrict__ verts, int64_t V,
                                                  const float* __restrict__ sh, const float* __restrict__ campos,
                                                  int B, int64_t v, float* __restrict__ out) {
  float coef[kCoeff][3];
#pragma unroll
  for (int k = 0; k < kCoeff; ++k) {
    const float* s = sh + ((int64_t)k * V + v) * 3;
    coef[k][0] = __ldg(s);
    coef[k][1] = __ldg(s + 1);
    coef[k][2] = __ldg(s + 2);
  }
  sh_colors<kCoeff>(verts, V, coef, campos, B, v, out);
}

__global__ void sh_forward_kernel(const float* __restrict__ verts, int64_t V, const float* __restrict__ sh,
                                  int n_coeff, const float* __restrict__ campos, int B, float* __restrict__ out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    switch (n_coeff) {
      case 1: sh_forward_vertex<1>(verts, V, sh, campos, B, v, out); break;
      case 4: sh_forward_vertex<4>(verts, V, sh, campos, B, v, out); break;
      case 9: sh_forward_vertex<9>(verts, V, sh, campos, B, v, out); break;
      default: sh_forward_vertex<16>(verts, V, sh, campos, B, v, out); break;
    }
  }
}

// d sh_k = sum_b basis_k(dir_b) * d rgb_b * [rgb_b + 0.5 > 0]; the mask is
// read from the forward output (out > 0 exactly when the pre-clamp value is).
// Every row of the output is written (rows k >= n_coeff get zeros).
__global__ void sh_backward_kernel(const float* __restrict__ verts, int64_t V, int n_coeff, int C,
                                   const float* __restrict__ campos, int B, const float* __restrict__ colors,
                                   const float* __restrict__ dcolors, float* __restrict__ dsh) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    float acc[16][3];
    for (int k = 0; k < 16; ++k) acc[k][0] = acc[k][1] = acc[k][2] = 0.f;
    for (int b = 0; b < B; ++b) {
      const int64_t o = ((int64_t)b * V + v) * 3;
      float g[3];
      bool any = false;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        g[c] = colors[o + c] > 0.0f ? dcolors[o + c] : 0.0f;
        any |= g[c] != 0.0f;
      }
      if (!any) continue;
      float x, y, z;
      view_dir(verts, v, campos + 3 * b, x, y, z);
      float basis[16];
      sh_basis(x, y, z, n_coeff, basis);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        if (k < n_coeff) {
#pragma unroll
          for (int c = 0; c < 3; ++c) acc[k][c] += basis[k] * g[c];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k < C) {
        float* d = dsh + ((int64_t)k * V + v) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) d[c] = acc[k][c];
      }
    }
    for (int k = 16; k < C; ++k) {
      float* d = dsh + ((int64_t)k * V + v) * 3;
      d[0] = d[1] = d[2] = 0.f;
    }
  }
}

// ---------------------------------------------------------------------------
// bound_triangles.slang:62-192: back-face and near-plane culling, tile AABB
// with min = int(x) / ts (truncation), max = int(ceil(x / ts)), clamped.
// ---------------------------------------------------------------------------
struct TileBounds {
  int r0, c0, r1, c1;
};

// ymax / tile as the reference divides it: for a power-of-two tile the
// product with the exact reciprocal is the same correctly rounded quotient.
__device__ __forceinline__ float div_by_tile(float x, int tile) {
  if ((tile & (tile - 1)) == 0) return __fmul_rn(x, __int_as_float((127 - (__ffs(tile) - 1)) << 23));
  return __fdiv_rn(x, (float)tile);
}

// max(v / tile, 0) with C's truncating division; for a power-of-two tile a
// shift (flooring) differs only for negative v, where both clamp to 0.
__device__ __forceinline__ int first_tile(int v, int tile) {
  if ((tile & (tile - 1)) == 0) return max(v >> (__ffs(tile) - 1), 0);
  return max(v / tile, 0);
}

// Tile rectangle of one projected triangle; mean_depth receives
// (ad + bd + cd) / 3 (keys.slang's key depth) when the face is not culled.
__device__ __forceinline__ TileBounds bounds_from_corners(float ax, float ay, float ad, float bx, float by, float bd,
                                                          float cx, float cy, float cd, int tile_h, int tile_w,
                                                          int rows, int cols, float near, float& mean_depth) {
  TileBounds t{0, 0, 0, 0};
  const float check = __fsub_rn(__fmul_rn(__fsub_rn(bx, ax), __fsub_rn(cy, ay)),
                                __fmul_rn(__fsub_rn(by, ay), __fsub_rn(cx, ax)));
  if (check < 0.0f) return t;
  if (fminf(fminf(ad, bd), cd) < near) return t;
  mean_depth = __fdiv_rn(__fadd_rn(__fadd_rn(ad, bd), cd), 3.0f);
  const float ymin = fminf(fminf(ay, by), cy), ymax = fmaxf(fmaxf(ay, by), cy);
  const float xmin = fminf(fminf(ax, bx), cx), xmax = fmaxf(fmaxf(ax, bx), cx);
  t.r0 = min(first_tile(f2i_rz(ymin), tile_h), rows);
  t.r1 = min(max(f2i_rz(ceilf(div_by_tile(ymax, tile_h))), 0), rows);
  t.c0 = min(first_tile(f2i_rz(xmin), tile_w), cols);
  t.c1 = min(max(f2i_rz(ceilf(div_by_tile(xmax, tile_w))), 0), cols);
  return t;
}

__device__ __forceinline__ bool face_in_range(int32_t ia, int32_t ib, int32_t ic, int64_t V) {
  return (uint64_t)ia < (uint64_t)V && (uint64_t)ib < (uint64_t)V && (uint64_t)ic < (uint64_t)V;
}

__device__ __forceinline__ TileBounds triangle_tile_bounds(const float* __restrict__ xy,
                                                           const float* __restrict__ depth, int64_t V,
                                                           const int32_t* __restrict__ faces, int64_t f, int b,
                                                           int tile_h, int tile_w, int rows, int cols, float near,
                                                           float& mean_depth) {
  const int64_t base = (int64_t)b * V;
  const int32_t ia = faces[3 * f], ib = faces[3 * f + 1], ic = faces[3 * f + 2];
  // A face that names a vertex outside [0, V) (only possible when an upstream
  // capacity overflowed) covers no tile.
  if (!face_in_range(ia, ib, ic, V)) return TileBounds{0, 0, 0, 0};
  return bounds_from_corners(xy[2 * (base + ia)], xy[2 * (base + ia) + 1], depth[base + ia], xy[2 * (base + ib)],
                             xy[2 * (base + ib) + 1], depth[base + ib], xy[2 * (base + ic)], xy[2 * (base + ic) + 1],
                             depth[base + ic], tile_h, tile_w, rows, cols, near, mean_depth);
}

// Rows f >= num_faces (a device value; all F when NULL) cover no tile.
// cameras: NULL (every camera has rows x cols tiles) or the ragged camera
// table [B, 6] whose first two columns give each camera's own grid.
__global__ void bound_kernel(const float* __restrict__ xy, const float* __restrict__ depth, int64_t V,
                             const int32_t* __restrict__ faces, int64_t F, const int32_t* __restrict__ num_faces,
                             int B, int tile_h, int tile_w, int rows, int cols, const int64_t* __restrict__ cameras,
                             float near, int32_t* __restrict__ out_min, int32_t* __restrict__ out_max,
                             int32_t* __restrict__ out_count) {
  const int64_t total = (int64_t)B * F;
  const int64_t live = num_faces ? min((int64_t)max(*num_faces, 0), F) : F;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / F);
    const int64_t f = i - (int64_t)b * F;
    const int rb = cameras ? (int)cameras[6 * b] : rows, cb = cameras ? (int)cameras[6 * b + 1] : cols;
    float mean;
    const TileBounds t = f < live ? triangle_tile_bounds(xy, depth, V, faces, f, b, tile_h, tile_w, rb, cb, near, mean)
                                  : TileBounds{0, 0, 0, 0};
    out_min[2 * i] = t.r0;
    out_min[2 * i + 1] = t.c0;
    out_max[2 * i] = t.r1;
    out_max[2 * i + 1] = t.c1;
    out_count[i] = (t.r1 - t.r0) * (t.c1 - t.c0);
  }
}

// ---------------------------------------------------------------------------
// generate_keys.slang:4-68 + keys.slang:6-22. One thread per (camera, face);
// keys land at the exclusive offset of (camera, face) in row-major tile order,
// so the unsorted order (and therefore the stable sort's tie order) is the
// reference's.
// ---------------------------------------------------------------------------
struct KeyLayout {
  int cam_off, cam_len, shell_off, shell_len, tile_off, tile_len, depth_off;
};

__device__ __forceinline__ uint64_t field_mask(int len) { return (uint64_t)((1u << len) - 1u); }

__global__ void keys_kernel(const float* __restrict__ depth, int64_t V, const int32_t* __restrict__ faces,
                            int64_t F, const int32_t* __restrict__ sfb, int S, const int32_t* __restrict__ tmin,
                            const int32_t* __restrict__ tmax, const int64_t* __restrict__ offsets, int B,
                            int grid_width, const int64_t* __restrict__ cameras, KeyLayout L, int64_t K,
                            uint64_t* __restrict__ out_keys, int32_t* __restrict__ out_tri) {
  const int64_t total = (int64_t)B * F;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / F);
    const int64_t f = i - (int64_t)b * F;
    const int r0 = tmin[2 * i], c0 = tmin[2 * i + 1], r1 = tmax[2 * i], c1 = tmax[2 * i + 1];
    if (r1 <= r0 || c1 <= c0) continue;
    uint32_t shell = 0;
    for (; shell < (uint32_t)S; ++shell)
      if (f < sfb[shell]) break;
    const int64_t base = (int64_t)b * V;
    const float da = depth[base + faces[3 * f]], db = depth[base + faces[3 * f + 1]],
                dc = depth[base + faces[3 * f + 2]];
    const float mean = __fdiv_rn(__fadd_rn(__fadd_rn(da, db), dc), 3.0f);
    const uint64_t fixed = (((uint64_t)b & field_mask(L.cam_len)) << L.cam_off) |
                           (((uint64_t)shell & field_mask(L.shell_len)) << L.shell_off) |
                           ((uint64_t)__float_as_uint(mean) << L.depth_off);
    int64_t k = (i == 0) ? 0 : offsets[i - 1];
    const int width = cameras ? (int)cameras[6 * b + 1] : grid_width;  // tiles per row of this camera
    for (int r = r0; r < r1; ++r) {
      for (int c = c0; c < c1; ++c) {
        if (k >= K) return;  // guarded: offsets and K always agree for valid inputs
        const uint32_t tile = (uint32_t)(r * width + c);
        out_keys[k] = fixed | (((uint64_t)tile & field_mask(L.tile_len)) << L.tile_off);
        out_tri[k] = (int32_t)f;
        ++k;
      }
    }
  }
}

// Shell of face f: the first boundary above f (keys.slang's shell field).
__device__ __forceinline__ uint32_t face_shell(const int32_t* __restrict__ sfb, int S, int64_t f) {
  uint32_t shell = 0;
  for (; shell < (uint32_t)S; ++shell)
    if (f < sfb[shell]) break;
  return shell;
}

// ---------------------------------------------------------------------------
// Tile bounds, key offsets and keys for calls with a key capacity (nothing is
// read back). The keys and their order equal bound_kernel followed by an
// inclusive scan of the counts and keys_kernel: item i = (camera, face) in
// row-major order writes its keys at the sum of the counts of items < i.
//
// The B*F items are split into chunks of kFusedItems x kFusedThreads items,
// one CTA each, striped (item j * kFusedThreads + tid of the chunk) so that a
// warp's loads are adjacent. Three launches, no CTA waits on another:
//   chunk_bounds_kernel  each item's tile rectangle (int4) and key depth into
//                        workspace records, and each chunk's key count;
//   chunk_scan_kernel    one CTA: exclusive scan of the chunk counts, and the
//                        total key count;
//   chunk_keys_kernel    reads its chunk's records back (coalesced), scans
//                        them and writes the keys load-balanced.
// ---------------------------------------------------------------------------
constexpr int kFusedThreads = 256;
constexpr int kFusedItems = 4;
constexpr int kFusedSubTile = kFusedThreads * kFusedItems;
constexpr int kChunkScanThreads = 1024;
// Workspace: [0,256) status word (unused here), chunk counts (int64 per
// chunk), the rectangle records (int4 per item), the key depths (float per
// item); each region starts on a 256-byte boundary.
constexpr size_t kFusedHeader = 256;

__host__ __device__ inline size_t round256(size_t x) { return (x + 255) / 256 * 256; }

struct FusedArgs {
  const float* xy;
  const float* depth;
  int64_t V;
  const int32_t* faces;
  int64_t F;
  const int32_t* num_faces;
  int B, tile_h, tile_w, rows, cols;
  const int64_t* cameras;
  float near;
  int64_t chunk;  // items per chunk (a multiple of kFusedSubTile)
};

// Bounds (and key depth) of this thread's kFusedItems items of the sub-tile
// starting at item `first`, loads of all items issued together.
__device__ __forceinline__ void subtile_bounds(const FusedArgs& a, int64_t first, int64_t end, int64_t live,
                                               int (&cam)[kFusedItems], int64_t (&face)[kFusedItems],
                                               TileBounds (&t)[kFusedItems], float (&mean)[kFusedItems]) {
  {
    const int64_t i0 = first + threadIdx.x;
    int b = (int)(i0 / a.F);
    int64_t f = i0 - (int64_t)b * a.F;
#pragma unroll
    for (int j = 0; j < kFusedItems; ++j) {
      // Items at or past `end` (the chunk's end or B*F) get camera B.
      cam[j] = (i0 + (int64_t)j * kFusedThreads < end) ? b : a.B;
      face[j] = f;
      f += kFusedThreads;
      while (f >= a.F) {
        f -= a.F;
        ++b;
      }
    }
  }
  int32_t corner[kFusedItems][3];
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    const bool ok = cam[j] < a.B && face[j] < live;
#pragma unroll
    for (int c = 0; c < 3; ++c) corner[j][c] = ok ? __ldg(a.faces + 3 * face[j] + c) : -1;
  }
  float2 p[kFusedItems][3];
  float d[kFusedItems][3];
  bool ok[kFusedItems];
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    ok[j] = face_in_range(corner[j][0], corner[j][1], corner[j][2], a.V);
    const int64_t base = (int64_t)cam[j] * a.V;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t v = base + (ok[j] ? corner[j][c] : 0);
      p[j][c] = ok[j] ? __ldg(reinterpret_cast<const float2*>(a.xy) + v) : make_float2(0.f, 0.f);
      d[j][c] = ok[j] ? __ldg(a.depth + v) : 0.f;
    }
  }
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    t[j] = TileBounds{0, 0, 0, 0};
    mean[j] = 0.0f;
    if (ok[j]) {
      const int rb = a.cameras ? (int)a.cameras[6 * cam[j]] : a.rows;
      const int cb = a.cameras ? (int)a.cameras[6 * cam[j] + 1] : a.cols;
      t[j] = bounds_from_corners(p[j][0].x, p[j][0].y, d[j][0], p[j][1].x, p[j][1].y, d[j][1], p[j][2].x, p[j][2].y,
                                 d[j][2], a.tile_h, a.tile_w, rb, cb, a.near, mean[j]);
    }
  }
}

// The int32 count of bound_kernel, widened as the scan widens it.
__device__ __forceinline__ int64_t tile_count(const TileBounds& t) {
  return (int64_t)((t.r1 - t.r0) * (t.c1 - t.c0));
}

template <typename T>
__device__ __forceinline__ T block_sum(T x, T* s_warp) {
  x = warp_sum(x);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = x;
  __syncthreads();
  T total = 0;
#pragma unroll
  for (int w = 0; w < kFusedThreads / 32; ++w) total += s_warp[w];
  return total;
}

__global__ void __launch_bounds__(kFusedThreads, 3)
    chunk_bounds_kernel(FusedArgs a, int4* __restrict__ rect, float* __restrict__ key_depth,
                        int64_t* __restrict__ chunk_counts) {
  __shared__ int64_t s_warp[kFusedThreads / 32];
  const int64_t items = (int64_t)a.B * a.F;
  const int64_t first = blockIdx.x * a.chunk, end = min(first + a.chunk, items);
  const int64_t live = a.num_faces ? min((int64_t)max(*a.num_faces, 0), a.F) : a.F;
  int64_t sum = 0;
  for (int64_t sub = first; sub < end; sub += kFusedSubTile) {
    int cam[kFusedItems];
    int64_t face[kFusedItems];
    TileBounds t[kFusedItems];
    float mean[kFusedItems];
    subtile_bounds(a, sub, end, live, cam, face, t, mean);
#pragma unroll
    for (int j = 0; j < kFusedItems; ++j) {
      const int64_t i = sub + (int64_t)j * kFusedThreads + threadIdx.x;
      if (i < end) {
        rect[i] = make_int4(t[j].r0, t[j].c0, t[j].r1, t[j].c1);
        key_depth[i] = mean[j];
      }
      sum += tile_count(t[j]);
    }
  }
  const int64_t total = block_sum(sum, s_warp);
  if (threadIdx.x == 0) chunk_counts[blockIdx.x] = total;
}

// Exclusive scan of the chunk counts in place (one CTA); *out_count = total.
// Rounds of kChunkScanThreads x 4 counts, each thread's four loaded together.
__global__ void __launch_bounds__(kChunkScanThreads)
    chunk_scan_kernel(int64_t* __restrict__ counts, int64_t chunks, int64_t* __restrict__ out_count) {
  constexpr int kPer = 4;
  __shared__ int64_t s_warp[kChunkScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int64_t running = 0;
  for (int64_t base = 0; base < chunks; base += (int64_t)kChunkScanThreads * kPer) {
    const int64_t c0 = base + (int64_t)tid * kPer;
    int64_t x[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) x[k] = c0 + k < chunks ? counts[c0 + k] : 0;
    int64_t mine = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) mine += x[k];
    const int64_t inc = warp_inclusive_sum(mine);
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    int64_t below = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kChunkScanThreads / 32; ++w) {
      const int64_t y = s_warp[w];
      all += y;
      below += (w < warp) ? y : 0;
    }
    int64_t run = running + below + inc - mine;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      if (c0 + k < chunks) counts[c0 + k] = run;
      run += x[k];
    }
    running += all;
    __syncthreads();
  }
  if (tid == 0) *out_count = running;
}

// Each thread writes the keys of its own items (in row-major tile order, at
// the item's exclusive offset: the chunk's offset + the CTA scan of the
// counts), as keys_kernel does, from the records instead of gathers.
__global__ void __launch_bounds__(kFusedThreads)
    chunk_keys_kernel(FusedArgs a, const int4* __restrict__ rect, const float* __restrict__ key_depth,
                      const int64_t* __restrict__ chunk_offsets, const int32_t* __restrict__ sfb, int S,
                      KeyLayout L, int64_t K, uint64_t* __restrict__ out_keys, int32_t* __restrict__ out_tri) {
  __shared__ int64_t s_warp[kFusedItems][kFusedThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t items = (int64_t)a.B * a.F;
  const int64_t sub = (int64_t)blockIdx.x * kFusedSubTile;
  const int64_t end = min(sub + kFusedSubTile, items);
  TileBounds t[kFusedItems];
  float kd[kFusedItems];
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    const int64_t i = sub + (int64_t)j * kFusedThreads + tid;
    const int4 r = i < end ? __ldcs(rect + i) : make_int4(0, 0, 0, 0);
    kd[j] = i < end ? __ldcs(key_depth + i) : 0.0f;
    t[j] = TileBounds{r.x, r.y, r.z, r.w};
  }
  int64_t inc[kFusedItems];
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    inc[j] = warp_inclusive_sum(tile_count(t[j]));
    if (lane == 31) s_warp[j][warp] = inc[j];
  }
  __syncthreads();
  int64_t base = chunk_offsets[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    int64_t below = 0, row = 0;
#pragma unroll
    for (int w = 0; w < kFusedThreads / 32; ++w) {
      const int64_t x = s_warp[j][w];
      row += x;
      below += (w < warp) ? x : 0;
    }
    inc[j] += base + below;  // inclusive offset of item j
    base += row;
  }
  int b;
  int64_t f;
  {
    const int64_t i0 = sub + tid;
    b = (int)(i0 / a.F);
    f = i0 - (int64_t)b * a.F;
  }
#pragma unroll
  for (int j = 0; j < kFusedItems; ++j) {
    const TileBounds& tb = t[j];
    if (tb.r1 > tb.r0 && tb.c1 > tb.c0) {
      int64_t k = inc[j] - tile_count(tb);
      const uint64_t fixed = (((uint64_t)b & field_mask(L.cam_len)) << L.cam_off) |
                             (((uint64_t)face_shell(sfb, S, f) & field_mask(L.shell_len)) << L.shell_off) |
                             ((uint64_t)__float_as_uint(kd[j]) << L.depth_off);
      const int width = a.cameras ? (int)a.cameras[6 * b + 1] : a.cols;
      for (int r = tb.r0; r < tb.r1 && k < K; ++r) {
        for (int c = tb.c0; c < tb.c1; ++c) {
          if (k >= K || k < 0) break;  // past the capacity
          const uint32_t tile_index = (uint32_t)(r * width + c);
          out_keys[k] = fixed | (((uint64_t)tile_index & field_mask(L.tile_len)) << L.tile_off);
          out_tri[k] = (int32_t)f;
          ++k;
        }
      }
    }
    f += kFusedThreads;
    while (f >= a.F) {
      f -= a.F;
      ++b;
    }
  }
}

// ---------------------------------------------------------------------------
// delineate_tiles.slang:14-58: [start, end) per (camera, shell|0, tile) where
// the (camera, shell|0, tile) index changes between consecutive sorted keys.
// ---------------------------------------------------------------------------
__global__ void delineate_kernel(const uint64_t* __restrict__ keys, int64_t K_capacity,
                                 const int64_t* __restrict__ num_keys, KeyLayout L, int separate_shells, int B,
                                 int Sd, int64_t T, int64_t* __restrict__ out) {
  const int64_t K = num_keys ? min(max(*num_keys, (int64_t)0), K_capacity) : K_capacity;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < K; i += (int64_t)gridDim.x * blockDim.x) {
    auto index_of = [&](uint64_t key) -> int64_t {
      const int64_t cam = (int64_t)((key >> L.cam_off) & field_mask(L.cam_len));
      const int64_t sh = separate_shells ? (int64_t)((key >> L.shell_off) & field_mask(L.shell_len)) : 0;
      const int64_t tile = (int64_t)((key >> L.tile_off) & field_mask(L.tile_len));
      if (cam >= B || sh >= Sd || tile >= T) return -1;
      return (cam * Sd + sh) * T + tile;
    };
    const int64_t here = index_of(keys[i]);
    if (i > 0) {
      const int64_t prev = index_of(keys[i - 1]);
      if (here != prev) {
        if (prev >= 0) out[2 * prev + 1] = i;
        if (here >= 0) out[2 * here] = i;
      }
    }
    if (i == K - 1 && here >= 0) out[2 * here + 1] = K;
  }
}

inline bool layout_ok(const KeyLayout& L) {
  auto ok = [](int off, int len) { return off >= 0 && len >= 0 && len <= 31 && off + len <= 64; };
  return ok(L.cam_off, L.cam_len) && ok(L.shell_off, L.shell_len) && ok(L.tile_off, L.tile_len) &&
         L.depth_off >= 0 && L.depth_off + 32 <= 64;
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

int mt_camera_positions(const float* extrinsics, int32_t B, float* out, mt_stream_t stream) {
  MT_REQUIRE(B >= 0);
  if (B == 0) return MT_OK;
  MT_REQUIRE(extrinsics && out);
  camera_positions_kernel<<<grid_1d((int64_t)B * 32, 128), 128, 0, as_stream(stream)>>>(extrinsics, B, out);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_project_vertices(const float* vertices, int64_t V, const float* extrinsics, const float* intrinsics, int32_t B,
                        float* out_xy, float* out_depth, mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && B >= 0);
  if (V == 0 || B == 0) return MT_OK;
  MT_REQUIRE(vertices && extrinsics && intrinsics && out_xy && out_depth);
  project_kernel<<<grid_stride_blocks(V, 256), 256, 0, as_stream(stream)>>>(vertices, V, extrinsics, intrinsics, B,
                                                                           out_xy, out_depth);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_evaluate_spherical_harmonics(const float* vertices, int64_t V, const float* spherical_harmonics, int32_t C,
                                    int32_t sh_degree, const float* camera_positions, int32_t B, float* out_colors,
                                    mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && B >= 0 && sh_degree >= 0 && sh_degree <= 3);
  const int n = (sh_degree + 1) * (sh_degree + 1);
  MT_REQUIRE(C >= n);
  if (V == 0 || B == 0) return MT_OK;
  MT_REQUIRE(vertices && spherical_harmonics && camera_positions && out_colors);
  sh_forward_kernel<<<grid_stride_blocks(V, 256), 256, 0, as_stream(stream)>>>(vertices, V, spherical_harmonics, n,
                                                                              camera_positions, B, out_colors);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_evaluate_spherical_harmonics_backward(const float* vertices, int64_t V, int32_t C, int32_t sh_degree,
                                             const float* camera_positions, int32_t B, const float* out_colors,
                                             const float* grad_colors, float* grad_spherical_harmonics,
                                             mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && B >= 0 && sh_degree >= 0 && sh_degree <= 3);
  const int n = (sh_degree + 1) * (sh_degree + 1);
  MT_REQUIRE(C >= n);
  if (V == 0) return MT_OK;
  MT_REQUIRE(grad_spherical_harmonics);
  if (B == 0) {
    const size_t bytes = (size_t)C * (size_t)V * 3 * sizeof(float);
    return cudaMemsetAsync(grad_spherical_harmonics, 0, bytes, as_stream(stream)) == cudaSuccess ? MT_OK : MT_ERR_CUDA;
  }
  MT_REQUIRE(vertices && camera_positions && out_colors && grad_colors);
  sh_backward_kernel<<<grid_stride_blocks(V, 128), 128, 0, as_stream(stream)>>>(
      vertices, V, n, C, camera_positions, B, out_colors, grad_colors, grad_spherical_harmonics);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_bound_triangles(const float* xy, const float* depth, int64_t V, const int32_t* faces, int64_t F,
                       const int32_t* num_faces, int32_t B, int32_t tile_h, int32_t tile_w, int32_t rows,
                       int32_t cols, const int64_t* cameras, float near_plane, int32_t* out_min, int32_t* out_max,
                       int32_t* out_count, mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && F >= 0 && B >= 0 && tile_h > 0 && tile_w > 0 && rows >= 0 && cols >= 0);
  if (F == 0 || B == 0) return MT_OK;
  MT_REQUIRE(xy && depth && faces && out_min && out_max && out_count);
  bound_kernel<<<grid_stride_blocks((int64_t)B * F, 256), 256, 0, as_stream(stream)>>>(
      xy, depth, V, faces, F, num_faces, B, tile_h, tile_w, rows, cols, cameras, near_plane, out_min, out_max,
      out_count);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_generate_keys(const float* depth, int64_t V, const int32_t* faces, int64_t F,
                     const int32_t* shell_face_boundaries, int32_t S, const int32_t* tile_min,
                     const int32_t* tile_max, const int64_t* offsets, int32_t B, int32_t grid_width,
                     const int64_t* cameras, const int32_t* layout, int64_t K, int64_t* out_keys,
                     int32_t* out_triangles, mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && F >= 0 && B >= 0 && S >= 0 && K >= 0 && layout);
  KeyLayout L{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], layout[6]};
  MT_REQUIRE(layout_ok(L));
  if (F == 0 || B == 0 || K == 0) return MT_OK;
  MT_REQUIRE(depth && faces && tile_min && tile_max && offsets && out_keys && out_triangles);
  MT_REQUIRE(S == 0 || shell_face_boundaries);
  keys_kernel<<<grid_stride_blocks((int64_t)B * F, 256), 256, 0, as_stream(stream)>>>(
      depth, V, faces, F, shell_face_boundaries, S, tile_min, tile_max, offsets, B, grid_width, cameras, L, K,
      reinterpret_cast<uint64_t*>(out_keys), out_triangles);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

static int64_t fused_chunks(int64_t items) { return (items + kFusedSubTile - 1) / kFusedSubTile; }

size_t mt_bound_and_generate_keys_workspace_bytes(int64_t items) {
  if (items < 0) items = 0;
  return kFusedHeader + round256((size_t)fused_chunks(items) * sizeof(int64_t)) +
         round256((size_t)items * sizeof(int4)) + (size_t)items * sizeof(float);
}

int mt_bound_and_generate_keys(const float* xy, const float* depth, int64_t V, const int32_t* faces, int64_t F,
                               const int32_t* num_faces, const int32_t* shell_face_boundaries, int32_t S, int32_t B,
                               int32_t tile_h, int32_t tile_w, int32_t rows, int32_t cols, const int64_t* cameras,
                               float near_plane, const int32_t* layout, int64_t K, int64_t* out_keys,
                               int32_t* out_triangles, int64_t* out_num_keys, void* workspace, size_t workspace_bytes,
                               mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && F >= 0 && B >= 0 && S >= 0 && K >= 0 && layout);
  MT_REQUIRE(tile_h > 0 && tile_w > 0 && rows >= 0 && cols >= 0);
  KeyLayout L{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], layout[6]};
  MT_REQUIRE(layout_ok(L));
  MT_REQUIRE(out_num_keys);
  const cudaStream_t s = as_stream(stream);
  const int64_t items = (int64_t)B * F;
  if (items == 0)
    return cudaMemsetAsync(out_num_keys, 0, sizeof(int64_t), s) == cudaSuccess ? MT_OK : MT_ERR_CUDA;
  MT_REQUIRE(xy && depth && faces && workspace);
  MT_REQUIRE((reinterpret_cast<uintptr_t>(xy) & 7) == 0);  // positions are read as float2
  MT_REQUIRE(K == 0 || (out_keys && out_triangles));
  MT_REQUIRE(S == 0 || shell_face_boundaries);
  if (workspace_bytes < mt_bound_and_generate_keys_workspace_bytes(items)) return MT_ERR_WORKSPACE_TOO_SMALL;
  const int64_t chunks = fused_chunks(items);
  MT_REQUIRE(chunks < (int64_t)0x7fffffff);
  FusedArgs a{xy, depth, V, faces, F, num_faces, B, tile_h, tile_w, rows, cols, cameras, near_plane, kFusedSubTile};
  MT_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 15) == 0);
  char* base = static_cast<char*>(workspace);
  int64_t* counts = reinterpret_cast<int64_t*>(base + kFusedHeader);
  int4* rect = reinterpret_cast<int4*>(base + kFusedHeader + round256((size_t)chunks * sizeof(int64_t)));
  float* key_depth = reinterpret_cast<float*>(reinterpret_cast<char*>(rect) + round256((size_t)items * sizeof(int4)));
  chunk_bounds_kernel<<<(unsigned)chunks, kFusedThreads, 0, s>>>(a, rect, key_depth, counts);
  MT_CHECK_LAUNCH();
  chunk_scan_kernel<<<1, kChunkScanThreads, 0, s>>>(counts, chunks, out_num_keys);
  MT_CHECK_LAUNCH();
  chunk_keys_kernel<<<(unsigned)chunks, kFusedThreads, 0, s>>>(a, rect, key_depth, counts, shell_face_boundaries, S,
                                                               L, K, reinterpret_cast<uint64_t*>(out_keys),
                                                               out_triangles);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_delineate_tiles(const int64_t* sorted_keys, int64_t K, const int64_t* num_keys, const int32_t* layout,
                       int32_t separate_shells, int32_t B, int32_t shell_dim, int64_t num_tiles,
                       int64_t* out_boundaries, mt_stream_t stream) {
  MT_REQUIRE(K >= 0 && B >= 0 && shell_dim >= 1 && num_tiles >= 0 && layout);
  KeyLayout L{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], layout[6]};
  MT_REQUIRE(layout_ok(L));
  const size_t bytes = (size_t)B * shell_dim * num_tiles * 2 * sizeof(int64_t);
  if (bytes == 0) return MT_OK;
  MT_REQUIRE(out_boundaries);
  if (cudaMemsetAsync(out_boundaries, 0, bytes, as_stream(stream)) != cudaSuccess) return MT_ERR_CUDA;
  if (K == 0) return MT_OK;
  MT_REQUIRE(sorted_keys);
  delineate_kernel<<<grid_stride_blocks(K, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const uint64_t*>(sorted_keys), K, num_keys, L, separate_shells, B, shell_dim, num_tiles,
      out_boundaries);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
