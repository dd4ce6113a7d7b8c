// Sparse-voxel extraction and per-step marching cubes for sm_103a.
//
// Voxel topology (extract_voxels) follows triangle_extraction/
// compute_vertex_occupancy.slang, count_occupancy.slang, create_voxels.slang
// and dilate_occupancy.slang; per-step tessellation follows
// count_triangle_vertices.slang, create_triangle_vertices.slang,
// count_triangle_faces.slang and create_triangle_faces.slang.
//
// Layout choices: every per-word kernel indexes the packed k axis fastest so
// a warp reads consecutive words; create_voxels runs one warp per packed word
// with lane = bit, turning the reference's serial 32-bit walk into warp-ballot
// stream compaction (popcount of the lanes below); all [*, G] / [*, Nv] tables
// are read one row at a time so every row read is coalesced.
//
// For the captured training step the per-vertex SH rows can be skipped: the
// grid-SH colour kernels evaluate vertex colours straight from the grid
// coefficients (evaluate_spherical_harmonics.slang with the interpolation of
// create_triangle_vertices.slang) and send the SH gradient straight back to
// the grid through the per-grid-vertex contribution list, with the same bits
// as the row path.

#include "mc_tables.h"
#include "mt_common.cuh"
#include "sh.cuh"

namespace mt {
namespace {

__constant__ uint8_t c_mc_count[256] = {MT_MC_CASE_COUNT_VALUES};
__constant__ uint64_t c_mc_edges[256] = {MT_MC_CASE_EDGES_VALUES};
__constant__ int8_t c_mc_owner[12] = {MT_MC_EDGE_OWNER_VALUES};
__constant__ uint8_t c_mc_axis[12] = {MT_MC_EDGE_AXIS_VALUES};

// ---------------------------------------------------------------------------
// compute_vertex_occupancy.slang:9-68
// ---------------------------------------------------------------------------
__global__ void vertex_occupancy_kernel(const int32_t* __restrict__ occ, int I, int J, int KP,
                                        int32_t* __restrict__ vocc, int32_t* __restrict__ vcounts) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int kp = (int)(w % (KP + 1));
    const int64_t ij = w / (KP + 1);
    const int j = (int)(ij % (J + 1));
    const int i = (int)(ij / (J + 1));
    uint32_t result = 0;
#pragma unroll
    for (int di = 0; di < 2; ++di) {
#pragma unroll
      for (int dj = 0; dj < 2; ++dj) {
        if ((i == 0 && di == 1) || (j == 0 && dj == 1)) continue;
        if ((i == I && di == 0) || (j == J && dj == 0)) continue;
        const int64_t row = ((int64_t)(i - di) * J + (j - dj)) * KP;
        const uint32_t cur = (kp == KP) ? 0u : (uint32_t)occ[row + kp];
        const uint32_t prev_packed = (kp == 0) ? 0u : (uint32_t)occ[row + kp - 1];
        result |= cur | ((prev_packed >> 31) | (cur << 1));
      }
    }
    vocc[w] = (int32_t)result;
    vcounts[w] = __popc(result);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) vcounts[total] = 0;
}

// count_occupancy.slang:3-20 plus the zero fill of count_occupancy.py:30.
__global__ void count_occupancy_kernel(const int32_t* __restrict__ occ, int I, int J, int KP,
                                       int32_t* __restrict__ counts) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int kp = (int)(w % (KP + 1));
    const int64_t ij = w / (KP + 1);
    const int j = (int)(ij % (J + 1));
    const int i = (int)(ij / (J + 1));
    int c = 0;
    if (i < I && j < J && kp < KP) c = __popc((uint32_t)occ[((int64_t)i * J + j) * KP + kp]);
    counts[w] = c;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counts[total] = 0;
}

// ---------------------------------------------------------------------------
// create_voxels.slang:3-276, one warp per vertex-grid word, lane = bit.
// ---------------------------------------------------------------------------
struct VoxelGrid {
  const int32_t* occ;   // [I, J, KP]
  const int32_t* xoff;  // [I+1, J+1, KP+1] voxel offsets
  const int32_t* vocc;  // [I+1, J+1, KP+1]
  const int32_t* voff;  // [I+1, J+1, KP+1] vertex offsets
  int I, J, KP;
  int64_t Nv;

  __device__ __forceinline__ int64_t vw(int i, int j, int kp) const {
    return ((int64_t)i * (J + 1) + j) * (KP + 1) + kp;
  }
  // Voxel occupancy word; 0 outside the voxel grid.
  __device__ __forceinline__ uint32_t vx(int i, int j, int kp) const {
    if (i >= I || j >= J || kp >= KP) return 0u;
    return (uint32_t)occ[((int64_t)i * J + j) * KP + kp];
  }
};

// Per-neighbour-word state at a given bit: the reference's local_* arrays.
struct WordState {
  int32_t vidx, xidx, sidx;  // indices of the entry at this bit (-64 when out of range)
  uint32_t vo, vx, so;       // vertex / voxel / subvoxel occupancy words
};

__device__ __forceinline__ WordState word_state(const VoxelGrid& g, int i, int j, int kp, uint32_t below) {
  WordState s;
  if (i > g.I || j > g.J) {
    s.vidx = s.xidx = s.sidx = -64;
    s.vo = s.vx = s.so = 0u;
    return s;
  }
  const int64_t w = g.vw(i, j, kp);
  s.vo = (uint32_t)g.vocc[w];
  s.vx = g.vx(i, j, kp);
  s.so = s.vo & ~s.vx;
  const int32_t xo = g.xoff[w], vo = g.voff[w];
  s.vidx = vo + __popc(s.vo & below);
  s.xidx = xo + __popc(s.vx & below);
  s.sidx = (int32_t)g.Nv + (vo - xo) + __popc(s.so & below);
  return s;
}

__device__ __forceinline__ int32_t pick_diag(bool diag_sub, bool side_sub, const WordState& s) {
  // Neighbour one step along +x from a side neighbour (see create_voxels.slang:164-172).
  return diag_sub ? (side_sub ? s.sidx + 1 : s.sidx) : (side_sub ? s.xidx : s.xidx + 1);
}

__global__ void create_voxels_kernel(VoxelGrid g, float* __restrict__ vertices, int32_t* __restrict__ neighbors,
                                     int32_t* __restrict__ lower, int32_t* __restrict__ upper,
                                     int32_t* __restrict__ indices, int64_t G) {
  const int lane = threadIdx.x & 31;
  const int64_t warps_total = (int64_t)(g.I + 1) * (g.J + 1) * (g.KP + 1);
  const int64_t warp_global = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t warp_stride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t below = (1u << lane) - 1u;
  const uint32_t bit = 1u << lane;
  const int64_t Nv = g.Nv;
  const float inv_i = 1.0f / (float)g.I;
  const float inv_j = 1.0f / (float)g.J;
  const float inv_k = 1.0f / (float)(32 * g.KP);
  const int32_t k_max = 32 * g.KP;

  for (int64_t w = warp_global; w < warps_total; w += warp_stride) {
    const int kp = (int)(w % (g.KP + 1));
    const int64_t ij = w / (g.KP + 1);
    const int j = (int)(ij % (g.J + 1));
    const int i = (int)(ij / (g.J + 1));
    const uint32_t vo00 = (uint32_t)g.vocc[w];
    if (vo00 == 0u) continue;  // warp-uniform
    const int k = 32 * kp + lane;

    const WordState s00 = word_state(g, i, j, kp, below);
    const WordState s01 = word_state(g, i, j + 1, kp, below);
    const WordState s10 = word_state(g, i + 1, j, kp, below);
    const WordState s11 = word_state(g, i + 1, j + 1, kp, below);

    // Vertices (create_voxels.slang:37-53).
    if (vo00 & bit) {
      float* v = vertices + (int64_t)s00.vidx * 3;
      v[0] = (float)k * inv_k;
      v[1] = (float)j * inv_j;
      v[2] = (float)i * inv_i;
    }

    const bool is_voxel = (s00.vx & bit) != 0u;
    const bool is_sub = (s00.so & bit) != 0u;
    if (!is_voxel && !is_sub) continue;

    // Lower corners (create_voxels.slang:108-127, last bit fixed up at :201-206).
    const int32_t chosen = is_voxel ? s00.xidx : s00.sidx;
    bool x_valid;
    if (lane < 31) {
      x_valid = is_voxel || ((s00.vo >> (lane + 1)) & 1u);
    } else {
      x_valid = is_voxel || (kp < g.KP && (g.vocc[g.vw(i, j, kp + 1)] & 1));
    }
    const bool y_valid = is_voxel || (s01.vo & bit);
    const bool z_valid = is_voxel || (s10.vo & bit);
    lower[chosen] = s00.vidx;
    lower[G + chosen] = x_valid ? s00.vidx + 1 : -64;
    lower[2 * G + chosen] = y_valid ? s01.vidx : -64;
    lower[3 * G + chosen] = z_valid ? s10.vidx : -64;

    if (!is_voxel) continue;
    const int32_t vi = s00.xidx;

    // Upper corners and linear index (create_voxels.slang:129-136).
    upper[vi] = s11.vidx + 1;
    upper[Nv + vi] = s11.vidx;
    upper[2 * Nv + vi] = s10.vidx + 1;
    upper[3 * Nv + vi] = s01.vidx + 1;
    indices[vi] = k_max * (g.J * i + j) + k;

    // Neighbours (create_voxels.slang:138-193 for bits 0..30, :211-275 for bit 31).
    bool x_sub, y_sub, z_sub, xy_sub, yz_sub, xz_sub, xyz_sub;
    if (lane < 31) {
      const uint32_t nb = bit << 1;
      x_sub = (s00.so & nb) != 0u;
      y_sub = (s01.so & bit) != 0u;
      z_sub = (s10.so & bit) != 0u;
      xy_sub = (s01.so & nb) != 0u;
      yz_sub = (s11.so & bit) != 0u;
      xz_sub = (s10.so & nb) != 0u;
      xyz_sub = (s11.so & nb) != 0u;
    } else {
      const bool cx = kp < g.KP - 1, cy = j < g.J - 1, cz = i < g.I - 1;
      const uint32_t top = 1u << 31;
      x_sub = cx ? ((g.vx(i, j, kp + 1) & 1u) == 0u) : true;
      y_sub = cy ? ((g.vx(i, j + 1, kp) & top) == 0u) : true;
      z_sub = cz ? ((g.vx(i + 1, j, kp) & top) == 0u) : true;
      xy_sub = (cx && cy) ? ((g.vx(i, j + 1, kp + 1) & 1u) == 0u) : true;
      yz_sub = (cy && cz) ? ((g.vx(i + 1, j + 1, kp) & top) == 0u) : true;
      xz_sub = (cx && cz) ? ((g.vx(i + 1, j, kp + 1) & 1u) == 0u) : true;
      xyz_sub = (cx && cy && cz) ? ((g.vx(i + 1, j + 1, kp + 1) & 1u) == 0u) : true;
    }
    neighbors[vi] = x_sub ? s00.sidx : s00.xidx + 1;
    neighbors[Nv + vi] = y_sub ? s01.sidx : s01.xidx;
    neighbors[2 * Nv + vi] = z_sub ? s10.sidx : s10.xidx;
    neighbors[3 * Nv + vi] = pick_diag(xy_sub, y_sub, s01);
    neighbors[4 * Nv + vi] = yz_sub ? s11.sidx : s11.xidx;
    neighbors[5 * Nv + vi] = pick_diag(xz_sub, z_sub, s10);
    neighbors[6 * Nv + vi] = pick_diag(xyz_sub, yz_sub, s11);
  }
}

// ---------------------------------------------------------------------------
// dilate_occupancy.slang:9-94 (box dilation, 0 < d < 32).
// ---------------------------------------------------------------------------
__global__ void dilate_kernel(const int32_t* __restrict__ occ, int I, int J, int KP, int d,
                              int32_t* __restrict__ out) {
  const int64_t total = (int64_t)I * J * KP;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int kp = (int)(w % KP);
    const int64_t ij = w / KP;
    const int j = (int)(ij % J);
    const int i = (int)(ij / J);
    uint32_t prev = 0, cur = 0, next = 0;
    const int i0 = max(i - d, 0), i1 = min(i + d, I - 1);
    const int j0 = max(j - d, 0), j1 = min(j + d, J - 1);
    for (int ii = i0; ii <= i1; ++ii) {
      for (int jj = j0; jj <= j1; ++jj) {
        const int32_t* row = occ + ((int64_t)ii * J + jj) * KP;
        cur |= (uint32_t)row[kp];
        if (kp > 0) prev |= (uint32_t)row[kp - 1];
        if (kp < KP - 1) next |= (uint32_t)row[kp + 1];
      }
    }
    uint32_t result = cur;
    // Bits that spill in from the previous word (dilate_occupancy.slang:41-44).
    if (kp > 0) {
      uint32_t p = prev >> (32 - d);
      for (int b = 0; b < d; ++b) {
        result |= p;
        p >>= 1;
      }
    }
    uint32_t l = cur, r = cur;
    for (int b = 0; b < d; ++b) {
      r >>= 1;
      l <<= 1;
      result |= l | r;
    }
    if (kp < KP - 1) {
      uint32_t n = next << (32 - d);
      for (int b = 0; b < d; ++b) {
        result |= n;
        n <<= 1;
      }
    }
    out[w] = (int32_t)result;
  }
}

// ---------------------------------------------------------------------------
// count_triangle_vertices.slang:3-37
// ---------------------------------------------------------------------------
struct Corners4 {
  float d0, d[3];
  int32_t idx[3];  // lower_corners[1..3], may be negative
};

__device__ __forceinline__ Corners4 load_corners(const float* __restrict__ sdf, const int32_t* __restrict__ lower,
                                                 int64_t G, int64_t g) {
  Corners4 c;
  const int32_t i0 = __ldg(lower + g);
  c.d0 = __ldg(sdf + i0);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int32_t ia = __ldg(lower + (a + 1) * G + g);
    c.idx[a] = ia;
    c.d[a] = (ia >= 0) ? __ldg(sdf + ia) : c.d0;
  }
  return c;
}

__global__ void count_vertices_kernel(const float* __restrict__ sdf, const int32_t* __restrict__ lower, int64_t G,
                                      const float* __restrict__ level_sets, int S, int32_t* __restrict__ counts) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
    const Corners4 c = load_corners(sdf, lower, G, g);
    for (int s = 0; s < S; ++s) {
      const float iso = __ldg(level_sets + s);
      const bool b0 = c.d0 < iso;
      counts[(int64_t)s * G + g] = (b0 != (c.d[0] < iso)) + (b0 != (c.d[1] < iso)) + (b0 != (c.d[2] < iso));
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counts[(int64_t)S * G] = 0;
}

// Bit a of the result: edge `a` of entry g crosses level set `iso`. The same
// predicate sizes the outputs (count) and places vertices (create), so the
// writes always stay inside the counted range.
__device__ __forceinline__ uint32_t crossing_mask(const Corners4& c, float iso) {
  const bool b0 = c.d0 < iso;
  return (uint32_t)(b0 != (c.d[0] < iso)) | ((uint32_t)(b0 != (c.d[1] < iso)) << 1) |
         ((uint32_t)(b0 != (c.d[2] < iso)) << 2);
}

// create_triangle_vertices.slang:87-96: t is detached; positions / SH / sdf
// are linear in the corner values with weights (1 - t, t).
__device__ __forceinline__ float mc_weight(float d0, float d1, float iso) {
  if (d0 == d1) return 0.5f;
  const float t = (iso - d0) / (d1 - d0);
  return fminf(fmaxf(t, 0.0f), 1.0f);
}

// a + t * (b - a), rounded after each operation as the reference source
// writes it (create_triangle_vertices.slang:105-127).
__device__ __forceinline__ float lerp_ref(float a, float b, float t) {
  return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}

// ---------------------------------------------------------------------------
// create_triangle_vertices.slang:145-199 (forward), in two passes.
//
// Pass 1, one thread per entry g: positions, signed distance and type of
// every vertex on g's crossing edges, plus the vertex's source record
// (origin corner, axis corner, t) in vertex order.
// Pass 2, one thread per (coefficient row k, vertex): the SH row k of the
// vertex from its two corners. Consecutive threads write consecutive
// vertices of one row, so the [C, V, 3] output is written coalesced.
// ---------------------------------------------------------------------------
__global__ void create_vertices_kernel(const float* __restrict__ gv, const float* __restrict__ gsdf,
                                       const int32_t* __restrict__ lower, int64_t G,
                                       const float* __restrict__ level_sets, int S,
                                       const int32_t* __restrict__ voff, int64_t V, float* __restrict__ out_v,
                                       float* __restrict__ out_sdf, uint8_t* __restrict__ out_type,
                                       int32_t* __restrict__ sources) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
    const Corners4 c = load_corners(gsdf, lower, G, g);
    const int32_t i0 = __ldg(lower + g);
    uint32_t any = 0;
    for (int s = 0; s < S; ++s) any |= crossing_mask(c, __ldg(level_sets + s));
    if (any == 0) continue;
    const float v0x = __ldg(gv + 3 * (int64_t)i0), v0y = __ldg(gv + 3 * (int64_t)i0 + 1),
                v0z = __ldg(gv + 3 * (int64_t)i0 + 2);
    for (int a = 0; a < 3; ++a) {
      if (!((any >> a) & 1u)) continue;
      const int32_t i1 = c.idx[a];
      const float d1 = c.d[a];
      const float v1x = __ldg(gv + 3 * (int64_t)i1), v1y = __ldg(gv + 3 * (int64_t)i1 + 1),
                  v1z = __ldg(gv + 3 * (int64_t)i1 + 2);
      const uint32_t below_a = (1u << a) - 1u;
      for (int s = 0; s < S; ++s) {
        const float iso = __ldg(level_sets + s);
        const uint32_t m = crossing_mask(c, iso);
        if (!((m >> a) & 1u)) continue;
        const int64_t vi = (int64_t)__ldg(voff + (int64_t)s * G + g) + __popc(m & below_a);
        if (vi >= V) continue;  // beyond the caller's capacity (reported by the caller's count check)
        const float t = mc_weight(c.d0, d1, iso);
        out_v[3 * vi + 0] = lerp_ref(v0x, v1x, t);
        out_v[3 * vi + 1] = lerp_ref(v0y, v1y, t);
        out_v[3 * vi + 2] = lerp_ref(v0z, v1z, t);
        out_sdf[vi] = lerp_ref(c.d0, d1, t);
        out_type[vi] = (uint8_t)a;
        sources[vi] = i0;
        sources[V + vi] = i1;
        sources[2 * V + vi] = __float_as_int(t);
      }
    }
  }
}

// Rows have stride V (the buffer's capacity); only the first `count`
// vertices (device value, clamped to V; all V when count is NULL) are real.
__global__ void interpolate_vertex_sh_kernel(const float* __restrict__ gsh, int C, int64_t G,
                                             const int32_t* __restrict__ sources, int64_t V,
                                             const int32_t* __restrict__ count, float* __restrict__ out_sh) {
  const int64_t n = count ? min((int64_t)max(*count, 0), V) : V;
  const int64_t total = (int64_t)C * n;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = o / n, vi = o - k * n;
    const int32_t i0 = __ldg(sources + vi), i1 = __ldg(sources + V + vi);
    const float t = __int_as_float(__ldg(sources + 2 * V + vi));
    const float* p0 = gsh + (k * G + i0) * 3;
    const float* p1 = gsh + (k * G + i1) * 3;
    float* q = out_sh + (k * V + vi) * 3;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) q[ch] = lerp_ref(__ldg(p0 + ch), __ldg(p1 + ch), t);
  }
}

// ---------------------------------------------------------------------------
// Live marching-cubes weight (not in the reference, which detaches t at
// create_triangle_vertices.slang:92-96). With t = (iso - d0) / (d1 - d0) live,
// a vertex's position and SH depend on its two corner SDFs through t:
//   dL/dt = g_pos . (p1 - p0) + sum_k g_sh_k . (sh1_k - sh0_k),
//   dt/dd0 = -(1 - t) / (d1 - d0),  dt/dd1 = -t / (d1 - d0),
// and its SDF, d0 + t (d1 - d0) = iso, does not depend on them at all. t is
// constant where the reference clamps it or sets it to 0.5 (d0 == d1), so
// only 0 < t < 1 contributes. One thread per vertex adds the two corner
// terms to the grid SDF gradient with atomics. Rows have stride V; only the
// first `count` vertices (device value; all V when NULL) are real.
// ---------------------------------------------------------------------------
__global__ void live_t_backward_kernel(const float* __restrict__ gv, const float* __restrict__ gsdf,
                                       const float* __restrict__ gsh, int C, int64_t G,
                                       const int32_t* __restrict__ sources, int64_t V,
                                       const int32_t* __restrict__ count, const float* __restrict__ grad_v,
                                       const float* __restrict__ grad_sh, float* __restrict__ grad_gsdf) {
  const int64_t n = count ? min((int64_t)max(*count, 0), V) : V;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i0 = __ldg(sources + v), i1 = __ldg(sources + V + v);
    const float t = __int_as_float(__ldg(sources + 2 * V + v));
    const float d0 = __ldg(gsdf + i0), d1 = __ldg(gsdf + i1);
    if (!(t > 0.0f && t < 1.0f) || d0 == d1) continue;
    float dldt = 0.0f;
    if (grad_v) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        dldt += __ldg(grad_v + 3 * v + c) * (__ldg(gv + 3 * (int64_t)i1 + c) - __ldg(gv + 3 * (int64_t)i0 + c));
    }
    if (grad_sh) {
      for (int k = 0; k < C; ++k) {
        const float* g = grad_sh + ((int64_t)k * V + v) * 3;
        const float* p0 = gsh + ((int64_t)k * G + i0) * 3;
        const float* p1 = gsh + ((int64_t)k * G + i1) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) dldt += __ldg(g + c) * (__ldg(p1 + c) - __ldg(p0 + c));
      }
    }
    if (dldt == 0.0f) continue;
    const float q = dldt / (d1 - d0);
    atomicAdd(grad_gsdf + i0, -q * (1.0f - t));
    atomicAdd(grad_gsdf + i1, -q * t);
  }
}

// ---------------------------------------------------------------------------
// create_triangle_vertices.slang:201-291 (backward) as a gather. The detached
// weight t routes d(vertex) to the origin corner with (1 - t) and to the axis
// corner with t. Grid vertex x receives from the vertices of the one entry
// whose origin it is and from the vertices on axis a of the (at most three)
// entries whose axis-a corner it is; `inverse` [4, G] lists those entries.
// One thread per grid vertex writes all of x's gradients (zeros included),
// so no atomics and no zero-filled outputs are needed.
//
// Crossings are packed 3 bits per shell into 64-bit masks, shells taken in
// chunks of 21; the first chunk writes, later chunks add.
// ---------------------------------------------------------------------------
// `zero0` [G+1] and `zero1` [G] (either may be NULL) are cleared on the way,
// for the per-entry list passes that follow.
__global__ void invert_corners_kernel(const int32_t* __restrict__ lower, int64_t G, int32_t* __restrict__ inverse,
                                      int32_t* __restrict__ zero0 = nullptr, uint32_t* __restrict__ zero1 = nullptr) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G; e += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int32_t x = __ldg(lower + r * G + e);
      if (x >= 0 && x < G) inverse[r * G + x] = (int32_t)e;
    }
    if (zero0) zero0[e] = 0;
    if (zero1) zero1[e] = 0u;
  }
  if (zero0 && blockIdx.x == 0 && threadIdx.x == 0) zero0[G] = 0;
}

constexpr int kShellsPerChunk = 21;

__device__ __forceinline__ uint64_t crossing_bits(const Corners4& c, const float* __restrict__ level_sets, int s0,
                                                  int s1) {
  uint64_t bits = 0;
  for (int s = s0; s < s1; ++s) bits |= (uint64_t)crossing_mask(c, __ldg(level_sets + s)) << (3 * (s - s0));
  return bits;
}

// One contribution list of grid vertex x for the shells of one chunk: the
// vertex index and weight of every triangle vertex that x feeds.
struct GatherChunk {
  uint64_t own;       // crossings of x's own entry (3 bits per shell)
  uint64_t nb[3];     // crossings of the entry whose axis-a corner x is
  int64_t e, h[3];    // those entries (-1 = none)
  float d0, d1[3];    // own entry: origin and axis-corner signed distances
  float nd0[3], nd1[3];  // entry h[a]: origin and axis-a corner signed distances
};

__device__ __forceinline__ int64_t vertex_of(const int32_t* __restrict__ voff, int64_t G, int64_t entry, int s,
                                             uint64_t bits, int s0, int a) {
  const uint32_t m = (uint32_t)(bits >> (3 * (s - s0))) & 7u;
  return (int64_t)__ldg(voff + (int64_t)s * G + entry) + __popc(m & ((1u << a) - 1u));
}

// Calls f(vertex, weight) for each of x's contributions in this shell chunk:
// weight (1 - t) for the vertices of x's own entry, t for the axis-a vertices
// of the entries whose axis-a corner x is.
// Vertices at or past V (the buffers' capacity; only reached when the live
// count overflowed it) were never written and are skipped.
template <typename F>
__device__ __forceinline__ void for_each_contribution(const GatherChunk& q, const float* __restrict__ level_sets,
                                                      int s0, const int32_t* __restrict__ voff, int64_t G,
                                                      int64_t V, F&& f) {
  uint64_t bits = q.own;
  while (bits) {
    const int j = __ffsll((long long)bits) - 1;
    bits &= bits - 1;
    const int sl = j / 3, a = j - 3 * sl, s = s0 + sl;
    const int64_t vi = vertex_of(voff, G, q.e, s, q.own, s0, a);
    if (vi >= V) continue;
    f(vi, mc_weight(q.d0, q.d1[a], __ldg(level_sets + s)), true);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    uint64_t nbits = q.nb[a] & (0x1249249249249249ull << a);  // axis-a bits only
    while (nbits) {
      const int j = __ffsll((long long)nbits) - 1;
      nbits &= nbits - 1;
      const int s = s0 + j / 3;
      const int64_t vi = vertex_of(voff, G, q.h[a], s, q.nb[a], s0, a);
      if (vi >= V) continue;
      f(vi, mc_weight(q.nd0[a], q.nd1[a], __ldg(level_sets + s)), false);
    }
  }
}

// (1 - t) g, written g - t g as the reference's adjoint forms it, or t g.
__device__ __forceinline__ float weighted(float g, float t, bool origin) { return origin ? g - t * g : t * g; }

constexpr int kRowsPerPass = 16;  // SH coefficient rows accumulated in registers at once

__global__ void create_vertices_backward_kernel(const float* __restrict__ gsdf, int C,
                                                const int32_t* __restrict__ lower, int64_t G,
                                                const float* __restrict__ level_sets, int S,
                                                const int32_t* __restrict__ voff,
                                                const int32_t* __restrict__ inverse,
                                                const float* __restrict__ dv, const float* __restrict__ dsdf,
                                                const float* __restrict__ dsh, int64_t V, float* __restrict__ gdv,
                                                float* __restrict__ gdsdf, float* __restrict__ gdsh) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < G; x += (int64_t)gridDim.x * blockDim.x) {
    GatherChunk q;
    q.e = __ldg(inverse + x);
    Corners4 own{};
    if (q.e >= 0) own = load_corners(gsdf, lower, G, q.e);
    q.d0 = own.d0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      q.d1[a] = own.d[a];
      q.h[a] = __ldg(inverse + (int64_t)(a + 1) * G + x);
    }
    Corners4 nb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (q.h[a] >= 0) {
        nb[a] = load_corners(gsdf, lower, G, q.h[a]);
        q.nd0[a] = nb[a].d0;
        q.nd1[a] = nb[a].d[a];
      }
    }
    const int chunks = S > 0 ? (S + kShellsPerChunk - 1) / kShellsPerChunk : 1;
    for (int chunk = 0; chunk < chunks; ++chunk) {
      const int s0 = chunk * kShellsPerChunk, s1 = min(S, s0 + kShellsPerChunk);
      q.own = q.e >= 0 ? crossing_bits(own, level_sets, s0, s1) : 0ull;
#pragma unroll
      for (int a = 0; a < 3; ++a) q.nb[a] = q.h[a] >= 0 ? crossing_bits(nb[a], level_sets, s0, s1) : 0ull;
      const bool first = chunk == 0;
      auto put = [&](float* dst, float value) { *dst = first ? value : *dst + value; };

      float d = 0.f, p[3] = {0.f, 0.f, 0.f};
      for_each_contribution(q, level_sets, s0, voff, G, V, [&](int64_t vi, float t, bool origin) {
        if (dsdf) d += weighted(__ldg(dsdf + vi), t, origin);
        if (dv) {
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) p[ch] += weighted(__ldg(dv + 3 * vi + ch), t, origin);
        }
      });
      put(gdsdf + x, d);
      if (gdv) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) put(gdv + 3 * x + ch, p[ch]);
      }
      // SH rows in passes of 16: every contribution's 48 loads are independent.
      for (int k0 = 0; k0 < C; k0 += kRowsPerPass) {
        float r[kRowsPerPass][3];
#pragma unroll
        for (int kk = 0; kk < kRowsPerPass; ++kk) r[kk][0] = r[kk][1] = r[kk][2] = 0.f;
        if (dsh) {
          for_each_contribution(q, level_sets, s0, voff, G, V, [&](int64_t vi, float t, bool origin) {
#pragma unroll
            for (int kk = 0; kk < kRowsPerPass; ++kk) {
              if (k0 + kk < C) {
                const float* src = dsh + ((int64_t)(k0 + kk) * V + vi) * 3;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) r[kk][ch] += weighted(__ldg(src + ch), t, origin);
              }
            }
          });
        }
#pragma unroll
        for (int kk = 0; kk < kRowsPerPass; ++kk) {
          if (k0 + kk < C) {
            float* dst = gdsh + ((int64_t)(k0 + kk) * G + x) * 3;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) put(dst + ch, r[kk][ch]);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The same backward as a contribution list and a gather (S <= 21 shells).
//
// Pass 1 (count) and pass 2 (fill), one thread per grid vertex x, enumerate
// x's contributions exactly as create_vertices_backward_kernel does; pass 2
// writes the signed distance and position gradients and lists every
// contribution (vertex | origin flag << 31, t) at x's offset in a CSR list of
// at most 2V entries. Pass 3, one thread per (SH row k, grid vertex x), sums
// the row-k gradient over x's list in list order (the same sums, so the same
// bits) and writes it: consecutive threads write consecutive grid vertices
// of one row, and low register use keeps the SMs full.
// ---------------------------------------------------------------------------
__device__ __forceinline__ GatherChunk gather_entries(const float* __restrict__ gsdf,
                                                      const int32_t* __restrict__ lower, int64_t G,
                                                      const float* __restrict__ level_sets, int S,
                                                      const int32_t* __restrict__ inverse, int64_t x) {
  GatherChunk q;
  q.e = __ldg(inverse + x);
  Corners4 own{};
  if (q.e >= 0) own = load_corners(gsdf, lower, G, q.e);
  q.d0 = own.d0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    q.d1[a] = own.d[a];
    q.h[a] = __ldg(inverse + (int64_t)(a + 1) * G + x);
  }
  q.own = q.e >= 0 ? crossing_bits(own, level_sets, 0, S) : 0ull;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    q.nb[a] = 0ull;
    if (q.h[a] >= 0) {
      const Corners4 nb = load_corners(gsdf, lower, G, q.h[a]);
      q.nd0[a] = nb.d0;
      q.nd1[a] = nb.d[a];
      q.nb[a] = crossing_bits(nb, level_sets, 0, S);
    }
  }
  return q;
}

template <bool kFill>
__global__ void vertex_grad_list_kernel(const float* __restrict__ gsdf, const int32_t* __restrict__ lower, int64_t G,
                                        const float* __restrict__ level_sets, int S,
                                        const int32_t* __restrict__ voff, const int32_t* __restrict__ inverse,
                                        int64_t V, int32_t* __restrict__ counts, int2* __restrict__ list,
                                        const float* __restrict__ dv, const float* __restrict__ dsdf,
                                        float* __restrict__ gdv, float* __restrict__ gdsdf) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < G; x += (int64_t)gridDim.x * blockDim.x) {
    const GatherChunk q = gather_entries(gsdf, lower, G, level_sets, S, inverse, x);
    if (!kFill) {
      int n = 0;
      for_each_contribution(q, level_sets, 0, voff, G, V, [&](int64_t, float, bool) { ++n; });
      counts[x] = n;
    } else {
      int64_t pos = counts[x];  // scanned: x's first list entry
      float d = 0.f, p[3] = {0.f, 0.f, 0.f};
      for_each_contribution(q, level_sets, 0, voff, G, V, [&](int64_t vi, float t, bool origin) {
        list[pos++] = make_int2((int)vi | (origin ? (int)0x80000000 : 0), __float_as_int(t));
        if (dsdf) d += weighted(__ldg(dsdf + vi), t, origin);
        if (dv) {
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) p[ch] += weighted(__ldg(dv + 3 * vi + ch), t, origin);
        }
      });
      if (gdsdf) gdsdf[x] = d;
      if (gdv) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gdv[3 * x + ch] = p[ch];
      }
    }
  }
  if (!kFill && blockIdx.x == 0 && threadIdx.x == 0) counts[G] = 0;
}

__global__ void vertex_sh_gather_kernel(const float* __restrict__ dsh, int C, int64_t V, int64_t G,
                                        const int32_t* __restrict__ offsets, const int2* __restrict__ list,
                                        float* __restrict__ gdsh) {
  const int64_t total = (int64_t)C * G;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = o / G, x = o - k * G;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (dsh) {
      const int32_t end = __ldg(offsets + x + 1);
      for (int32_t p = __ldg(offsets + x); p < end; ++p) {
        const int2 e = __ldg(list + p);
        const int64_t vi = e.x & 0x7fffffff;
        const bool origin = e.x < 0;
        const float t = __int_as_float(e.y);
        const float* src = dsh + (k * V + vi) * 3;
        a0 += weighted(__ldg(src + 0), t, origin);
        a1 += weighted(__ldg(src + 1), t, origin);
        a2 += weighted(__ldg(src + 2), t, origin);
      }
    }
    float* dst = gdsh + (k * G + x) * 3;
    dst[0] = a0;
    dst[1] = a1;
    dst[2] = a2;
  }
}

// The signed-distance and position gradients of the list (pass 2's sums,
// in list order, so the same bits), for a list built ahead of the backward.
__global__ void vertex_grads_from_list_kernel(const int32_t* __restrict__ offsets, const int2* __restrict__ list,
                                              int64_t G, const float* __restrict__ dv, const float* __restrict__ dsdf,
                                              float* __restrict__ gdv, float* __restrict__ gdsdf) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < G; x += (int64_t)gridDim.x * blockDim.x) {
    float d = 0.f, p[3] = {0.f, 0.f, 0.f};
    const int32_t end = __ldg(offsets + x + 1);
    for (int32_t q = __ldg(offsets + x); q < end; ++q) {
      const int2 e = __ldg(list + q);
      const int64_t vi = e.x & 0x7fffffff;
      const bool origin = e.x < 0;
      const float t = __int_as_float(e.y);
      if (dsdf) d += weighted(__ldg(dsdf + vi), t, origin);
      if (dv) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) p[ch] += weighted(__ldg(dv + 3 * vi + ch), t, origin);
      }
    }
    gdsdf[x] = d;
    if (gdv) {
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) gdv[3 * x + ch] = p[ch];
    }
  }
}

// ---------------------------------------------------------------------------
// The same contribution list built per grid entry (mt_build_vertex_grad_list).
//
// Grid vertex x's list is four segments: the vertices of the entry whose
// origin x is, then the axis-0, axis-1 and axis-2 vertices of the entries
// whose axis-a corner x is, each in shell order (the order of
// for_each_contribution). Entry e owns segment r of x = lower[r][e] when the
// corner inverse names e there (so exactly the entries the per-vertex
// enumeration visits, also for inputs where two entries share a corner).
// Pass 1 adds each owned segment's length to x's count and stores it in byte
// r of x's segment word; pass 2 writes the segment at x's scanned offset plus
// the lengths of x's earlier segments. Each entry loads its own corners once
// (the per-vertex passes load four entries' corners per grid vertex).
// Counts and segment words start at zero (cleared by invert_corners_kernel).
// ---------------------------------------------------------------------------
template <bool kFill>
__global__ void entry_list_kernel(const float* __restrict__ gsdf, const int32_t* __restrict__ lower, int64_t G,
                                  const float* __restrict__ level_sets, int S, const int32_t* __restrict__ voff,
                                  const int32_t* __restrict__ inverse, int64_t V, int32_t* __restrict__ counts,
                                  uint32_t* __restrict__ segments, int2* __restrict__ list) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G; e += (int64_t)gridDim.x * blockDim.x) {
    const Corners4 c = load_corners(gsdf, lower, G, e);
    const uint64_t bits = crossing_bits(c, level_sets, 0, S);
    if (bits == 0) continue;
    int64_t x[4];
    x[0] = __ldg(lower + e);
#pragma unroll
    for (int a = 0; a < 3; ++a) x[a + 1] = c.idx[a];
    bool owns[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) owns[r] = x[r] >= 0 && x[r] < G && __ldg(inverse + r * G + x[r]) == (int32_t)e;
    if (!(owns[0] || owns[1] || owns[2] || owns[3])) continue;
    if (!kFill) {
      int n[4] = {0, 0, 0, 0};
      for (int s = 0; s < S; ++s) {
        const uint32_t m = (uint32_t)(bits >> (3 * s)) & 7u;
        if (m == 0) continue;
        const int64_t base = __ldg(voff + (int64_t)s * G + e);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (!((m >> a) & 1u) || base + __popc(m & ((1u << a) - 1u)) >= V) continue;
          ++n[0];
          ++n[a + 1];
        }
      }
      uint8_t* seg = reinterpret_cast<uint8_t*>(segments);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (owns[r] && n[r] > 0) {
          atomicAdd(counts + x[r], n[r]);
          seg[4 * x[r] + r] = (uint8_t)n[r];  // n[0] <= 3 * 21, n[a + 1] <= 21
        }
      }
    } else {
      const int64_t cap = 2 * V;
      int64_t pos[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        pos[r] = 0;
        if (owns[r]) {
          const uint32_t w = __ldg(segments + x[r]);
          uint32_t earlier = 0;
#pragma unroll
          for (int q = 0; q < r; ++q) earlier += (w >> (8 * q)) & 0xffu;
          pos[r] = (int64_t)__ldg(counts + x[r]) + earlier;  // counts = scanned offsets here
        }
      }
      for (int s = 0; s < S; ++s) {
        const uint32_t m = (uint32_t)(bits >> (3 * s)) & 7u;
        if (m == 0) continue;
        const float iso = __ldg(level_sets + s);
        const int64_t base = __ldg(voff + (int64_t)s * G + e);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (!((m >> a) & 1u)) continue;
          const int64_t vi = base + __popc(m & ((1u << a) - 1u));
          if (vi >= V) continue;
          const int tb = __float_as_int(mc_weight(c.d0, c.d[a], iso));
          if (owns[0] && pos[0] < cap) list[pos[0]] = make_int2((int)vi | (int)0x80000000, tb);
          ++pos[0];
          if (owns[a + 1] && pos[a + 1] < cap) list[pos[a + 1]] = make_int2((int)vi, tb);
          ++pos[a + 1];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Grid SH -> vertex colours without per-vertex SH rows: the interpolation of
// create_triangle_vertices.slang:145-199 (coefficients of vertex v from its
// two grid corners with weight t) followed by
// evaluate_spherical_harmonics.slang:4-270 for every camera, the coefficients
// kept in registers. Same operations as interpolate_vertex_sh_kernel then
// sh_forward_kernel, so the same bits. Vertices at or past the live count are
// not touched.
// ---------------------------------------------------------------------------
template <int kCoeff>
__device__ __forceinline__ void grid_sh_vertex(const float* __restrict__ gsh, int64_t G,
                                               const int32_t* __restrict__ sources, int64_t V,
                                               const float* __restrict__ verts, const float* __restrict__ campos,
                                               int B, int64_t v, float* __restrict__ out) {
  const int32_t i0 = __ldg(sources + v), i1 = __ldg(sources + V + v);
  const float t = __int_as_float(__ldg(sources + 2 * V + v));
  float coef[kCoeff][3];
#pragma unroll
  for (int k = 0; k < kCoeff; ++k) {
    const float* p0 = gsh + ((int64_t)k * G + i0) * 3;
    const float* p1 = gsh + ((int64_t)k * G + i1) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) coef[k][c] = lerp_ref(__ldg(p0 + c), __ldg(p1 + c), t);
  }
  sh_colors<kCoeff>(verts, V, coef, campos, B, v, out);
}

__global__ void grid_sh_colors_kernel(const float* __restrict__ gsh, int64_t G, const int32_t* __restrict__ sources,
                                      int64_t V, const int32_t* __restrict__ count, const float* __restrict__ verts,
                                      int n_coeff, const float* __restrict__ campos, int B, float* __restrict__ out) {
  const int64_t n = count ? min((int64_t)max(*count, 0), V) : V;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    switch (n_coeff) {
      case 1: grid_sh_vertex<1>(gsh, G, sources, V, verts, campos, B, v, out); break;
      case 4: grid_sh_vertex<4>(gsh, G, sources, V, verts, campos, B, v, out); break;
      case 9: grid_sh_vertex<9>(gsh, G, sources, V, verts, campos, B, v, out); break;
      default: grid_sh_vertex<16>(gsh, G, sources, V, verts, campos, B, v, out); break;
    }
  }
}

// Backward: grid vertex x's SH gradient is sum over its list entries (v, t)
// of weighted(d sh_v), with d sh_v[k] = sum_b basis_k(dir_bv) d rgb_bv
// [rgb_bv > 0] formed on the fly (the sums of sh_backward_kernel, cameras in
// order, then of vertex_sh_gather_kernel, entries in list order: the same
// bits without the [C, V, 3] rows). One thread per (group of kRowsPerThread
// rows, grid vertex); consecutive threads write consecutive grid vertices of
// each row. Rows k >= n_coeff (up to C) are written as zeros.
// A CTA takes kShX consecutive grid vertices; their list entries are
// contiguous. In rounds of kShThreads entries, thread i forms entry i's
// weighted SH gradient (all rows: the per-vertex d sh_v of sh_backward_kernel,
// cameras in order, then weighted by the entry's (t, origin)) in shared
// memory; then thread (row half h, grid vertex x) adds x's entries of the
// round to its 8 rows in list order, carrying its sums across rounds. The
// same sums in the same order as sh_backward_kernel + vertex_sh_gather_kernel.
constexpr int kShThreads = 128;
constexpr int kShX = 64;
constexpr int kShStride = 49;  // 48 values per entry; odd stride spreads rows over banks

__device__ __forceinline__ void entry_sh_gradient(int2 e, int64_t V, const float* __restrict__ verts, int n_coeff,
                                                  const float* __restrict__ campos, int B,
                                                  const float* __restrict__ colors,
                                                  const float* __restrict__ dcolors, float* __restrict__ out) {
  const int64_t vi = e.x & 0x7fffffff;
  const bool origin = e.x < 0;
  const float t = __int_as_float(e.y);
  const float px = __ldg(verts + 3 * vi), py = __ldg(verts + 3 * vi + 1), pz = __ldg(verts + 3 * vi + 2);
  float d[16][3];
#pragma unroll
  for (int k = 0; k < 16; ++k) d[k][0] = d[k][1] = d[k][2] = 0.f;
#pragma unroll 2
  for (int b = 0; b < B; ++b) {
    const int64_t ob = ((int64_t)b * V + vi) * 3;
    float col[3], dcol[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      col[c] = __ldg(colors + ob + c);
      dcol[c] = __ldg(dcolors + ob + c);
    }
    float g[3];
    bool any = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      g[c] = col[c] > 0.0f ? dcol[c] : 0.0f;
      any |= g[c] != 0.0f;
    }
    if (!any) continue;
    float dx, dy, dz;
    view_dir_at(px, py, pz, campos + 3 * b, dx, dy, dz);
    float basis[16];
    sh_basis(dx, dy, dz, n_coeff, basis);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k < n_coeff) {
#pragma unroll
        for (int c = 0; c < 3; ++c) d[k][c] += basis[k] * g[c];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) {
#pragma unroll
    for (int c = 0; c < 3; ++c) out[3 * k + c] = weighted(d[k][c], t, origin);
  }
}

__global__ void __launch_bounds__(kShThreads)
    grid_sh_colors_backward_kernel(const int32_t* __restrict__ offsets, const int2* __restrict__ list, int64_t G,
                                   int64_t V, const float* __restrict__ verts, int C, int n_coeff,
                                   const float* __restrict__ campos, int B, const float* __restrict__ colors,
                                   const float* __restrict__ dcolors, float* __restrict__ gdsh) {
  __shared__ float s_grad[kShThreads * kShStride];
  const int tid = threadIdx.x;
  const int half = tid / kShX, xl = tid % kShX;  // rows 8*half .. 8*half+7 of grid vertex x0 + xl
  for (int64_t x0 = (int64_t)blockIdx.x * kShX; x0 < G; x0 += (int64_t)gridDim.x * kShX) {
    const int64_t x = x0 + xl;
    const int32_t e_begin = __ldg(offsets + x0), e_end = __ldg(offsets + min(x0 + kShX, G));
    const int32_t my_begin = x < G ? __ldg(offsets + x) : 0, my_end = x < G ? __ldg(offsets + x + 1) : 0;
    float acc[8][3];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) acc[kk][0] = acc[kk][1] = acc[kk][2] = 0.f;
    for (int32_t base = e_begin; base < e_end; base += kShThreads) {
      if (base + tid < e_end)
        entry_sh_gradient(__ldg(list + base + tid), V, verts, n_coeff, campos, B, colors, dcolors,
                          s_grad + tid * kShStride);
      __syncthreads();
      const int32_t lo = max(my_begin, base), hi = min(my_end, base + kShThreads);
      for (int32_t q = lo; q < hi; ++q) {
        const float* src = s_grad + (q - base) * kShStride + 24 * half;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
#pragma unroll
          for (int c = 0; c < 3; ++c) acc[kk][c] += src[3 * kk + c];
        }
      }
      __syncthreads();
    }
    if (x < G) {
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const int k = 8 * half + kk;
        if (k < C) {
          float* dst = gdsh + ((int64_t)k * G + x) * 3;
#pragma unroll
          for (int c = 0; c < 3; ++c) dst[c] = k < n_coeff ? acc[kk][c] : 0.f;
        }
      }
    }
  }
}

// Two-pass form of the same backward (with scratch): pass 1, one thread per
// live vertex v, forms d sh_v (cameras in order, as sh_backward_kernel) once
// into a vertex-major array [V][16][3]; pass 2, one thread per (8-row half h,
// grid vertex x), sums x's list entries of rows 8h .. 8h + 7 (96 contiguous
// bytes per entry) weighted, in list order. The same bits as the one-pass
// kernel, with each vertex's gradient formed once instead of once per entry.
constexpr int kShGradThreads = 128;

__global__ void __launch_bounds__(kShGradThreads)
    vertex_sh_grad_kernel(const float* __restrict__ verts, int64_t V, const int32_t* __restrict__ count,
                          int n_coeff, const float* __restrict__ campos, int B, const float* __restrict__ colors,
                          const float* __restrict__ dcolors, float4* __restrict__ out) {
  // Each round, the CTA's kShGradThreads consecutive vertices form their
  // rows in shared memory, then write them as one contiguous block (full
  // 128-byte lines, where each thread's own 192-byte row would be written
  // 16 bytes at a time at a 192-byte stride).
  __shared__ float4 s_rows[kShGradThreads * 12];
  const int64_t n = count ? min((int64_t)max(*count, 0), V) : V;
  for (int64_t v0 = (int64_t)blockIdx.x * kShGradThreads; v0 < n; v0 += (int64_t)gridDim.x * kShGradThreads) {
    const int64_t v = v0 + threadIdx.x;
    if (v < n) {
      const float px = __ldg(verts + 3 * v), py = __ldg(verts + 3 * v + 1), pz = __ldg(verts + 3 * v + 2);
      float d[16][3];
#pragma unroll
      for (int k = 0; k < 16; ++k) d[k][0] = d[k][1] = d[k][2] = 0.f;
      // Cameras two at a time: both cameras' colours and colour gradients
      // are loaded together, then the cameras are added in order.
      for (int b0 = 0; b0 < B; b0 += 2) {
        float col[2][3], dcol[2][3];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const bool in = b0 + j < B;
          const int64_t ob = ((int64_t)(b0 + j) * V + v) * 3;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            col[j][c] = in ? __ldg(colors + ob + c) : 0.0f;
            dcol[j][c] = in ? __ldg(dcolors + ob + c) : 0.0f;
          }
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          float g[3];
          bool any = false;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            g[c] = col[j][c] > 0.0f ? dcol[j][c] : 0.0f;
            any |= g[c] != 0.0f;
          }
          if (!any) continue;  // also every camera past B (its g is zero)
          float dx, dy, dz;
          view_dir_at(px, py, pz, campos + 3 * (b0 + j), dx, dy, dz);
          float basis[16];
          sh_basis(dx, dy, dz, n_coeff, basis);
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            if (k < n_coeff) {
#pragma unroll
              for (int c = 0; c < 3; ++c) d[k][c] += basis[k] * g[c];
            }
          }
        }
      }
      float4* row = s_rows + threadIdx.x * 12;
#pragma unroll
      for (int q = 0; q < 12; ++q) {
        const int j = 4 * q;
        row[q] = make_float4(d[j / 3][j % 3], d[(j + 1) / 3][(j + 1) % 3], d[(j + 2) / 3][(j + 2) % 3],
                             d[(j + 3) / 3][(j + 3) % 3]);
      }
    }
    __syncthreads();
    const int64_t rows = min((int64_t)kShGradThreads, n - v0);
    for (int i = threadIdx.x; i < rows * 12; i += kShGradThreads) out[v0 * 12 + i] = s_rows[i];
    __syncthreads();  // s_rows is written again by the next round
  }
}

__global__ void grid_sh_gather_kernel(const int32_t* __restrict__ offsets, const int2* __restrict__ list, int64_t G,
                                      const float4* __restrict__ dsh, int C, int n_coeff,
                                      float* __restrict__ gdsh) {
  const int64_t total = 2 * G;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
    // Adjacent threads take the two halves of one grid vertex, so a vertex's
    // 192-byte gradient row is read by neighbouring lanes together.
    const int half = (int)(o & 1);
    const int64_t x = o >> 1;
    float acc[24];
#pragma unroll
    for (int j = 0; j < 24; ++j) acc[j] = 0.f;
    const int32_t end = __ldg(offsets + x + 1);
    for (int32_t q = __ldg(offsets + x); q < end; ++q) {
      const int2 e = __ldg(list + q);
      const int64_t vi = e.x & 0x7fffffff;
      const bool origin = e.x < 0;
      const float t = __int_as_float(e.y);
      const float4* src = dsh + vi * 12 + 6 * half;
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const float4 val = __ldg(src + r);
        acc[4 * r + 0] += weighted(val.x, t, origin);
        acc[4 * r + 1] += weighted(val.y, t, origin);
        acc[4 * r + 2] += weighted(val.z, t, origin);
        acc[4 * r + 3] += weighted(val.w, t, origin);
      }
    }
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int k = 8 * half + kk;
      if (k < C) {
        float* dst = gdsh + ((int64_t)k * G + x) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) dst[c] = k < n_coeff ? acc[3 * kk + c] : 0.f;
      }
    }
  }
}

size_t vertex_grad_bytes(int64_t G, int64_t V, int32_t** counts, int2** list, void** scan_ws, size_t* scan_bytes,
                         char* base) {
  size_t off = 256;  // the workspace status word
  auto take = [&](size_t bytes) {
    char* q = base ? base + off : nullptr;
    off += (bytes + 255) & ~(size_t)255;
    return q;
  };
  char* c = take((size_t)(G + 1) * sizeof(int32_t));
  char* l = take((size_t)2 * (V > 0 ? V : 0) * sizeof(int2));
  const size_t sb = mt_scan_workspace_bytes(G + 1);
  char* sw = take(sb);
  if (counts) *counts = reinterpret_cast<int32_t*>(c);
  if (list) *list = reinterpret_cast<int2*>(l);
  if (scan_ws) *scan_ws = sw;
  if (scan_bytes) *scan_bytes = sb;
  return off;
}

// ---------------------------------------------------------------------------
// count_triangle_faces.slang:15-50: cube code bit i <=> corner i >= iso with
// corner order (origin, +x, +xy, +y, +z, +xz, +xyz, +yz).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_cube(const float* __restrict__ sdf, const int32_t* __restrict__ lower, int64_t G,
                                          const int32_t* __restrict__ upper, int64_t Nv, int64_t v, float (&cube)[8]) {
  cube[0] = __ldg(sdf + __ldg(lower + v));
  cube[1] = __ldg(sdf + __ldg(lower + G + v));
  cube[2] = __ldg(sdf + __ldg(upper + 3 * Nv + v));
  cube[3] = __ldg(sdf + __ldg(lower + 2 * G + v));
  cube[4] = __ldg(sdf + __ldg(lower + 3 * G + v));
  cube[5] = __ldg(sdf + __ldg(upper + 2 * Nv + v));
  cube[6] = __ldg(sdf + __ldg(upper + v));
  cube[7] = __ldg(sdf + __ldg(upper + Nv + v));
}

__global__ void count_faces_kernel(const float* __restrict__ sdf, const int32_t* __restrict__ lower, int64_t G,
                                   const int32_t* __restrict__ upper, int64_t Nv,
                                   const float* __restrict__ level_sets, int S, int32_t* __restrict__ counts,
                                   uint8_t* __restrict__ codes) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nv; v += (int64_t)gridDim.x * blockDim.x) {
    float cube[8];
    load_cube(sdf, lower, G, upper, Nv, v, cube);
    for (int s = 0; s < S; ++s) {
      const float iso = __ldg(level_sets + s);
      uint32_t code = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) code |= (uint32_t)(cube[q] >= iso) << q;
      codes[(int64_t)s * Nv + v] = (uint8_t)code;
      counts[(int64_t)s * Nv + v] = c_mc_count[code];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counts[(int64_t)S * Nv] = 0;
}

// ---------------------------------------------------------------------------
// create_triangle_faces.slang:5-78. Edge id -> owning entry (self or upper
// neighbour) -> that entry's vertices at this level set -> the one whose
// type is the edge's axis. Triangles are written in reversed slot order.
// ---------------------------------------------------------------------------
// Writes only faces below F and searches only vertices below V (the
// buffers' capacities); with consistent offsets neither bound is reached.
//
// Work is dealt by face slot: a warp reads 32 consecutive (shell, voxel)
// items (shell-major, the order of the slot offsets) in one coalesced load;
// their slots are contiguous, so lane r takes the r-th slot of the span (its
// item by a shuffle search over the warp's running edge counts) and every
// lane resolves one edge: full lanes, and consecutive lanes write
// consecutive face corners. The case tables sit in shared memory, as lanes
// read different cases.
__global__ void __launch_bounds__(256)
    create_faces_kernel(const int32_t* __restrict__ neighbors, const int32_t* __restrict__ indices, int64_t Nv,
                        int64_t G, int64_t V, const int32_t* __restrict__ voff, const uint8_t* __restrict__ types,
                        const uint8_t* __restrict__ codes, int S, const int32_t* __restrict__ foff, int64_t F,
                        int32_t* __restrict__ faces, int32_t* __restrict__ voxel_indices) {
  __shared__ uint64_t s_edges[256];
  __shared__ uint8_t s_count[256];
  __shared__ int8_t s_owner[12];
  __shared__ uint8_t s_axis[12];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    s_edges[i] = c_mc_edges[i];
    s_count[i] = c_mc_count[i];
  }
  if (threadIdx.x < 12) {
    s_owner[threadIdx.x] = c_mc_owner[threadIdx.x];
    s_axis[threadIdx.x] = c_mc_axis[threadIdx.x];
  }
  __syncthreads();
  const int64_t total = (int64_t)S * Nv;
  const int lane = threadIdx.x & 31;
  const int64_t first_warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = first_warp * 32; base < total; base += warps * 32) {
    const int64_t mine = base + lane;
    const uint32_t code = mine < total ? (uint32_t)codes[mine] : 0u;
    const int n = s_count[code];
    int incl = n;  // inclusive scan of the edge counts over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    const int span = __shfl_sync(0xffffffffu, incl, 31);
    if (span == 0) continue;
    const int64_t first_slot = __ldg(foff + base);
    const int64_t s_base = base / Nv;  // shell of the warp's first item (one division per warp step)
    for (int start = 0; start < span; start += 32) {
      const int r = start + lane;
      int src = 0;  // item holding slot r: smallest src with incl[src] > r
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int u = __shfl_sync(0xffffffffu, incl, src + step - 1);
        if (u <= r) src += step;
      }
      const uint32_t c = __shfl_sync(0xffffffffu, code, src);
      const int before = __shfl_sync(0xffffffffu, incl - n, src);
      if (r >= span) continue;
      const int e = r - before;
      const int64_t item = base + src;
      int s = (int)s_base;
      int64_t v = item - s_base * Nv;
      while (v >= Nv) {  // at most ceil(32 / Nv) steps
        v -= Nv;
        ++s;
      }
      const int eid = (int)((s_edges[c] >> (4 * e)) & 15u);
      const int owner = s_owner[eid];
      const uint8_t axis = s_axis[eid];
      const int64_t nb = (owner < 0) ? v : (int64_t)__ldg(neighbors + (int64_t)owner * Nv + v);
      const int64_t vo = (int64_t)s * G + nb;
      const int32_t vstart = __ldg(voff + vo);
      const int32_t count = __ldg(voff + vo + 1) - vstart;
      int32_t target = -1;
      for (int q = 0; q < count; ++q) {
        if ((int64_t)vstart + q >= V) break;
        if (types[vstart + q] == axis) {
          target = vstart + q;
          break;
        }
      }
      const int64_t slot = first_slot + r;
      const int64_t tri = slot / 3;
      if (tri >= F) continue;
      const int corner = 2 - (int)(slot % 3);
      faces[tri * 3 + corner] = target;
      if (corner == 0) voxel_indices[tri] = __ldg(indices + v);
    }
  }
}

// ---------------------------------------------------------------------------
// triangle_extraction/compute_sdf_regularizers.slang:18-128. Per voxel: the
// Eikonal terms of the trilinear SDF's gradient at the voxel centre (grid
// units) and a Laplacian curvature term at its +xyz corner. The operation
// order is the reference's (this unit is compiled without contraction).
// ---------------------------------------------------------------------------
struct VoxelCorners {
  int32_t i000, i001, i010, i100, i111, i110, i101, i011;  // grid vertex ids
  float d000, d001, d010, d100, d111, d110, d101, d011;
};

__device__ __forceinline__ VoxelCorners load_voxel_corners(const float* __restrict__ sdf,
                                                           const int32_t* __restrict__ lower, int64_t G,
                                                           const int32_t* __restrict__ upper, int64_t Nv, int64_t v) {
  VoxelCorners c;
  c.i000 = __ldg(lower + v);
  c.i001 = __ldg(lower + G + v);
  c.i010 = __ldg(lower + 2 * G + v);
  c.i100 = __ldg(lower + 3 * G + v);
  c.i111 = __ldg(upper + v);
  c.i110 = __ldg(upper + Nv + v);
  c.i101 = __ldg(upper + 2 * Nv + v);
  c.i011 = __ldg(upper + 3 * Nv + v);
  c.d000 = __ldg(sdf + c.i000);
  c.d001 = __ldg(sdf + c.i001);
  c.d010 = __ldg(sdf + c.i010);
  c.d100 = __ldg(sdf + c.i100);
  c.d111 = __ldg(sdf + c.i111);
  c.d110 = __ldg(sdf + c.i110);
  c.d101 = __ldg(sdf + c.i101);
  c.d011 = __ldg(sdf + c.i011);
  return c;
}

// Trilinear gradient at (0.5, 0.5, 0.5): weights (1 - t)(1 - t), t(1 - t), ...
// are all 0.25; the sums keep the reference's association.
__device__ __forceinline__ void centre_gradient(const VoxelCorners& c, float& dx, float& dy, float& dz) {
  const float t = 0.5f, t1 = 1.0f - t;
  const float w11 = t1 * t1, w01 = t * t1, w10 = t1 * t, w00 = t * t;
  dx = w11 * (c.d001 - c.d000) + w01 * (c.d011 - c.d010) + w10 * (c.d101 - c.d100) + w00 * (c.d111 - c.d110);
  dy = w11 * (c.d010 - c.d000) + w01 * (c.d011 - c.d001) + w10 * (c.d110 - c.d100) + w00 * (c.d111 - c.d101);
  dz = w11 * (c.d100 - c.d000) + w01 * (c.d101 - c.d001) + w10 * (c.d110 - c.d010) + w00 * (c.d111 - c.d011);
}

// stable_norm of compute_sdf_regularizers.slang:3-16.
__device__ __forceinline__ float stable_norm(float a, float b, float c) {
  const float scale = fmaxf(fmaxf(fabsf(a), fabsf(b)), fabsf(c));
  if (scale < 1e-10f) return 0.0f;
  const float inv = 1.0f / scale;
  const float sa = inv * a, sb = inv * b, sc = inv * c;
  return scale * sqrtf(sa * sa + sb * sb + sc * sc);
}

// Curvature sum: +yz, +xz, +xy corners, the present lower corners (+x, +y,
// +z) of the +xyz neighbour entry, minus (count) x the +xyz corner.
__device__ __forceinline__ float curvature_sum(const float* __restrict__ sdf, const VoxelCorners& c,
                                               const int32_t* __restrict__ lower, int64_t G, int32_t sub,
                                               int32_t (&extra)[3], int& counted) {
  float sum = c.d110 + c.d101 + c.d011;
  counted = 3;
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    const int32_t corner = __ldg(lower + (int64_t)i * G + sub);
    extra[i - 1] = corner;
    if (corner >= 0) {
      sum += __ldg(sdf + corner);
      ++counted;
    }
  }
  return sum - (float)counted * c.d111;
}

__global__ void sdf_regularizers_kernel(const float* __restrict__ sdf, const int32_t* __restrict__ neighbors,
                                        const int32_t* __restrict__ lower, int64_t G,
                                        const int32_t* __restrict__ upper, int64_t Nv, int vx, int vy, int vz,
                                        float* __restrict__ eik_pos, float* __restrict__ eik_neg,
                                        float* __restrict__ curv) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nv; v += (int64_t)gridDim.x * blockDim.x) {
    const VoxelCorners c = load_voxel_corners(sdf, lower, G, upper, Nv, v);
    float dx, dy, dz;
    centre_gradient(c, dx, dy, dz);
    const float delta = stable_norm((float)vx * dx, (float)vy * dy, (float)vz * dz) - 1.0f;
    float pos = 0.0f, neg = 0.0f;
    if (delta < 0.0f) neg += delta * delta;
    if (delta > 0.0f) pos += delta * delta;
    eik_pos[v] = pos / 1.0f;
    eik_neg[v] = neg / 1.0f;
    int32_t extra[3];
    int counted;
    const float cs = curvature_sum(sdf, c, lower, G, __ldg(neighbors + 6 * Nv + v), extra, counted);
    curv[v] = cs * cs;
  }
}

// Adjoint (the reference differentiates the kernel automatically): with
// n = |(a, b, c)| and delta = n - 1, d delta / d a = a / n (0 when n is 0);
// each loss's gradient is scattered to the corners it reads.
__global__ void sdf_regularizers_backward_kernel(const float* __restrict__ sdf,
                                                 const int32_t* __restrict__ neighbors,
                                                 const int32_t* __restrict__ lower, int64_t G,
                                                 const int32_t* __restrict__ upper, int64_t Nv, int vx, int vy,
                                                 int vz, const float* __restrict__ g_pos,
                                                 const float* __restrict__ g_neg, const float* __restrict__ g_curv,
                                                 float* __restrict__ grad_sdf) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nv; v += (int64_t)gridDim.x * blockDim.x) {
    const VoxelCorners c = load_voxel_corners(sdf, lower, G, upper, Nv, v);
    float dx, dy, dz;
    centre_gradient(c, dx, dy, dz);
    const float a = (float)vx * dx, b = (float)vy * dy, cc = (float)vz * dz;
    const float n = stable_norm(a, b, cc);
    const float delta = n - 1.0f;
    float g_delta = 0.0f;
    if (g_pos && delta > 0.0f) g_delta += 2.0f * delta * g_pos[v];
    if (g_neg && delta < 0.0f) g_delta += 2.0f * delta * g_neg[v];
    float gd[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // 000 001 010 100 111 110 101 011
    if (g_delta != 0.0f && n > 0.0f) {
      const float gx = g_delta * a / n * (float)vx, gy = g_delta * b / n * (float)vy,
                  gz = g_delta * cc / n * (float)vz;
      const float w = 0.25f;
      // dx: +(001, 011, 101, 111), -(000, 010, 100, 110)
      gd[1] += w * gx; gd[7] += w * gx; gd[6] += w * gx; gd[4] += w * gx;
      gd[0] -= w * gx; gd[2] -= w * gx; gd[3] -= w * gx; gd[5] -= w * gx;
      // dy: +(010, 011, 110, 111), -(000, 001, 100, 101)
      gd[2] += w * gy; gd[7] += w * gy; gd[5] += w * gy; gd[4] += w * gy;
      gd[0] -= w * gy; gd[1] -= w * gy; gd[3] -= w * gy; gd[6] -= w * gy;
      // dz: +(100, 101, 110, 111), -(000, 001, 010, 011)
      gd[3] += w * gz; gd[6] += w * gz; gd[5] += w * gz; gd[4] += w * gz;
      gd[0] -= w * gz; gd[1] -= w * gz; gd[2] -= w * gz; gd[7] -= w * gz;
    }
    int32_t extra[3];
    int counted;
    const float cs = curvature_sum(sdf, c, lower, G, __ldg(neighbors + 6 * Nv + v), extra, counted);
    const float g_cs = g_curv ? 2.0f * cs * g_curv[v] : 0.0f;
    if (g_cs != 0.0f) {
      gd[5] += g_cs;
      gd[6] += g_cs;
      gd[7] += g_cs;
      gd[4] -= (float)counted * g_cs;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (extra[i] >= 0) atomicAdd(grad_sdf + extra[i], g_cs);
    }
    const int32_t ids[8] = {c.i000, c.i001, c.i010, c.i100, c.i111, c.i110, c.i101, c.i011};
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (gd[q] != 0.0f) atomicAdd(grad_sdf + ids[q], gd[q]);
  }
}

// Last entry of every shell's block of an exclusive scan: the vertex and face
// boundaries of triangle_extraction/__init__.py:145-146 (faces / 3, floor),
// plus the face total of :131 (offsets are non-negative, so / is floor).
__global__ void shell_boundaries_kernel(const int32_t* __restrict__ voff, int64_t G,
                                        const int32_t* __restrict__ foff, int64_t Nv, int S,
                                        int32_t* __restrict__ vb, int32_t* __restrict__ fb,
                                        int32_t* __restrict__ num_faces) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < S) {
    vb[s] = G > 0 ? voff[(int64_t)(s + 1) * G] : 0;
    fb[s] = Nv > 0 ? foff[(int64_t)(s + 1) * Nv] / 3 : 0;
  }
  if (s == 0 && num_faces) *num_faces = foff[(int64_t)S * Nv] / 3;
}

__global__ void capacity_overflow_kernel(const int32_t* __restrict__ nv, int64_t cv, const int32_t* __restrict__ nf,
                                         int64_t cf, const int64_t* __restrict__ nk, int64_t ck,
                                         uint8_t* __restrict__ overflow) {
  bool over = false;
  if (nv) over |= (int64_t)*nv > cv;
  if (nf) over |= (int64_t)*nf > cf;
  if (nk) over |= *nk > ck;
  *overflow = over ? 1 : 0;
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

int mt_compute_vertex_occupancy(const int32_t* occupancy, int32_t I, int32_t J, int32_t KP, int32_t* vertex_occupancy,
                                int32_t* vertex_counts, mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0);
  MT_REQUIRE(vertex_occupancy && vertex_counts);
  MT_REQUIRE(occupancy || (int64_t)I * J * KP == 0);
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  vertex_occupancy_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(
      occupancy, I, J, KP, vertex_occupancy, vertex_counts);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_count_occupancy(const int32_t* occupancy, int32_t I, int32_t J, int32_t KP, int32_t* voxel_counts,
                       mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0);
  MT_REQUIRE(voxel_counts);
  MT_REQUIRE(occupancy || (int64_t)I * J * KP == 0);
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  count_occupancy_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(occupancy, I, J, KP,
                                                                                       voxel_counts);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_create_voxels(const int32_t* occupancy, const int32_t* voxel_offsets, const int32_t* vertex_occupancy,
                     const int32_t* vertex_offsets, int32_t I, int32_t J, int32_t KP, int64_t num_voxels,
                     int64_t num_vertices, float* vertices, int32_t* neighbors, int32_t* lower_corners,
                     int32_t* upper_corners, int32_t* indices, mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0 && num_voxels >= 0 && num_vertices >= num_voxels);
  if (num_vertices == 0) return MT_OK;
  MT_REQUIRE(I > 0 && J > 0 && KP > 0);
  MT_REQUIRE(occupancy && voxel_offsets && vertex_occupancy && vertex_offsets && vertices && lower_corners);
  MT_REQUIRE(num_voxels == 0 || (neighbors && upper_corners && indices));
  MT_REQUIRE((int64_t)32 * KP * J * I < ((int64_t)1 << 31));
  VoxelGrid g{occupancy, voxel_offsets, vertex_occupancy, vertex_offsets, I, J, KP, num_voxels};
  const int64_t words = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  const int threads = 256;
  const int64_t want = (words * 32 + threads - 1) / threads;
  const unsigned blocks = (unsigned)(want < (int64_t)kSmCount * 16 ? want : (int64_t)kSmCount * 16);
  create_voxels_kernel<<<blocks, threads, 0, as_stream(stream)>>>(g, vertices, neighbors, lower_corners,
                                                                  upper_corners, indices, num_vertices);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_dilate_occupancy(const int32_t* occupancy, int32_t I, int32_t J, int32_t KP, int32_t dilation, int32_t* out,
                        mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0);
  MT_REQUIRE(dilation > 0 && dilation < 32);
  const int64_t total = (int64_t)I * J * KP;
  if (total == 0) return MT_OK;
  MT_REQUIRE(occupancy && out && occupancy != out);
  dilate_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(occupancy, I, J, KP, dilation, out);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_count_triangle_vertices(const float* signed_distances, const int32_t* lower_corners, int64_t G,
                               const float* level_sets, int32_t S, int32_t* counts, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && S >= 0 && counts);
  MT_REQUIRE(G == 0 || (signed_distances && lower_corners));
  MT_REQUIRE(S == 0 || level_sets);
  count_vertices_kernel<<<grid_stride_blocks(G, 256), 256, 0, as_stream(stream)>>>(signed_distances, lower_corners, G,
                                                                                  level_sets, S, counts);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_create_triangle_vertices_live_t_backward(const float* grid_vertices, const float* grid_signed_distances,
                                                const float* grid_spherical_harmonics, int32_t C, int64_t G,
                                                const int32_t* vertex_sources, int64_t V, const int32_t* num_vertices,
                                                const float* grad_vertices, const float* grad_spherical_harmonics,
                                                float* grad_grid_signed_distances, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && V >= 0 && C >= 1);
  if (V == 0 || G == 0 || (grad_vertices == nullptr && grad_spherical_harmonics == nullptr)) return MT_OK;
  MT_REQUIRE(grid_signed_distances && vertex_sources && grad_grid_signed_distances);
  MT_REQUIRE(grad_vertices == nullptr || grid_vertices != nullptr);
  MT_REQUIRE(grad_spherical_harmonics == nullptr || grid_spherical_harmonics != nullptr);
  live_t_backward_kernel<<<grid_stride_blocks(V, 256), 256, 0, as_stream(stream)>>>(
      grid_vertices, grid_signed_distances, grid_spherical_harmonics, C, G, vertex_sources, V, num_vertices,
      grad_vertices, grad_spherical_harmonics, grad_grid_signed_distances);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_create_triangle_vertices(const float* grid_vertices, const float* grid_signed_distances,
                                const float* grid_spherical_harmonics, int32_t C, const int32_t* lower_corners,
                                int64_t G, const float* level_sets, int32_t S, const int32_t* vertex_offsets,
                                int64_t V, const int32_t* num_vertices, float* vertices, float* signed_distances,
                                float* spherical_harmonics, uint8_t* vertex_types, int32_t* vertex_sources,
                                mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && S >= 0 && C >= 1 && V >= 0);
  if (G == 0 || S == 0 || V == 0) return MT_OK;
  MT_REQUIRE(grid_vertices && grid_signed_distances && lower_corners && level_sets && vertex_offsets && vertices &&
             signed_distances && vertex_types && vertex_sources);
  create_vertices_kernel<<<grid_stride_blocks(G, 128), 128, 0, as_stream(stream)>>>(
      grid_vertices, grid_signed_distances, lower_corners, G, level_sets, S, vertex_offsets, V, vertices,
      signed_distances, vertex_types, vertex_sources);
  MT_CHECK_LAUNCH();
  if (spherical_harmonics == nullptr) return MT_OK;  // rows left to mt_grid_sh_colors
  MT_REQUIRE(grid_spherical_harmonics);
  interpolate_vertex_sh_kernel<<<grid_stride_blocks((int64_t)C * V, 256), 256, 0, as_stream(stream)>>>(
      grid_spherical_harmonics, C, G, vertex_sources, V, num_vertices, spherical_harmonics);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

size_t mt_create_triangle_vertices_backward_workspace_bytes(int64_t G, int64_t V) {
  if (G < 0 || V < 0) return 0;
  return vertex_grad_bytes(G, V, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int mt_create_triangle_vertices_backward(const float* grid_signed_distances, int32_t C, const int32_t* lower_corners,
                                         int64_t G, const float* level_sets, int32_t S,
                                         const int32_t* vertex_offsets, const float* grad_vertices,
                                         const float* grad_signed_distances, const float* grad_spherical_harmonics,
                                         int64_t V, int32_t* corner_inverse, float* grad_grid_vertices,
                                         float* grad_grid_signed_distances, float* grad_grid_spherical_harmonics,
                                         void* workspace, size_t workspace_bytes, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && S >= 0 && C >= 1 && V >= 0);
  if (G == 0) return MT_OK;
  MT_REQUIRE(grid_signed_distances && lower_corners && corner_inverse);
  MT_REQUIRE(grad_grid_signed_distances && grad_grid_spherical_harmonics);
  MT_REQUIRE(S == 0 || (level_sets && vertex_offsets));
  MT_REQUIRE(grad_vertices == nullptr || grad_grid_vertices != nullptr);
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(corner_inverse, 0xff, (size_t)G * 4 * sizeof(int32_t), st) != cudaSuccess) return MT_ERR_CUDA;
  invert_corners_kernel<<<grid_stride_blocks(G, 256), 256, 0, st>>>(lower_corners, G, corner_inverse);
  MT_CHECK_LAUNCH();
  // With no level sets or no vertices, the gather writes zeros everywhere.
  const float* gv = V > 0 ? grad_vertices : nullptr;
  const float* gd = V > 0 ? grad_signed_distances : nullptr;
  const float* gs = V > 0 ? grad_spherical_harmonics : nullptr;
  const bool listed = S <= kShellsPerChunk && V < (int64_t)0x7fffffff && workspace &&
                      workspace_bytes >= vertex_grad_bytes(G, V, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (!listed) {
    create_vertices_backward_kernel<<<grid_stride_blocks(G, 128), 128, 0, st>>>(
        grid_signed_distances, C, lower_corners, G, level_sets, S, vertex_offsets, corner_inverse, gv, gd, gs, V,
        grad_grid_vertices, grad_grid_signed_distances, grad_grid_spherical_harmonics);
    MT_CHECK_LAUNCH();
    return MT_OK;
  }
  int32_t* counts = nullptr;
  int2* list = nullptr;
  void* scan_ws = nullptr;
  size_t scan_bytes = 0;
  vertex_grad_bytes(G, V, &counts, &list, &scan_ws, &scan_bytes, static_cast<char*>(workspace));
  vertex_grad_list_kernel<false><<<grid_stride_blocks(G, 128), 128, 0, st>>>(
      grid_signed_distances, lower_corners, G, level_sets, S, vertex_offsets, corner_inverse, V, counts, nullptr,
      nullptr, nullptr, nullptr, nullptr);
  MT_CHECK_LAUNCH();
  const int rc = mt_exclusive_scan_i32(counts, G + 1, scan_ws, scan_bytes, stream);
  if (rc != MT_OK) return rc;
  vertex_grad_list_kernel<true><<<grid_stride_blocks(G, 128), 128, 0, st>>>(
      grid_signed_distances, lower_corners, G, level_sets, S, vertex_offsets, corner_inverse, V, counts, list, gv,
      gd, grad_grid_vertices, grad_grid_signed_distances);
  MT_CHECK_LAUNCH();
  vertex_sh_gather_kernel<<<grid_stride_blocks((int64_t)C * G, 256), 256, 0, st>>>(gs, C, V, G, counts, list,
                                                                                 grad_grid_spherical_harmonics);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_count_triangle_faces(const float* signed_distances, const int32_t* lower_corners, int64_t G,
                            const int32_t* upper_corners, int64_t Nv, const float* level_sets, int32_t S,
                            int32_t* face_counts, uint8_t* cell_codes, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && Nv >= 0 && S >= 0 && face_counts);
  MT_REQUIRE(Nv == 0 || (signed_distances && lower_corners && upper_corners && cell_codes));
  MT_REQUIRE(S == 0 || level_sets);
  count_faces_kernel<<<grid_stride_blocks(Nv, 256), 256, 0, as_stream(stream)>>>(
      signed_distances, lower_corners, G, upper_corners, Nv, level_sets, S, face_counts, cell_codes);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_create_triangle_faces(const int32_t* neighbors, const int32_t* indices, int64_t Nv, int64_t G, int64_t V,
                             const int32_t* vertex_offsets, const uint8_t* vertex_types, const uint8_t* cell_codes,
                             int32_t S, const int32_t* face_offsets, int64_t F, int32_t* faces,
                             int32_t* voxel_indices, mt_stream_t stream) {
  MT_REQUIRE(Nv >= 0 && G >= 0 && V >= 0 && S >= 0 && F >= 0);
  if (Nv == 0 || S == 0 || F == 0) return MT_OK;
  MT_REQUIRE(neighbors && indices && vertex_offsets && vertex_types && cell_codes && face_offsets && faces &&
             voxel_indices);
  create_faces_kernel<<<grid_stride_blocks((int64_t)S * Nv, 256), 256, 0, as_stream(stream)>>>(
      neighbors, indices, Nv, G, V, vertex_offsets, vertex_types, cell_codes, S, face_offsets, F, faces,
      voxel_indices);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_compute_sdf_regularizers(const float* grid_signed_distances, const int32_t* voxel_neighbors,
                                const int32_t* voxel_lower_corners, int64_t G, const int32_t* voxel_upper_corners,
                                int64_t Nv, int32_t voxel_x, int32_t voxel_y, int32_t voxel_z,
                                float* eikonal_loss_pos, float* eikonal_loss_neg, float* curvature_loss,
                                mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && Nv >= 0);
  if (Nv == 0) return MT_OK;
  MT_REQUIRE(grid_signed_distances && voxel_neighbors && voxel_lower_corners && voxel_upper_corners &&
             eikonal_loss_pos && eikonal_loss_neg && curvature_loss);
  sdf_regularizers_kernel<<<grid_stride_blocks(Nv, 256), 256, 0, as_stream(stream)>>>(
      grid_signed_distances, voxel_neighbors, voxel_lower_corners, G, voxel_upper_corners, Nv, voxel_x, voxel_y,
      voxel_z, eikonal_loss_pos, eikonal_loss_neg, curvature_loss);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_compute_sdf_regularizers_backward(const float* grid_signed_distances, const int32_t* voxel_neighbors,
                                         const int32_t* voxel_lower_corners, int64_t G,
                                         const int32_t* voxel_upper_corners, int64_t Nv, int32_t voxel_x,
                                         int32_t voxel_y, int32_t voxel_z, const float* grad_eikonal_loss_pos,
                                         const float* grad_eikonal_loss_neg, const float* grad_curvature_loss,
                                         float* grad_grid_signed_distances, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && Nv >= 0 && grad_grid_signed_distances);
  cudaStream_t st = as_stream(stream);
  if (G > 0 && cudaMemsetAsync(grad_grid_signed_distances, 0, (size_t)G * sizeof(float), st) != cudaSuccess)
    return MT_ERR_CUDA;
  if (Nv == 0) return MT_OK;
  MT_REQUIRE(grid_signed_distances && voxel_neighbors && voxel_lower_corners && voxel_upper_corners);
  sdf_regularizers_backward_kernel<<<grid_stride_blocks(Nv, 256), 256, 0, st>>>(
      grid_signed_distances, voxel_neighbors, voxel_lower_corners, G, voxel_upper_corners, Nv, voxel_x, voxel_y,
      voxel_z, grad_eikonal_loss_pos, grad_eikonal_loss_neg, grad_curvature_loss, grad_grid_signed_distances);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_shell_boundaries(const int32_t* vertex_offsets, int64_t G, const int32_t* face_offsets, int64_t Nv, int32_t S,
                        int32_t* vertex_boundaries, int32_t* face_boundaries, int32_t* num_faces,
                        mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && Nv >= 0 && S >= 0);
  if (S == 0 && !num_faces) return MT_OK;
  MT_REQUIRE(vertex_offsets && face_offsets);
  MT_REQUIRE(S == 0 || (vertex_boundaries && face_boundaries));
  shell_boundaries_kernel<<<grid_1d(S > 0 ? S : 1, 128), 128, 0, as_stream(stream)>>>(
      vertex_offsets, G, face_offsets, Nv, S, vertex_boundaries, face_boundaries, num_faces);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_capacity_overflow(const int32_t* num_vertices, int64_t vertex_capacity, const int32_t* num_faces,
                         int64_t face_capacity, const int64_t* num_keys, int64_t key_capacity, uint8_t* overflow,
                         mt_stream_t stream) {
  MT_REQUIRE(overflow);
  capacity_overflow_kernel<<<1, 1, 0, as_stream(stream)>>>(num_vertices, vertex_capacity, num_faces, face_capacity,
                                                          num_keys, key_capacity, overflow);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_vertex_grad_list_max_shells(void) { return kShellsPerChunk; }

// Workspace: status word, the segment words [G], the scan's scratch.
static size_t segment_bytes(int64_t G) { return ((size_t)G * sizeof(uint32_t) + 255) & ~(size_t)255; }

size_t mt_build_vertex_grad_list_workspace_bytes(int64_t G) {
  return 256 + segment_bytes(G) + mt_scan_workspace_bytes(G + 1);
}

int mt_build_vertex_grad_list(const float* grid_signed_distances, const int32_t* lower_corners, int64_t G,
                              const float* level_sets, int32_t S, const int32_t* vertex_offsets, int64_t V,
                              int32_t* corner_inverse, int32_t* list_offsets, int32_t* list, void* workspace,
                              size_t workspace_bytes, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && S >= 0 && V >= 0);
  if (S > kShellsPerChunk || V >= (int64_t)0x7fffffff) return MT_ERR_TOO_LARGE;
  if (G == 0) return MT_OK;
  MT_REQUIRE(grid_signed_distances && lower_corners && corner_inverse && list_offsets && workspace);
  MT_REQUIRE(S == 0 || (level_sets && vertex_offsets));
  MT_REQUIRE(V == 0 || list);
  if (workspace_bytes < mt_build_vertex_grad_list_workspace_bytes(G)) return MT_ERR_WORKSPACE_TOO_SMALL;
  cudaStream_t st = as_stream(stream);
  char* ws = static_cast<char*>(workspace);
  uint32_t* segments = reinterpret_cast<uint32_t*>(ws + 256);
  const size_t scan_off = 256 + segment_bytes(G);
  if (cudaMemsetAsync(corner_inverse, 0xff, (size_t)G * 4 * sizeof(int32_t), st) != cudaSuccess) return MT_ERR_CUDA;
  invert_corners_kernel<<<grid_stride_blocks(G, 256), 256, 0, st>>>(lower_corners, G, corner_inverse, list_offsets,
                                                                    segments);
  MT_CHECK_LAUNCH();
  entry_list_kernel<false><<<grid_stride_blocks(G, 256), 256, 0, st>>>(
      grid_signed_distances, lower_corners, G, level_sets, S, vertex_offsets, corner_inverse, V, list_offsets,
      segments, nullptr);
  MT_CHECK_LAUNCH();
  const int rc = mt_exclusive_scan_i32(list_offsets, G + 1, ws + scan_off, workspace_bytes - scan_off, stream);
  if (rc != MT_OK) return rc;
  entry_list_kernel<true><<<grid_stride_blocks(G, 256), 256, 0, st>>>(
      grid_signed_distances, lower_corners, G, level_sets, S, vertex_offsets, corner_inverse, V, list_offsets,
      segments, reinterpret_cast<int2*>(list));
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_vertex_grads_from_list(const int32_t* list_offsets, const int32_t* list, int64_t G,
                              const float* grad_vertices, const float* grad_signed_distances,
                              float* grad_grid_vertices, float* grad_grid_signed_distances, mt_stream_t stream) {
  MT_REQUIRE(G >= 0);
  if (G == 0) return MT_OK;
  MT_REQUIRE(list_offsets && grad_grid_signed_distances);
  MT_REQUIRE(grad_vertices == nullptr || grad_grid_vertices != nullptr);
  vertex_grads_from_list_kernel<<<grid_stride_blocks(G, 256), 256, 0, as_stream(stream)>>>(
      list_offsets, reinterpret_cast<const int2*>(list), G, grad_vertices, grad_signed_distances, grad_grid_vertices,
      grad_grid_signed_distances);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_grid_sh_colors(const float* grid_spherical_harmonics, int32_t C, int64_t G, const int32_t* vertex_sources,
                      int64_t V, const int32_t* num_vertices, const float* vertices, int32_t sh_degree,
                      const float* camera_positions, int32_t B, float* out_colors, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && V >= 0 && B >= 0 && sh_degree >= 0 && sh_degree <= 3);
  const int n = (sh_degree + 1) * (sh_degree + 1);
  MT_REQUIRE(C >= n);
  if (V == 0 || B == 0) return MT_OK;
  MT_REQUIRE(grid_spherical_harmonics && vertex_sources && vertices && camera_positions && out_colors);
  grid_sh_colors_kernel<<<grid_stride_blocks(V, 256), 256, 0, as_stream(stream)>>>(
      grid_spherical_harmonics, G, vertex_sources, V, num_vertices, vertices, n, camera_positions, B, out_colors);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

size_t mt_grid_sh_colors_backward_workspace_bytes(int64_t V) {
  return 256 + (size_t)(V > 0 ? V : 0) * 48 * sizeof(float);
}

int mt_grid_sh_colors_backward(const int32_t* list_offsets, const int32_t* list, int64_t G, int64_t V,
                               const float* vertices, int32_t C, int32_t sh_degree, const float* camera_positions,
                               int32_t B, const float* out_colors, const float* grad_colors,
                               float* grad_grid_spherical_harmonics, const int32_t* num_vertices, void* workspace,
                               size_t workspace_bytes, mt_stream_t stream) {
  MT_REQUIRE(G >= 0 && V >= 0 && B >= 0 && sh_degree >= 0 && sh_degree <= 3);
  const int n = (sh_degree + 1) * (sh_degree + 1);
  MT_REQUIRE(C >= n);
  if (G == 0) return MT_OK;
  MT_REQUIRE(list_offsets && grad_grid_spherical_harmonics);
  // No cameras or vertices: every list sum is empty and the rows are zeros.
  const int Bn = V > 0 ? B : 0;
  MT_REQUIRE(Bn == 0 || (list && vertices && camera_positions && out_colors && grad_colors));
  cudaStream_t st = as_stream(stream);
  if (C > 16 && cudaMemsetAsync(grad_grid_spherical_harmonics + (size_t)16 * G * 3, 0,
                                (size_t)(C - 16) * G * 3 * sizeof(float), st) != cudaSuccess)
    return MT_ERR_CUDA;  // rows past degree 3's sixteen are zeros
  if (workspace && workspace_bytes >= mt_grid_sh_colors_backward_workspace_bytes(V) && Bn > 0) {
    float4* dsh = reinterpret_cast<float4*>(static_cast<char*>(workspace) + 256);
    MT_REQUIRE((reinterpret_cast<uintptr_t>(dsh) & 15) == 0);
    vertex_sh_grad_kernel<<<grid_stride_blocks(V, kShGradThreads), kShGradThreads, 0, st>>>(vertices, V, num_vertices, n, camera_positions,
                                                                      Bn, out_colors, grad_colors, dsh);
    MT_CHECK_LAUNCH();
    grid_sh_gather_kernel<<<grid_stride_blocks(2 * G, 256), 256, 0, st>>>(
        list_offsets, reinterpret_cast<const int2*>(list), G, dsh, C, n, grad_grid_spherical_harmonics);
    MT_CHECK_LAUNCH();
    return MT_OK;
  }
  const int64_t xblocks = (G + kShX - 1) / kShX;
  grid_sh_colors_backward_kernel<<<(unsigned)min(xblocks, (int64_t)152 * 32), kShThreads, 0, st>>>(
      list_offsets, reinterpret_cast<const int2*>(list), G, V, vertices, C, n, camera_positions, Bn, out_colors,
      grad_colors, grad_grid_spherical_harmonics);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
