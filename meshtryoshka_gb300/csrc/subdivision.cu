// Coarse-to-fine subdivision, occupancy mesh and vertex de-duplication for
// sm_103a:
//   write_occupancy     triangle_extraction/write_occupancy.slang:1-20
//   upscale_occupancy   triangle_extraction/upscale_occupancy.slang:1-74
//   upscale_parameters  triangle_extraction/upscale_parameters.slang:1-198
//   get_occupancy_mesh  triangle_extraction/get_occupancy_mesh.slang:1-220
//   index_vertices      triangle_extraction/index_vertices.py:6-51 (keys,
//                       then the library's stable sort, then run heads)
//
// Packed occupancy: int32 [i, j, kp], bit b of word kp = voxel k = 32 kp + b.
// Floating-point results follow the reference source's operations in order
// (this unit is compiled without multiply-add contraction).

#include "mt_common.cuh"

namespace mt {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// write_occupancy: set the bit of every triangle's voxel. Indices outside the
// grid are skipped (the reference writes them unchecked).
// ---------------------------------------------------------------------------
__global__ void write_occupancy_kernel(const int32_t* __restrict__ voxel_indices, int64_t n,
                                       int32_t* __restrict__ occupancy, int64_t words) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = voxel_indices[t];
    if (v < 0 || (int64_t)(v >> 5) >= words) continue;
    atomicOr(reinterpret_cast<unsigned int*>(occupancy) + (v >> 5), 1u << (v & 31));
  }
}

// ---------------------------------------------------------------------------
// upscale_occupancy: a new voxel (i, j, k) is occupied when any of its 8
// corners, mapped to the old grid by the unsigned integer arithmetic
//   old = ((new + side) * old_extent - side) / new_extent,
// lands in an occupied old voxel (optionally masked: old word & mask word).
//
// One thread per new word. The corner rows are (is, js) for the four
// (di, dj) sides, and since the new grid is at least as fine as the old one,
// the 32 bits x 2 sides of a new word map to old k in [ks_lo, ks_lo + 32]:
// at most two old words per row. So a word needs 8 loads (the reference
// samples 256), OR-ed across the four rows before the per-bit selection.
// ---------------------------------------------------------------------------
__global__ void upscale_occupancy_kernel(const int32_t* __restrict__ occ, const int32_t* __restrict__ mask,
                                         uint32_t I, uint32_t J, uint32_t KP, uint32_t I2, uint32_t J2,
                                         uint32_t KP2, int32_t* __restrict__ out) {
  const int64_t total = (int64_t)I2 * J2 * KP2;
  const uint32_t K = KP << 5, K2 = KP2 << 5;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t kp = (uint32_t)(w % KP2), j = (uint32_t)((w / KP2) % J2), i = (uint32_t)(w / ((int64_t)KP2 * J2));
    const uint32_t k_base = kp << 5;
    const uint32_t lo = ((k_base * K) / K2) >> 5;
    const bool has_hi = lo + 1 < KP;
    uint32_t a = 0, b = 0;
#pragma unroll
    for (uint32_t di = 0; di < 2; ++di) {
      const uint32_t is = ((i + di) * I - di) / I2;
#pragma unroll
      for (uint32_t dj = 0; dj < 2; ++dj) {
        const uint32_t js = ((j + dj) * J - dj) / J2;
        const int64_t row = ((int64_t)is * J + js) * KP;
        uint32_t wa = (uint32_t)__ldg(occ + row + lo);
        uint32_t wb = has_hi ? (uint32_t)__ldg(occ + row + lo + 1) : 0u;
        if (mask) {
          wa &= (uint32_t)__ldg(mask + row + lo);
          wb &= has_hi ? (uint32_t)__ldg(mask + row + lo + 1) : 0u;
        }
        a |= wa;
        b |= wb;
      }
    }
    uint32_t result = 0;
    if (a | b) {
      // The old k of both sides, k0 = (k K) / K2 and k1 = ((k + 1) K - 1) / K2,
      // stepped along the word: each bit adds K to both numerators, and since
      // K <= K2 a quotient grows by at most one per step.
      const uint32_t n0 = k_base * K, n1 = k_base * K + K - 1;
      uint32_t k0 = n0 / K2, r0 = n0 - k0 * K2;
      uint32_t k1 = n1 / K2, r1 = n1 - k1 * K2;
#pragma unroll 8
      for (uint32_t bit = 0; bit < 32; ++bit) {
        const uint32_t w0 = (k0 >> 5) == lo ? a : b;
        const uint32_t w1 = (k1 >> 5) == lo ? a : b;
        const uint32_t v = ((w0 >> (k0 & 31)) | (w1 >> (k1 & 31))) & 1u;
        result |= v << bit;
        r0 += K;
        if (r0 >= K2) r0 -= K2, ++k0;
        r1 += K;
        if (r1 >= K2) r1 -= K2, ++k1;
      }
    }
    out[w] = (int32_t)result;
  }
}

// ---------------------------------------------------------------------------
// upscale_parameters: every new grid vertex samples the old vertices'
// signed distance and SH trilinearly, renormalising over the old vertices
// that exist. Vertex occupancy grids are [I+1, J+1, KP+1] words; offsets are
// the exclusive scan of their bit counts (one per word).
// ---------------------------------------------------------------------------
struct OldGrid {
  const int32_t* occ;      // old vertex occupancy
  const int32_t* offsets;  // old per-word vertex offsets
  const float* sdf;
  const float* sh;  // [C, Vold, 3]
  int64_t Vold;
  int I1, J1, KP1;  // old vertex occupancy dims
};

// The old vertex at (i, j, k), or -1 when outside the grid or unoccupied
// (read_vertex, upscale_parameters.slang:9-53; k is never negative here).
__device__ __forceinline__ int64_t old_vertex(const OldGrid& g, int i, int j, int k) {
  if (i < 0 || j < 0 || k < 0) return -1;
  const int kp = k / 32;
  if (i >= g.I1 || j >= g.J1 || kp >= g.KP1) return -1;
  const int bit = k % 32;
  const int64_t word = ((int64_t)i * g.J1 + j) * g.KP1 + kp;
  const uint32_t chunk = (uint32_t)__ldg(g.occ + word);
  if ((chunk & (1u << bit)) == 0) return -1;
  return (int64_t)__ldg(g.offsets + word) + __popc(chunk & ((1u << bit) - 1u));
}

// SH planes [c0, c0 + N) of one new vertex: per plane and channel, the sum
// over the present corners in corner order, times the normaliser. The N
// planes are independent sums, interleaved for memory-level parallelism.
template <int N>
__device__ __forceinline__ void upscale_planes(const OldGrid& g, int c0, const int64_t (&ids)[8],
                                               const float (&wts)[8], float mult, int64_t Vnew, int64_t vi,
                                               float* __restrict__ new_sh) {
  float acc[N][3];
#pragma unroll
  for (int n = 0; n < N; ++n) acc[n][0] = acc[n][1] = acc[n][2] = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (ids[q] < 0) continue;
#pragma unroll
    for (int n = 0; n < N; ++n) {
      const float* src = g.sh + ((int64_t)(c0 + n) * g.Vold + ids[q]) * 3;
      acc[n][0] += wts[q] * __ldg(src + 0);
      acc[n][1] += wts[q] * __ldg(src + 1);
      acc[n][2] += wts[q] * __ldg(src + 2);
    }
  }
#pragma unroll
  for (int n = 0; n < N; ++n) {
    float* dst = new_sh + ((int64_t)(c0 + n) * Vnew + vi) * 3;
    dst[0] = acc[n][0] * mult;
    dst[1] = acc[n][1] * mult;
    dst[2] = acc[n][2] * mult;
  }
}

// Position of the n-th (0-based) set bit of x (n < popc(x)).
__device__ __forceinline__ int select_bit(uint32_t x, int n) {
  int pos = 0;
#pragma unroll
  for (int width = 16; width > 0; width >>= 1) {
    const int c = __popc(x & ((1u << width) - 1u));
    if (n >= c) {
      n -= c;
      x >>= width;
      pos += width;
    }
  }
  return pos;
}

// A warp reads 32 consecutive new vertex-occupancy words (one coalesced
// load) and deals their vertices out 32 at a time: lane r takes the r-th
// vertex of the span, whose word is found by a shuffle search over the
// warp's running bit counts and whose bit by a popcount select. Offsets are
// an exclusive scan in word order, so that vertex is offset[first word] + r:
// every lane is busy and every [C, V, 3] row the warp stores is contiguous.
__global__ void __launch_bounds__(256)
    upscale_parameters_kernel(OldGrid g, int C, const int32_t* __restrict__ new_occ,
                              const int32_t* __restrict__ new_offsets, int I1n, int J1n, int KP1n, int64_t Vnew,
                              float* __restrict__ new_sdf, float* __restrict__ new_sh) {
  const int64_t total = (int64_t)I1n * J1n * KP1n;
  const int lane = threadIdx.x & 31;
  const int64_t first_warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // New grid position scale (upscale_parameters.slang:141-160).
  const int i_max = I1n - 1, j_max = J1n - 1, kp_max = KP1n - 1;
  const float inv_i_max = 1.0f / (float)i_max;
  const float inv_j_max = 1.0f / (float)j_max;
  const float inv_k_max = 1.0f / (float)(32 * kp_max);
  // Old grid scale (sample_trilinear, :63-65).
  const float sx = (float)((g.KP1 - 1) * 32), sy = (float)(g.J1 - 1), sz = (float)(g.I1 - 1);
  for (int64_t base = first_warp * 32; base < total; base += warps * 32) {
    const int64_t mine = base + lane;
    const uint32_t my_chunk = mine < total ? (uint32_t)__ldg(new_occ + mine) : 0u;
    const int my_count = __popc(my_chunk);
    int incl = my_count;  // inclusive scan of the bit counts over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int span = __shfl_sync(0xffffffffu, incl, 31);
    if (span == 0) continue;
    const int64_t first_vertex = __ldg(new_offsets + base);
    for (int start = 0; start < span; start += 32) {
      const int r = start + lane;
      // Smallest word index src with incl[src] > r.
      int src = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int v = __shfl_sync(0xffffffffu, incl, src + step - 1);
        if (v <= r) src += step;
      }
      const uint32_t chunk = __shfl_sync(0xffffffffu, my_chunk, src);
      const int before = __shfl_sync(0xffffffffu, incl - my_count, src);
      if (r >= span) continue;
      const int64_t vi = first_vertex + r;
      if (vi < 0 || vi >= Vnew) continue;
      const int bit = select_bit(chunk, r - before);
      const int64_t w = base + src;
      const int kp = (int)(w % KP1n), j = (int)((w / KP1n) % J1n), i = (int)(w / ((int64_t)KP1n * J1n));
      const int k = 32 * kp + bit;
      const float x = (float)k * inv_k_max, y = (float)j * inv_j_max, z = (float)i * inv_i_max;
      const float xu = x * sx, yu = y * sy, zu = z * sz;
      const int oi = (int)zu, oj = (int)yu, ok = (int)xu;
      const float ti = fmodf(zu, 1.0f), tj = fmodf(yu, 1.0f), tk = fmodf(xu, 1.0f);
      // Per-corner vertex (-1 = absent) and weight, indexed statically so
      // that both stay in registers.
      int64_t ids[8];
      float wts[8];
      float den = 0.0f, d = 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
        int64_t ov = old_vertex(g, oi + di, oj + dj, ok + dk);
        if (ov >= g.Vold) ov = -1;
        const float wgt = (di == 0 ? 1.0f - ti : ti) * (dj == 0 ? 1.0f - tj : tj) * (dk == 0 ? 1.0f - tk : tk);
        ids[q] = ov;
        wts[q] = wgt;
        if (ov >= 0) {
          d += wgt * __ldg(g.sdf + ov);
          den += wgt;
        }
      }
      const float mult = 1.0f / den;
      new_sdf[vi] = d * mult;
      int c = 0;
      for (; c + 4 <= C; c += 4) upscale_planes<4>(g, c, ids, wts, mult, Vnew, vi, new_sh);
      for (; c < C; ++c) upscale_planes<1>(g, c, ids, wts, mult, Vnew, vi, new_sh);
    }
  }
}

// ---------------------------------------------------------------------------
// get_occupancy_mesh: two triangles per boundary face between occupied and
// free voxels; each (i, j, kp) entry of the [I+1, J+1, KP+1] grid owns the
// faces on its lower i, j and k sides.
// ---------------------------------------------------------------------------
struct Neighbourhood {
  uint32_t here, minus_i, minus_j;
  bool minus_k;
};

__device__ __forceinline__ Neighbourhood neighbourhood(const int32_t* __restrict__ occ, int I, int J, int KP, int i,
                                                       int j, int kp) {
  const bool il = i == I, jl = j == J, kl = kp == KP;
  auto at = [&](int a, int b, int c) { return (uint32_t)__ldg(occ + ((int64_t)a * J + b) * KP + c); };
  Neighbourhood n;
  n.here = (il || jl || kl) ? 0u : at(i, j, kp);
  n.minus_i = (jl || kl || i == 0) ? 0u : at(i - 1, j, kp);
  n.minus_j = (il || kl || j == 0) ? 0u : at(i, j - 1, kp);
  n.minus_k = (il || jl || kp == 0) ? false : ((at(i, j, kp - 1) & 0x80000000u) != 0);
  return n;
}

// Bits with a face on the lower k side: where a bit differs from the one
// before it (bit 0 against bit 31 of the previous word).
__device__ __forceinline__ uint32_t k_faces(const Neighbourhood& n) {
  return n.here ^ ((n.here << 1) | (n.minus_k ? 1u : 0u));
}

__global__ void count_mesh_triangles_kernel(const int32_t* __restrict__ occ, int I, int J, int KP,
                                            int32_t* __restrict__ counts) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int kp = (int)(w % (KP + 1)), j = (int)((w / (KP + 1)) % (J + 1)), i = (int)(w / ((int64_t)(KP + 1) * (J + 1)));
    const Neighbourhood n = neighbourhood(occ, I, J, KP, i, j, kp);
    counts[w] = 2 * (__popc(n.here ^ n.minus_i) + __popc(n.here ^ n.minus_j) + __popc(k_faces(n)));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counts[total] = 0;
}

// create_face (get_occupancy_mesh.slang:56-120): the face of `axis` at the
// entry's lower side, two triangles wound by `upper`, each corner written
// as (component 2, 1, 0) of its (i, j, k)-ordered coordinates.
__device__ __forceinline__ void write_face(int64_t index, int i, int j, int k, const int (&ijk_max)[3], int axis,
                                           bool upper, float* __restrict__ verts, float* __restrict__ tri_colors,
                                           const float* __restrict__ colors) {
  const int ijk[3] = {i, j, k};
  const int a0 = (axis + 1) % 3, a1 = (axis + 2) % 3;
  float v00[3], v01[3], v10[3], v11[3];
  const float plane = (float)ijk[axis] / (float)ijk_max[axis];
  v00[axis] = v01[axis] = v10[axis] = v11[axis] = plane;
  const float v0x = (float)ijk[a0] / (float)ijk_max[a0];
  const float v1x = (float)(ijk[a0] + 1) / (float)ijk_max[a0];
  const float vx0 = (float)ijk[a1] / (float)ijk_max[a1];
  const float vx1 = (float)(ijk[a1] + 1) / (float)ijk_max[a1];
  v00[a0] = v0x;
  v00[a1] = vx0;
  v01[a0] = v0x;
  v01[a1] = vx1;
  v10[a0] = v1x;
  v10[a1] = vx0;
  v11[a0] = v1x;
  v11[a1] = vx1;
  const float* col = colors + (axis * 2 + (upper ? 1 : 0)) * 3;
  const float* tris[2][3] = {{v00, upper ? v01 : v10, upper ? v10 : v01}, {v11, upper ? v10 : v01, upper ? v01 : v10}};
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    float* out = verts + (index + t) * 9;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      out[3 * c + 0] = tris[t][c][2];
      out[3 * c + 1] = tris[t][c][1];
      out[3 * c + 2] = tris[t][c][0];
    }
    float* oc = tri_colors + (index + t) * 3;
    oc[0] = col[0];
    oc[1] = col[1];
    oc[2] = col[2];
  }
}

__global__ void create_mesh_triangles_kernel(const int32_t* __restrict__ occ, int I, int J, int KP,
                                             const int32_t* __restrict__ offsets, int64_t T,
                                             const float* __restrict__ colors, float* __restrict__ verts,
                                             float* __restrict__ tri_colors) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  const int ijk_max[3] = {I, J, KP * 32};
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int kp = (int)(w % (KP + 1)), j = (int)((w / (KP + 1)) % (J + 1)), i = (int)(w / ((int64_t)(KP + 1) * (J + 1)));
    const Neighbourhood n = neighbourhood(occ, I, J, KP, i, j, kp);
    const uint32_t fi = n.here ^ n.minus_i, fj = n.here ^ n.minus_j, fk = k_faces(n);
    uint32_t any = fi | fj | fk;
    int64_t index = offsets[w];
    while (any) {
      const int bit = __ffs(any) - 1;
      any &= any - 1;
      const bool h = (n.here >> bit) & 1u;
      const int k = kp * 32 + bit;
      // Faces with normals along i, then j, then k (get_occupancy_mesh.slang:168-210).
      if (((fi >> bit) & 1u) && index + 2 <= T) {
        write_face(index, i, j, k, ijk_max, 0, h, verts, tri_colors, colors);
        index += 2;
      }
      if (((fj >> bit) & 1u) && index + 2 <= T) {
        write_face(index, i, j, k, ijk_max, 1, h, verts, tri_colors, colors);
        index += 2;
      }
      if (((fk >> bit) & 1u) && index + 2 <= T) {
        write_face(index, i, j, k, ijk_max, 2, h, verts, tri_colors, colors);
        index += 2;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// index_vertices (index_vertices.py:6-51).
//
// Quantization follows torch's CUDA kernels for round(points / tol): a
// division by a host scalar is a multiplication by its float reciprocal,
// then round half to even, then a truncating conversion to int64.
// ---------------------------------------------------------------------------
__global__ void quantize_points_kernel(const float* __restrict__ points, int64_t n, float inv_tol,
                                       int64_t* __restrict__ q, unsigned long long* __restrict__ max_abs) {
  unsigned long long m = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float r = rintf(__fmul_rn(points[e], inv_tol));
    const int64_t v = (int64_t)r;
    q[e] = v;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    m = a > m ? a : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, m, o);
    m = other > m ? other : m;
  }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(max_abs, m);
}

// keys = (x << 2 shift) | (y << shift) | z with two's complement shifts,
// values = 0 .. V-1.
__global__ void pack_point_keys_kernel(const int64_t* __restrict__ q, int64_t V, int shift,
                                       int64_t* __restrict__ keys, int32_t* __restrict__ values) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t x = (uint64_t)q[3 * v + 0], y = (uint64_t)q[3 * v + 1], z = (uint64_t)q[3 * v + 2];
    keys[v] = (int64_t)((x << (2 * shift)) | (y << shift) | z);
    values[v] = (int32_t)v;
  }
}

__global__ void iota_kernel(int64_t n, int32_t* __restrict__ values) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    values[v] = (int32_t)v;
}

// Every sorted position p maps its original index to the original index at
// the start of its run of equal keys. The sort is stable over 0..n-1, so the
// run starts at the smallest original index: the first seen. The run start
// is the lower bound of the key (sorted in signed order) in [0, p].
__global__ void run_heads_kernel(const int64_t* __restrict__ sorted_keys, const int32_t* __restrict__ order,
                                 int64_t n, int32_t* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t key = sorted_keys[p];
    int64_t start = p;
    if (p > 0 && sorted_keys[p - 1] == key) {
      int64_t lo = 0, hi = p - 1;  // sorted_keys[hi] == key
      while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if (sorted_keys[mid] < key) lo = mid + 1;
        else hi = mid;
      }
      start = lo;
    }
    const int32_t dst = order[p];
    if (dst >= 0 && dst < n) out[dst] = order[start];
  }
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

int mt_write_occupancy(const int32_t* voxel_indices, int64_t n, int32_t* occupancy, int64_t words,
                       mt_stream_t stream) {
  MT_REQUIRE(n >= 0 && words >= 0);
  if (n == 0 || words == 0) return MT_OK;
  MT_REQUIRE(voxel_indices && occupancy);
  write_occupancy_kernel<<<grid_stride_blocks(n, kThreads), kThreads, 0, as_stream(stream)>>>(voxel_indices, n,
                                                                                            occupancy, words);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_upscale_occupancy(const int32_t* occupancy, const int32_t* mask, int32_t I, int32_t J, int32_t KP,
                         int32_t I2, int32_t J2, int32_t KP2, int32_t* out, mt_stream_t stream) {
  MT_REQUIRE(I > 0 && J > 0 && KP > 0 && I2 >= I && J2 >= J && KP2 >= KP);
  // The reference's corner arithmetic is 32-bit unsigned: keep it exact.
  MT_REQUIRE((uint64_t)(I2 + 1) * (uint64_t)I <= 0xffffffffull && (uint64_t)(J2 + 1) * (uint64_t)J <= 0xffffffffull &&
             (uint64_t)(KP2 + 1) * 32ull * (uint64_t)KP * 32ull <= 0xffffffffull);
  MT_REQUIRE(occupancy && out);
  const int64_t total = (int64_t)I2 * J2 * KP2;
  upscale_occupancy_kernel<<<grid_stride_blocks(total, kThreads), kThreads, 0, as_stream(stream)>>>(
      occupancy, mask, (uint32_t)I, (uint32_t)J, (uint32_t)KP, (uint32_t)I2, (uint32_t)J2, (uint32_t)KP2, out);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_upscale_parameters(const int32_t* old_vertex_occupancy, const int32_t* old_vertex_offsets,
                          const float* old_signed_distances, const float* old_spherical_harmonics, int32_t C,
                          int64_t Vold, int32_t I1, int32_t J1, int32_t KP1, const int32_t* new_vertex_occupancy,
                          const int32_t* new_vertex_offsets, int32_t I1n, int32_t J1n, int32_t KP1n, int64_t Vnew,
                          float* new_signed_distances, float* new_spherical_harmonics, mt_stream_t stream) {
  MT_REQUIRE(C >= 1 && Vold >= 0 && Vnew >= 0 && I1 >= 2 && J1 >= 2 && KP1 >= 2 && I1n >= 2 && J1n >= 2 &&
             KP1n >= 2);
  if (Vnew == 0) return MT_OK;
  MT_REQUIRE(old_vertex_occupancy && old_vertex_offsets && new_vertex_occupancy && new_vertex_offsets &&
             new_signed_distances && new_spherical_harmonics);
  MT_REQUIRE(Vold == 0 || (old_signed_distances && old_spherical_harmonics));
  OldGrid g{old_vertex_occupancy, old_vertex_offsets, old_signed_distances, old_spherical_harmonics, Vold, I1, J1,
            KP1};
  const int64_t total = (int64_t)I1n * J1n * KP1n;
  upscale_parameters_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(
      g, C, new_vertex_occupancy, new_vertex_offsets, I1n, J1n, KP1n, Vnew, new_signed_distances,
      new_spherical_harmonics);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_count_occupancy_mesh_triangles(const int32_t* occupancy, int32_t I, int32_t J, int32_t KP, int32_t* counts,
                                      mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0 && counts);
  MT_REQUIRE((I == 0 || J == 0 || KP == 0) || occupancy);
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  count_mesh_triangles_kernel<<<grid_stride_blocks(total, kThreads), kThreads, 0, as_stream(stream)>>>(
      occupancy, I, J, KP, counts);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_create_occupancy_mesh_triangles(const int32_t* occupancy, int32_t I, int32_t J, int32_t KP,
                                       const int32_t* offsets, int64_t T, const float* colors, float* vertices,
                                       float* triangle_colors, mt_stream_t stream) {
  MT_REQUIRE(I >= 0 && J >= 0 && KP >= 0 && T >= 0);
  if (T == 0) return MT_OK;
  MT_REQUIRE(occupancy && offsets && colors && vertices && triangle_colors);
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  create_mesh_triangles_kernel<<<grid_stride_blocks(total, 128), 128, 0, as_stream(stream)>>>(
      occupancy, I, J, KP, offsets, T, colors, vertices, triangle_colors);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_quantize_points(const float* points, int64_t V, float inv_tol, int64_t* quantized, uint64_t* max_abs,
                       mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && max_abs);
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(max_abs, 0, sizeof(uint64_t), s) != cudaSuccess) return MT_ERR_CUDA;
  if (V == 0) return MT_OK;
  MT_REQUIRE(points && quantized);
  quantize_points_kernel<<<grid_stride_blocks(3 * V, kThreads), kThreads, 0, s>>>(
      points, 3 * V, inv_tol, quantized, reinterpret_cast<unsigned long long*>(max_abs));
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_pack_point_keys(const int64_t* quantized, int64_t V, int32_t shift, int64_t* keys, int32_t* values,
                       mt_stream_t stream) {
  MT_REQUIRE(V >= 0 && V <= 0x7fffffffll && shift >= 0 && shift <= 21);
  if (V == 0) return MT_OK;
  MT_REQUIRE(quantized && keys && values);
  pack_point_keys_kernel<<<grid_stride_blocks(V, kThreads), kThreads, 0, as_stream(stream)>>>(quantized, V, shift,
                                                                                            keys, values);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_iota_i32(int64_t n, int32_t* values, mt_stream_t stream) {
  MT_REQUIRE(n >= 0 && n <= 0x7fffffffll);
  if (n == 0) return MT_OK;
  MT_REQUIRE(values);
  iota_kernel<<<grid_stride_blocks(n, kThreads), kThreads, 0, as_stream(stream)>>>(n, values);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_index_sorted_runs(const int64_t* sorted_keys, const int32_t* order, int64_t n, int32_t* out,
                         mt_stream_t stream) {
  MT_REQUIRE(n >= 0 && n <= 0x7fffffffll);
  if (n == 0) return MT_OK;
  MT_REQUIRE(sorted_keys && order && out);
  run_heads_kernel<<<grid_stride_blocks(n, kThreads), kThreads, 0, as_stream(stream)>>>(sorted_keys, order, n, out);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
