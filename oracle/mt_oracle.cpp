// CPU oracle for the meshtryoshka_gb300 render path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, on the host, the algorithm of
// each reference kernel on the path (Slang sources of dcharatan/meshtryoshka,
// cited per function as path:line). It is the parity checker for the CUDA
// library and the timed CPU baseline; nothing in the product imports it.
//
// Parity status: the integer/topology kernels restate the reference loops
// statement by statement (including the arithmetic-shift and last-bit cases of
// create_voxels). The reference itself cannot be executed in this environment
// (its kernels need slangtorch, which is absent), so bit patterns of the
// floating-point kernels are defined here by an explicit operation order:
// fused multiply-adds are written as std::fmaf where the GPU kernels use
// __fmaf_rn, everything else is a single IEEE operation, and the file is
// compiled with -ffp-contract=off so the host compiler adds no contraction.
//
// Conventions: host pointers, dense row-major arrays, the same shapes as the
// reference tensors. OpenMP parallelises independent work items; scatters
// that the reference performs with atomics use omp atomic.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../meshtryoshka_gb300/csrc/mc_tables.h"

namespace {

// ---------------------------------------------------------------------------
// The reference's flat MC tables (triangle_extraction/constants.slang:1-142),
// rebuilt from the per-case encoding. FIRST is a prefix sum of the per-case
// counts, IDS the concatenated edge lists.
// ---------------------------------------------------------------------------
struct McTables {
  int first[257];
  int ids[MT_MC_TOTAL_IDS];
  int owner[12];
  int axis[12];
  McTables() {
    static const uint8_t counts[256] = {MT_MC_CASE_COUNT_VALUES};
    static const uint64_t edges[256] = {MT_MC_CASE_EDGES_VALUES};
    static const int8_t owners[12] = {MT_MC_EDGE_OWNER_VALUES};
    static const uint8_t axes[12] = {MT_MC_EDGE_AXIS_VALUES};
    first[0] = 0;
    for (int c = 0; c < 256; ++c) {
      for (int e = 0; e < counts[c]; ++e) ids[first[c] + e] = (int)((edges[c] >> (4 * e)) & 15u);
      first[c + 1] = first[c] + counts[c];
    }
    for (int e = 0; e < 12; ++e) {
      owner[e] = owners[e];
      axis[e] = axes[e];
    }
  }
};
const McTables kMc;

inline uint64_t fnv1a(const int* v, int n) {
  uint64_t h = 0xCBF29CE484222325ull;
  for (int i = 0; i < n; ++i) {
    const uint32_t x = (uint32_t)v[i];
    for (int b = 0; b < 4; ++b) {
      h ^= (x >> (8 * b)) & 0xffu;
      h *= 0x100000001B3ull;
    }
  }
  return h;
}

inline int popcount32(uint32_t x) { return __builtin_popcount(x); }

}  // namespace

extern "C" {

// Checksums of the rebuilt flat tables; equal to the reference's if the
// per-case encoding round-trips.
uint64_t or_mc_first_checksum(void) { return fnv1a(kMc.first, 257); }
uint64_t or_mc_ids_checksum(void) { return fnv1a(kMc.ids, MT_MC_TOTAL_IDS); }

// std::exclusive_scan semantics (CUB DeviceScan::ExclusiveSum,
// triangle_extraction/compute_exclusive_cumsum.cu:17-38), in place.
void or_exclusive_scan_i32(int32_t* data, int64_t n) {
  int32_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t x = data[i];
    data[i] = acc;
    acc += x;
  }
}

void or_exclusive_scan_i64(int64_t* data, int64_t n) {
  int64_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t x = data[i];
    data[i] = acc;
    acc += x;
  }
}

// torch.cumsum(int32 -> int64), triangle_rasterization/generate_keys.py:48.
void or_inclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n) {
  int64_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    acc += in[i];
    out[i] = acc;
  }
}

// ---------------------------------------------------------------------------
// triangle_extraction/compute_vertex_occupancy.slang:9-68
// ---------------------------------------------------------------------------
void or_compute_vertex_occupancy(const int32_t* occ, int I, int J, int KP, int32_t* vocc, int32_t* vcounts) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
#pragma omp parallel for schedule(static)
  for (int i = 0; i <= I; ++i) {
    for (int j = 0; j <= J; ++j) {
      for (int kp = 0; kp <= KP; ++kp) {
        int32_t result = 0;
        for (int di = 0; di < 2; ++di) {
          for (int dj = 0; dj < 2; ++dj) {
            if ((i == 0 && di == 1) || (j == 0 && dj == 1)) continue;
            if ((i == I && di == 0) || (j == J && dj == 0)) continue;
            const int64_t row = ((int64_t)(i - di) * J + (j - dj)) * KP;
            const int32_t current = (kp == KP) ? 0 : occ[row + kp];
            const int32_t previous_packed = (kp == 0) ? 0 : occ[row + kp - 1];
            // logical_right_shift (compute_vertex_occupancy.slang:1-5)
            const int32_t previous = (int32_t)((uint32_t)previous_packed >> 31) | (int32_t)((uint32_t)current << 1);
            result |= (current | previous);
          }
        }
        const int64_t w = ((int64_t)i * (J + 1) + j) * (KP + 1) + kp;
        vocc[w] = result;
        vcounts[w] = popcount32((uint32_t)result);
      }
    }
  }
  vcounts[total] = 0;  // compute_vertex_occupancy.py:58
}

// triangle_extraction/count_occupancy.slang:3-20 (output zero-filled first,
// count_occupancy.py:30).
void or_count_occupancy(const int32_t* occ, int I, int J, int KP, int32_t* counts) {
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
  std::memset(counts, 0, (size_t)(total + 1) * sizeof(int32_t));
  for (int i = 0; i < I; ++i)
    for (int j = 0; j < J; ++j)
      for (int kp = 0; kp < KP; ++kp)
        counts[((int64_t)i * (J + 1) + j) * (KP + 1) + kp] = popcount32((uint32_t)occ[((int64_t)i * J + j) * KP + kp]);
}

// ---------------------------------------------------------------------------
// triangle_extraction/create_voxels.slang:3-276, one loop iteration per GPU
// thread of the reference (one packed word of the vertex grid), with the same
// serial 32-bit walk. Slang `int >>=` is an arithmetic shift; C++20 defines
// signed right shift the same way.
// ---------------------------------------------------------------------------
void or_create_voxels(const int32_t* occ, const int32_t* xoff, const int32_t* vocc, const int32_t* voff, int I,
                      int J, int KP, int64_t num_voxels, int64_t num_vertices, float* vertices, int32_t* neighbors,
                      int32_t* lower, int32_t* upper, int32_t* indices) {
  if (num_voxels <= 0) return;  // create_voxels.py:67
  const int64_t G = num_vertices, Nv = num_voxels;
  auto W = [&](int i, int j, int kp) { return ((int64_t)i * (J + 1) + j) * (KP + 1) + kp; };
  auto OCC = [&](int i, int j, int kp) { return occ[((int64_t)i * J + j) * KP + kp]; };
  const float inv_i_max = 1.0f / (float)I;
  const float inv_j_max = 1.0f / (float)J;
  const float inv_k_max = 1.0f / (float)(32 * KP);
  const int32_t k_max = KP * 32;

#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i <= I; ++i) {
    for (int j = 0; j <= J; ++j) {
      for (int kp = 0; kp <= KP; ++kp) {
        const int32_t k_unpacked = 32 * kp;
        // Vertices (:37-53).
        int32_t vertex_index = voff[W(i, j, kp)];
        int32_t chunk = vocc[W(i, j, kp)];
        int32_t k = k_unpacked;
        for (int bit = 0; bit < 32; ++bit) {
          if ((chunk & 1) == 1) {
            vertices[3 * (int64_t)vertex_index + 0] = (float)k * inv_k_max;
            vertices[3 * (int64_t)vertex_index + 1] = (float)j * inv_j_max;
            vertices[3 * (int64_t)vertex_index + 2] = (float)i * inv_i_max;
            vertex_index++;
          }
          chunk >>= 1;
          k++;
        }

        // Local state of the 2x2 neighbouring words (:55-93).
        int32_t lvi[2][2], lvo[2][2], lxi[2][2], lxo[2][2], lsi[2][2], lso[2][2];
        for (int di = 0; di < 2; ++di) {
          for (int dj = 0; dj < 2; ++dj) {
            const int ii = i + di, jj = j + dj;
            if (ii > I || jj > J) {
              lvi[di][dj] = -64;
              lvo[di][dj] = 0;
              lxi[di][dj] = -64;
              lxo[di][dj] = 0;
              lsi[di][dj] = -64;
              lso[di][dj] = 0;
              continue;
            }
            const bool valid_voxel = (ii < I && jj < J && kp < KP);
            const int32_t local_voxel_index = xoff[W(ii, jj, kp)];
            const int32_t local_voxel_occupancy = valid_voxel ? OCC(ii, jj, kp) : 0;
            const int32_t local_vertex_index = voff[W(ii, jj, kp)];
            const int32_t local_vertex_occupancy = vocc[W(ii, jj, kp)];
            lvi[di][dj] = local_voxel_index;
            lvo[di][dj] = local_voxel_occupancy;
            lxi[di][dj] = local_vertex_index;
            lxo[di][dj] = local_vertex_occupancy;
            lsi[di][dj] = (int32_t)(Nv + local_vertex_index - local_voxel_index);
            lso[di][dj] = local_vertex_occupancy & ~local_voxel_occupancy;
          }
        }

        k = k_unpacked;
        for (int bit = 0; bit < 32; ++bit) {
          const bool is_voxel = (lvo[0][0] & 1) != 0;
          const bool is_subvoxel = (lso[0][0] & 1) != 0;
          const int32_t voxel_index = lvi[0][0];

          if (is_voxel || is_subvoxel) {  // :108-127
            const int64_t chosen = is_voxel ? voxel_index : lsi[0][0];
            lower[chosen] = lxi[0][0];
            const bool x_valid = is_voxel || ((lxo[0][0] & 2) != 0);
            const bool y_valid = is_voxel || ((lxo[0][1] & 1) != 0);
            const bool z_valid = is_voxel || ((lxo[1][0] & 1) != 0);
            lower[G + chosen] = x_valid ? lxi[0][0] + 1 : -64;
            lower[2 * G + chosen] = y_valid ? lxi[0][1] : -64;
            lower[3 * G + chosen] = z_valid ? lxi[1][0] : -64;
          }

          if (is_voxel) {  // :129-136
            upper[voxel_index] = lxi[1][1] + 1;
            upper[Nv + voxel_index] = lxi[1][1];
            upper[2 * Nv + voxel_index] = lxi[1][0] + 1;
            upper[3 * Nv + voxel_index] = lxi[0][1] + 1;
            indices[voxel_index] = k_max * (J * i + j) + k;
          }

          if (is_voxel && bit != 31) {  // :138-193
            const bool x_is_subvoxel = (lso[0][0] & 2) != 0;
            neighbors[voxel_index] = x_is_subvoxel ? lsi[0][0] : lvi[0][0] + 1;
            const bool y_is_subvoxel = (lso[0][1] & 1) != 0;
            neighbors[Nv + voxel_index] = y_is_subvoxel ? lsi[0][1] : lvi[0][1];
            const bool z_is_subvoxel = (lso[1][0] & 1) != 0;
            neighbors[2 * Nv + voxel_index] = z_is_subvoxel ? lsi[1][0] : lvi[1][0];
            const bool xy_is_subvoxel = (lso[0][1] & 2) != 0;
            neighbors[3 * Nv + voxel_index] = xy_is_subvoxel ? (y_is_subvoxel ? lsi[0][1] + 1 : lsi[0][1])
                                                             : (y_is_subvoxel ? lvi[0][1] : lvi[0][1] + 1);
            const bool yz_is_subvoxel = (lso[1][1] & 1) != 0;
            neighbors[4 * Nv + voxel_index] = yz_is_subvoxel ? lsi[1][1] : lvi[1][1];
            const bool xz_is_subvoxel = (lso[1][0] & 2) != 0;
            neighbors[5 * Nv + voxel_index] = xz_is_subvoxel ? (z_is_subvoxel ? lsi[1][0] + 1 : lsi[1][0])
                                                             : (z_is_subvoxel ? lvi[1][0] : lvi[1][0] + 1);
            const bool xyz_is_subvoxel = (lso[1][1] & 2) != 0;
            neighbors[6 * Nv + voxel_index] = xyz_is_subvoxel ? (yz_is_subvoxel ? lsi[1][1] + 1 : lsi[1][1])
                                                              : (yz_is_subvoxel ? lvi[1][1] : lvi[1][1] + 1);
          }

          if (bit != 31) {  // :195-207
            for (int di = 0; di < 2; ++di) {
              for (int dj = 0; dj < 2; ++dj) {
                lvi[di][dj] += (lvo[di][dj] & 1);
                lvo[di][dj] >>= 1;
                lxi[di][dj] += (lxo[di][dj] & 1);
                lxo[di][dj] >>= 1;
                lsi[di][dj] += (lso[di][dj] & 1);
                lso[di][dj] >>= 1;
              }
            }
          }
          k++;
        }

        // +x lower corner of a subvoxel at the last bit (:211-216).
        if ((lso[0][0] & 1) != 0) {
          const bool x_valid = (kp < KP) && ((vocc[W(i, j, kp + 1)] & 1) != 0);
          lower[G + lsi[0][0]] = x_valid ? lxi[0][0] + 1 : -64;
        }

        // Neighbours of a voxel at the last bit (:218-275).
        if ((lvo[0][0] & 1) == 0) continue;
        const int32_t voxel_index = lvi[0][0];
        const bool can_x = (kp < KP - 1), can_y = (j < J - 1), can_z = (i < I - 1);
        const int32_t top = (int32_t)0x80000000u;
        const bool x_is_subvoxel = can_x ? ((OCC(i, j, kp + 1) & 1) == 0) : true;
        neighbors[voxel_index] = x_is_subvoxel ? lsi[0][0] : lvi[0][0] + 1;
        const bool y_is_subvoxel = can_y ? ((OCC(i, j + 1, kp) & top) == 0) : true;
        neighbors[Nv + voxel_index] = y_is_subvoxel ? lsi[0][1] : lvi[0][1];
        const bool z_is_subvoxel = can_z ? ((OCC(i + 1, j, kp) & top) == 0) : true;
        neighbors[2 * Nv + voxel_index] = z_is_subvoxel ? lsi[1][0] : lvi[1][0];
        const bool xy_is_subvoxel = (can_x && can_y) ? ((OCC(i, j + 1, kp + 1) & 1) == 0) : true;
        neighbors[3 * Nv + voxel_index] = xy_is_subvoxel ? (y_is_subvoxel ? lsi[0][1] + 1 : lsi[0][1])
                                                         : (y_is_subvoxel ? lvi[0][1] : lvi[0][1] + 1);
        const bool yz_is_subvoxel = (can_y && can_z) ? ((OCC(i + 1, j + 1, kp) & top) == 0) : true;
        neighbors[4 * Nv + voxel_index] = yz_is_subvoxel ? lsi[1][1] : lvi[1][1];
        const bool xz_is_subvoxel = (can_x && can_z) ? ((OCC(i + 1, j, kp + 1) & 1) == 0) : true;
        neighbors[5 * Nv + voxel_index] = xz_is_subvoxel ? (z_is_subvoxel ? lsi[1][0] + 1 : lsi[1][0])
                                                         : (z_is_subvoxel ? lvi[1][0] : lvi[1][0] + 1);
        const bool xyz_is_subvoxel = (can_x && can_y && can_z) ? ((OCC(i + 1, j + 1, kp + 1) & 1) == 0) : true;
        neighbors[6 * Nv + voxel_index] = xyz_is_subvoxel ? (yz_is_subvoxel ? lsi[1][1] + 1 : lsi[1][1])
                                                          : (yz_is_subvoxel ? lvi[1][1] : lvi[1][1] + 1);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// triangle_extraction/dilate_occupancy.slang:9-94
// ---------------------------------------------------------------------------
void or_dilate_occupancy(const int32_t* occ, int I, int J, int KP, int d, int32_t* out) {
  auto OCC = [&](int i, int j, int kp) { return occ[((int64_t)i * J + j) * KP + kp]; };
  auto lrs = [](int32_t x, int s) { return (int32_t)((uint32_t)x >> s); };
#pragma omp parallel for schedule(static)
  for (int i = 0; i < I; ++i) {
    for (int j = 0; j < J; ++j) {
      for (int kp = 0; kp < KP; ++kp) {
        int32_t result = 0;
        if (kp > 0) {
          int32_t at_previous = 0;
          for (int di = -d; di <= d; ++di)
            for (int dj = -d; dj <= d; ++dj) {
              const int ii = i + di, jj = j + dj;
              if (ii < 0 || ii >= I || jj < 0 || jj >= J) continue;
              at_previous |= OCC(ii, jj, kp - 1);
            }
          at_previous = lrs(at_previous, 32 - d);
          for (int bit = 0; bit < d; ++bit) {
            result |= at_previous;
            at_previous = lrs(at_previous, 1);
          }
        }
        int32_t at_current = 0;
        for (int di = -d; di <= d; ++di)
          for (int dj = -d; dj <= d; ++dj) {
            const int ii = i + di, jj = j + dj;
            if (ii < 0 || ii >= I || jj < 0 || jj >= J) continue;
            at_current |= OCC(ii, jj, kp);
          }
        result |= at_current;
        int32_t left = at_current, right = at_current;
        for (int bit = 0; bit < d; ++bit) {
          right = lrs(right, 1);
          left = (int32_t)((uint32_t)left << 1);
          result |= left;
          result |= right;
        }
        if (kp < KP - 1) {
          int32_t at_next = 0;
          for (int di = -d; di <= d; ++di)
            for (int dj = -d; dj <= d; ++dj) {
              const int ii = i + di, jj = j + dj;
              if (ii < 0 || ii >= I || jj < 0 || jj >= J) continue;
              at_next |= OCC(ii, jj, kp + 1);
            }
          at_next = (int32_t)((uint32_t)at_next << (32 - d));
          for (int bit = 0; bit < d; ++bit) {
            result |= at_next;
            at_next = (int32_t)((uint32_t)at_next << 1);
          }
        }
        out[((int64_t)i * J + j) * KP + kp] = result;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// triangle_extraction/count_triangle_vertices.slang:3-37
// ---------------------------------------------------------------------------
void or_count_triangle_vertices(const float* sdf, const int32_t* lower, int64_t G, const float* level_sets, int S,
                                int32_t* counts) {
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    const float d0 = sdf[lower[g]];
    const float dx = lower[G + g] >= 0 ? sdf[lower[G + g]] : d0;
    const float dy = lower[2 * G + g] >= 0 ? sdf[lower[2 * G + g]] : d0;
    const float dz = lower[3 * G + g] >= 0 ? sdf[lower[3 * G + g]] : d0;
    for (int s = 0; s < S; ++s) {
      const float iso = level_sets[s];
      int n = 0;
      if ((d0 < iso) != (dx < iso)) n += 1;
      if ((d0 < iso) != (dy < iso)) n += 1;
      if ((d0 < iso) != (dz < iso)) n += 1;
      counts[(int64_t)s * G + g] = n;
    }
  }
  counts[(int64_t)S * G] = 0;  // count_triangle_vertices.py:36
}

// ---------------------------------------------------------------------------
// triangle_extraction/create_triangle_vertices.slang:15-199 (forward)
// ---------------------------------------------------------------------------
namespace {
struct OracleVoxel {
  float d0;
  float v0[3];
  float d1[3];
  float v1[3][3];
  int32_t i0, i1[3];
};

// create_triangle_vertices.slang:15-53 (load_voxel), SH loaded on demand.
inline OracleVoxel oracle_load_voxel(const float* gv, const float* gsdf, const int32_t* lower, int64_t G, int64_t g) {
  OracleVoxel vx;
  vx.i0 = lower[g];
  vx.d0 = gsdf[vx.i0];
  for (int c = 0; c < 3; ++c) vx.v0[c] = gv[3 * (int64_t)vx.i0 + c];
  for (int a = 0; a < 3; ++a) {
    const int32_t i1 = lower[(a + 1) * G + g];
    vx.i1[a] = i1;
    if (i1 >= 0) {
      vx.d1[a] = gsdf[i1];
      for (int c = 0; c < 3; ++c) vx.v1[a][c] = gv[3 * (int64_t)i1 + c];
    } else {
      vx.d1[a] = vx.d0;
      for (int c = 0; c < 3; ++c) vx.v1[a][c] = 0.0f;
    }
  }
  return vx;
}

// :55-69
inline bool should_compute_triangle_vertex(const OracleVoxel& vx, int axis, float level_set) {
  if (vx.d0 < level_set && vx.d1[axis] < level_set) return false;
  if (vx.d0 >= level_set && vx.d1[axis] >= level_set) return false;
  return true;
}

// :80-96 (t is detached)
inline float mc_weight(float d0, float d1, float level_set) {
  if (d0 == d1) return 0.5f;
  const float t = (level_set - d0) / (d1 - d0);
  return std::min(std::max(t, 0.0f), 1.0f);
}
}  // namespace

void or_create_triangle_vertices(const float* gv, const float* gsdf, const float* gsh, int C, const int32_t* lower,
                                 int64_t G, const float* level_sets, int S, const int32_t* voff, int64_t V,
                                 float* out_v, float* out_sdf, float* out_sh, uint8_t* out_type) {
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    const OracleVoxel vx = oracle_load_voxel(gv, gsdf, lower, G, g);
    for (int s = 0; s < S; ++s) {
      int64_t vi = voff[(int64_t)s * G + g];
      const float ls = level_sets[s];
      for (int a = 0; a < 3; ++a) {
        if (!should_compute_triangle_vertex(vx, a, ls)) continue;
        const float t = mc_weight(vx.d0, vx.d1[a], ls);
        for (int c = 0; c < 3; ++c) out_v[3 * vi + c] = std::fmaf(t, vx.v1[a][c] - vx.v0[c], vx.v0[c]);
        for (int k = 0; k < C; ++k)
          for (int ch = 0; ch < 3; ++ch) {
            const float s0 = gsh[((int64_t)k * G + vx.i0) * 3 + ch];
            const float s1 = gsh[((int64_t)k * G + vx.i1[a]) * 3 + ch];
            out_sh[((int64_t)k * V + vi) * 3 + ch] = std::fmaf(t, s1 - s0, s0);
          }
        out_sdf[vi] = std::fmaf(t, vx.d1[a] - vx.d0, vx.d0);
        out_type[vi] = (uint8_t)a;
        vi++;
      }
    }
  }
}

// create_triangle_vertices.slang:201-291 (backward). d(v0 + t(v1 - v0)) with
// t detached: origin receives (1 - t) * grad, the axis corner t * grad; the
// per-voxel differential is summed over level sets and axes, then scattered
// (atomics in the reference, common.slang:76-88).
void or_create_triangle_vertices_backward(const float* gsdf, int C, const int32_t* lower, int64_t G,
                                          const float* level_sets, int S, const int32_t* voff, const float* dv,
                                          const float* dsdf, const float* dsh, int64_t V, float* gdv, float* gdsdf,
                                          float* gdsh) {
  (void)V;
#pragma omp parallel
  {
    std::vector<float> o_sh((size_t)C * 3), a_sh((size_t)3 * C * 3);
#pragma omp for schedule(static)
    for (int64_t g = 0; g < G; ++g) {
      OracleVoxel vx;
      vx.i0 = lower[g];
      vx.d0 = gsdf[vx.i0];
      for (int a = 0; a < 3; ++a) {
        vx.i1[a] = lower[(a + 1) * G + g];
        vx.d1[a] = vx.i1[a] >= 0 ? gsdf[vx.i1[a]] : vx.d0;
      }
      float o_d = 0.f, o_v[3] = {0.f, 0.f, 0.f};
      float a_d[3] = {0.f, 0.f, 0.f}, a_v[3][3] = {{0.f}};
      std::fill(o_sh.begin(), o_sh.end(), 0.f);
      std::fill(a_sh.begin(), a_sh.end(), 0.f);
      for (int s = 0; s < S; ++s) {
        int64_t vi = voff[(int64_t)s * G + g];
        const float ls = level_sets[s];
        for (int a = 0; a < 3; ++a) {
          if (!should_compute_triangle_vertex(vx, a, ls)) continue;
          const float t = mc_weight(vx.d0, vx.d1[a], ls);
          const float gd = dsdf ? dsdf[vi] : 0.f;
          o_d += gd - t * gd;
          a_d[a] += t * gd;
          if (dv)
            for (int c = 0; c < 3; ++c) {
              const float gx = dv[3 * vi + c];
              o_v[c] += gx - t * gx;
              a_v[a][c] += t * gx;
            }
          if (dsh)
            for (int k = 0; k < C; ++k)
              for (int ch = 0; ch < 3; ++ch) {
                const float gq = dsh[((int64_t)k * V + vi) * 3 + ch];
                o_sh[k * 3 + ch] += gq - t * gq;
                a_sh[(a * C + k) * 3 + ch] += t * gq;
              }
          vi++;
        }
      }
      // bwd_diff(load_voxel): origin always, axes when valid.
#pragma omp atomic
      gdsdf[vx.i0] += o_d;
      if (gdv)
        for (int c = 0; c < 3; ++c) {
#pragma omp atomic
          gdv[3 * (int64_t)vx.i0 + c] += o_v[c];
        }
      for (int k = 0; k < C * 3; ++k) {
#pragma omp atomic
        gdsh[((int64_t)(k / 3) * G + vx.i0) * 3 + k % 3] += o_sh[k];
      }
      for (int a = 0; a < 3; ++a) {
        const int32_t i1 = vx.i1[a];
        if (i1 < 0) continue;
#pragma omp atomic
        gdsdf[i1] += a_d[a];
        if (gdv)
          for (int c = 0; c < 3; ++c) {
#pragma omp atomic
            gdv[3 * (int64_t)i1 + c] += a_v[a][c];
          }
        for (int k = 0; k < C * 3; ++k) {
#pragma omp atomic
          gdsh[((int64_t)(k / 3) * G + i1) * 3 + k % 3] += a_sh[(a * C + k / 3) * 3 + k % 3];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// triangle_extraction/count_triangle_faces.slang:3-50
// ---------------------------------------------------------------------------
void or_count_triangle_faces(const float* sdf, const int32_t* lower, int64_t G, const int32_t* upper, int64_t Nv,
                             const float* level_sets, int S, int32_t* counts, uint8_t* codes) {
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < Nv; ++v) {
    const float cube[8] = {
        sdf[lower[v]],          sdf[lower[G + v]],     sdf[upper[3 * Nv + v]], sdf[lower[2 * G + v]],
        sdf[lower[3 * G + v]],  sdf[upper[2 * Nv + v]], sdf[upper[v]],          sdf[upper[Nv + v]],
    };
    for (int s = 0; s < S; ++s) {
      const float iso = level_sets[s];
      int code = 0;
      for (int q = 0; q < 8; ++q)
        if (cube[q] >= iso) code |= 1 << q;
      codes[(int64_t)s * Nv + v] = (uint8_t)code;
      counts[(int64_t)s * Nv + v] = kMc.first[code + 1] - kMc.first[code];
    }
  }
  counts[(int64_t)S * Nv] = 0;  // count_triangle_faces.py:48
}

// ---------------------------------------------------------------------------
// triangle_extraction/create_triangle_faces.slang:5-78
// ---------------------------------------------------------------------------
void or_create_triangle_faces(const int32_t* neighbors, const int32_t* indices, int64_t Nv, int64_t G,
                              const int32_t* voff, const uint8_t* types, const uint8_t* codes, int S,
                              const int32_t* foff, int32_t* faces, int32_t* voxel_indices) {
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < Nv; ++v) {
    for (int s = 0; s < S; ++s) {
      const int64_t face_offset = (int64_t)s * Nv + v;
      const int32_t triangle_write_ctr = foff[face_offset];
      const int code = codes[(int64_t)s * Nv + v];
      const int num_i = kMc.first[code + 1] - kMc.first[code];
      const int first_in = kMc.first[code];
      for (int j = 0; j < num_i; ++j) {
        const int eid = kMc.ids[first_in + j];
        const int neighbor_index = kMc.owner[eid];
        const int edge_nr = kMc.axis[eid];
        const int64_t nb = (neighbor_index == -1) ? v : neighbors[(int64_t)neighbor_index * Nv + v];
        const int64_t vo = (int64_t)s * G + nb;
        const int32_t start = voff[vo];
        const int32_t n = voff[vo + 1] - start;
        int32_t target = -1;
        for (int q = 0; q < n; ++q)
          if (types[start + q] == edge_nr) {
            target = start + q;
            break;
          }
        const int32_t tri = (triangle_write_ctr + j) / 3;
        const int corner = 2 - (triangle_write_ctr + j) % 3;
        faces[3 * (int64_t)tri + corner] = target;
        if (corner == 0) voxel_indices[tri] = indices[v];
      }
    }
  }
}

}  // extern "C"
