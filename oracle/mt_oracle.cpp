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
// floating-point kernels follow the reference source's operations in their
// order, each rounded once (IEEE-754 single precision), and the file is
// compiled with -ffp-contract=off so the host compiler fuses nothing.
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
// triangle_extraction/compute_sdf_regularizers.slang:18-128 (forward) and its
// automatic derivative (backward, derived here by hand).
// ---------------------------------------------------------------------------
namespace {
struct RegCorners {
  int32_t id[8];  // 000 001 010 100 111 110 101 011
  float d[8];
};

inline RegCorners reg_corners(const float* sdf, const int32_t* lower, int64_t G, const int32_t* upper, int64_t Nv,
                              int64_t v) {
  RegCorners c;
  const int32_t ids[8] = {lower[v], lower[G + v], lower[2 * G + v], lower[3 * G + v],
                          upper[v], upper[Nv + v], upper[2 * Nv + v], upper[3 * Nv + v]};
  for (int q = 0; q < 8; ++q) {
    c.id[q] = ids[q];
    c.d[q] = sdf[ids[q]];
  }
  return c;
}

inline void reg_gradient(const RegCorners& c, float& dx, float& dy, float& dz) {
  const float d000 = c.d[0], d001 = c.d[1], d010 = c.d[2], d100 = c.d[3], d111 = c.d[4], d110 = c.d[5],
              d101 = c.d[6], d011 = c.d[7];
  const float t = 0.5f, t1 = 1.0f - t;
  dx = t1 * t1 * (d001 - d000) + t * t1 * (d011 - d010) + t1 * t * (d101 - d100) + t * t * (d111 - d110);
  dy = t1 * t1 * (d010 - d000) + t * t1 * (d011 - d001) + t1 * t * (d110 - d100) + t * t * (d111 - d101);
  dz = t1 * t1 * (d100 - d000) + t * t1 * (d101 - d001) + t1 * t * (d110 - d010) + t * t * (d111 - d011);
}

inline float reg_norm(float a, float b, float c) {
  const float scale = std::fmax(std::fmax(std::fabs(a), std::fabs(b)), std::fabs(c));
  if (scale < 1e-10f) return 0.0f;
  const float inv = 1.0f / scale;
  const float sa = inv * a, sb = inv * b, sc = inv * c;
  return scale * std::sqrt(sa * sa + sb * sb + sc * sc);
}

inline float reg_curvature(const float* sdf, const RegCorners& c, const int32_t* lower, int64_t G, int32_t sub,
                           int32_t* extra, int& counted) {
  float sum = c.d[5] + c.d[6] + c.d[7];
  counted = 3;
  for (int i = 1; i < 4; ++i) {
    extra[i - 1] = lower[(int64_t)i * G + sub];
    if (extra[i - 1] >= 0) {
      sum += sdf[extra[i - 1]];
      ++counted;
    }
  }
  return sum - (float)counted * c.d[4];
}
}  // namespace

void or_compute_sdf_regularizers(const float* sdf, const int32_t* neighbors, const int32_t* lower, int64_t G,
                                 const int32_t* upper, int64_t Nv, int vx, int vy, int vz, float* pos, float* neg,
                                 float* curv) {
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < Nv; ++v) {
    const RegCorners c = reg_corners(sdf, lower, G, upper, Nv, v);
    float dx, dy, dz;
    reg_gradient(c, dx, dy, dz);
    const float delta = reg_norm((float)vx * dx, (float)vy * dy, (float)vz * dz) - 1.0f;
    float p = 0.f, n = 0.f;
    if (delta < 0) n += delta * delta;
    if (delta > 0) p += delta * delta;
    pos[v] = p / 1.0f;
    neg[v] = n / 1.0f;
    int32_t extra[3];
    int counted;
    const float cs = reg_curvature(sdf, c, lower, G, neighbors[6 * Nv + v], extra, counted);
    curv[v] = cs * cs;
  }
}

// d delta / d a = a / n (n = |(a, b, c)| > 0), gradients scattered to the
// corners each term reads; grad_sdf is accumulated (+=).
void or_compute_sdf_regularizers_backward(const float* sdf, const int32_t* neighbors, const int32_t* lower, int64_t G,
                                          const int32_t* upper, int64_t Nv, int vx, int vy, int vz,
                                          const float* g_pos, const float* g_neg, const float* g_curv,
                                          float* grad_sdf) {
  for (int64_t v = 0; v < Nv; ++v) {
    const RegCorners c = reg_corners(sdf, lower, G, upper, Nv, v);
    float dx, dy, dz;
    reg_gradient(c, dx, dy, dz);
    const float a = (float)vx * dx, b = (float)vy * dy, cc = (float)vz * dz;
    const float n = reg_norm(a, b, cc);
    const float delta = n - 1.0f;
    float g_delta = 0.f;
    if (g_pos && delta > 0) g_delta += 2.0f * delta * g_pos[v];
    if (g_neg && delta < 0) g_delta += 2.0f * delta * g_neg[v];
    if (g_delta != 0.f && n > 0.f) {
      const float gx = g_delta * a / n * (float)vx, gy = g_delta * b / n * (float)vy, gz = g_delta * cc / n * (float)vz;
      const float w = 0.25f;
      // sign of each corner in dx, dy, dz (000 001 010 100 111 110 101 011)
      const int sx[8] = {-1, 1, -1, -1, 1, -1, 1, 1}, sy[8] = {-1, -1, 1, -1, 1, 1, -1, 1},
                sz[8] = {-1, -1, -1, 1, 1, 1, 1, -1};
      for (int q = 0; q < 8; ++q) grad_sdf[c.id[q]] += w * (sx[q] * gx + sy[q] * gy + sz[q] * gz);
    }
    int32_t extra[3];
    int counted;
    const float cs = reg_curvature(sdf, c, lower, G, neighbors[6 * Nv + v], extra, counted);
    const float g_cs = g_curv ? 2.0f * cs * g_curv[v] : 0.f;
    if (g_cs != 0.f) {
      grad_sdf[c.id[5]] += g_cs;
      grad_sdf[c.id[6]] += g_cs;
      grad_sdf[c.id[7]] += g_cs;
      grad_sdf[c.id[4]] -= (float)counted * g_cs;
      for (int i = 0; i < 3; ++i)
        if (extra[i] >= 0) grad_sdf[extra[i]] += g_cs;
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
// Coarse-to-fine subdivision and the occupancy mesh.
// ---------------------------------------------------------------------------

// write_occupancy.slang:1-20 (one atomic OR per index; indices outside the
// grid are skipped).
void or_write_occupancy(const int32_t* voxel_indices, int64_t n, int32_t* occ, int64_t words) {
  for (int64_t t = 0; t < n; ++t) {
    const int32_t v = voxel_indices[t];
    if (v < 0 || (int64_t)(v >> 5) >= words) continue;
    occ[v >> 5] = (int32_t)((uint32_t)occ[v >> 5] | (1u << (v % 32)));
  }
}

// upscale_occupancy.slang:1-74: per new voxel, the 8 corners sampled with
// unsigned 32-bit arithmetic (sample_corner, :1-24); `mask` (nullable) is
// AND-ed into every old word (upscale_parameters.py:49).
void or_upscale_occupancy(const int32_t* occ, const int32_t* mask, int I, int J, int KP, int I2, int J2, int KP2,
                          int32_t* out) {
  const uint32_t i_max_sampled = (uint32_t)I, j_max_sampled = (uint32_t)J, k_max_sampled = (uint32_t)KP << 5;
  const uint32_t i_max = (uint32_t)I2, j_max = (uint32_t)J2, k_max = (uint32_t)KP2 << 5;
  auto word = [&](uint32_t i, uint32_t j, uint32_t kp) {
    const int64_t w = ((int64_t)i * J + j) * KP + kp;
    uint32_t x = (uint32_t)occ[w];
    if (mask) x &= (uint32_t)mask[w];
    return x;
  };
#pragma omp parallel for schedule(static)
  for (int i = 0; i < I2; ++i)
    for (int j = 0; j < J2; ++j)
      for (int kp = 0; kp < KP2; ++kp) {
        int32_t result = 0;
        for (int bit = 0; bit < 32; ++bit) {
          const uint32_t k = ((uint32_t)kp << 5) + (uint32_t)bit;
          bool value = false;
          for (uint32_t di = 0; di < 2; ++di)
            for (uint32_t dj = 0; dj < 2; ++dj)
              for (uint32_t dk = 0; dk < 2; ++dk) {
                const uint32_t is = (((uint32_t)i + di) * i_max_sampled - di) / i_max;
                const uint32_t js = (((uint32_t)j + dj) * j_max_sampled - dj) / j_max;
                const uint32_t ks = ((k + dk) * k_max_sampled - dk) / k_max;
                value |= ((word(is, js, ks >> 5) >> (ks % 32)) & 1u) != 0;
              }
          result |= (int32_t)((uint32_t)value << bit);
        }
        out[((int64_t)i * J2 + j) * KP2 + kp] = result;
      }
}

// upscale_parameters.slang:1-198: every new vertex (in vertex-occupancy
// order) samples the old vertices trilinearly (sample_trilinear, :55-127),
// skipping absent corners and renormalising by the summed weight.
void or_upscale_parameters(const int32_t* ovocc, const int32_t* ovoff, const float* osdf, const float* osh, int C,
                           int64_t Vold, int I1, int J1, int KP1, const int32_t* nvocc, const int32_t* nvoff, int I1n,
                           int J1n, int KP1n, int64_t Vnew, float* nsdf, float* nsh) {
  const int i_max = I1n - 1, j_max = J1n - 1, k_packed_max = KP1n - 1;
  const float inv_i_max = 1 / (float)i_max;
  const float inv_j_max = 1 / (float)j_max;
  const float inv_k_max = 1 / (float)(32 * k_packed_max);
  // read_vertex (:9-53): the old vertex index, or -1.
  auto read_vertex = [&](int i, int j, int k) -> int64_t {
    if (i < 0 || j < 0 || k < 0) return -1;
    const int k_packed = k / 32;
    if (i >= I1 || j >= J1 || k_packed >= KP1) return -1;
    const int bit = k % 32;
    const int64_t w = ((int64_t)i * J1 + j) * KP1 + k_packed;
    uint32_t chunk = (uint32_t)ovocc[w];
    if ((chunk & (1u << bit)) == 0) return -1;
    int64_t index = ovoff[w];
    for (int d = 0; d < bit; ++d) {
      if (chunk & 1u) ++index;
      chunk >>= 1;
    }
    return index < Vold ? index : -1;
  };
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i <= i_max; ++i) {
    std::vector<float> sh((size_t)C * 3);
    for (int j = 0; j <= j_max; ++j)
      for (int kp = 0; kp <= k_packed_max; ++kp) {
        const int64_t w = ((int64_t)i * J1n + j) * KP1n + kp;
        int64_t vertex_index = nvoff[w];
        uint32_t chunk = (uint32_t)nvocc[w];
        int k = 32 * kp;
        for (int bit = 0; bit < 32; ++bit, chunk >>= 1, ++k) {
          if ((chunk & 1u) == 0) continue;
          const float x = (float)k * inv_k_max, y = (float)j * inv_j_max, z = (float)i * inv_i_max;
          const float xu = x * (float)((KP1 - 1) * 32), yu = y * (float)(J1 - 1), zu = z * (float)(I1 - 1);
          const int oi = (int)zu, oj = (int)yu, ok = (int)xu;
          const float ti = std::fmod(zu, 1.0f), tj = std::fmod(yu, 1.0f), tk = std::fmod(xu, 1.0f);
          std::fill(sh.begin(), sh.end(), 0.0f);
          float sd = 0.0f, denominator = 0.0f;
          for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj)
              for (int dk = 0; dk < 2; ++dk) {
                const int64_t v = read_vertex(oi + di, oj + dj, ok + dk);
                if (v < 0) continue;
                const float weight = (di == 0 ? 1 - ti : ti) * (dj == 0 ? 1 - tj : tj) * (dk == 0 ? 1 - tk : tk);
                for (int s = 0; s < C; ++s)
                  for (int c = 0; c < 3; ++c) sh[s * 3 + c] += weight * osh[((int64_t)s * Vold + v) * 3 + c];
                sd += weight * osdf[v];
                denominator += weight;
              }
          const float multiplier = 1 / denominator;
          if (vertex_index >= 0 && vertex_index < Vnew) {
            for (int s = 0; s < C; ++s)
              for (int c = 0; c < 3; ++c) nsh[((int64_t)s * Vnew + vertex_index) * 3 + c] = sh[s * 3 + c] * multiplier;
            nsdf[vertex_index] = sd * multiplier;
          }
          ++vertex_index;
        }
      }
  }
}

// get_occupancy_mesh.slang:1-54 count_triangles, over (I+1)(J+1)(KP+1)
// entries; counts has one more entry, set to 0.
void or_count_occupancy_mesh_triangles(const int32_t* occ, int I, int J, int KP, int32_t* counts) {
  auto OCC = [&](int i, int j, int kp) { return (uint32_t)occ[((int64_t)i * J + j) * KP + kp]; };
  const int64_t total = (int64_t)(I + 1) * (J + 1) * (KP + 1);
#pragma omp parallel for schedule(static)
  for (int i = 0; i <= I; ++i)
    for (int j = 0; j <= J; ++j)
      for (int kp = 0; kp <= KP; ++kp) {
        const bool il = i == I, jl = j == J, kl = kp == KP;
        uint32_t here = (il || jl || kl) ? 0u : OCC(i, j, kp);
        uint32_t minus_i = (jl || kl || i == 0) ? 0u : OCC(i - 1, j, kp);
        uint32_t minus_j = (il || kl || j == 0) ? 0u : OCC(i, j - 1, kp);
        bool minus_k = (il || jl || kp == 0) ? false : (OCC(i, j, kp - 1) & 0x80000000u) != 0;
        int faces = 0;
        for (int bit = 0; bit < 32; ++bit) {
          const bool h = here & 1u, mi = minus_i & 1u, mj = minus_j & 1u;
          faces += (int)(h != mi) + (int)(h != mj) + (int)(h != minus_k);
          minus_k = h;
          here >>= 1;
          minus_i >>= 1;
          minus_j >>= 1;
        }
        counts[((int64_t)i * (J + 1) + j) * (KP + 1) + kp] = 2 * faces;
      }
  counts[total] = 0;
}

// get_occupancy_mesh.slang:56-220 create_face / create_triangles.
void or_create_occupancy_mesh_triangles(const int32_t* occ, int I, int J, int KP, const int32_t* offsets,
                                        const float* colors, float* verts, float* tri_colors) {
  auto OCC = [&](int i, int j, int kp) { return (uint32_t)occ[((int64_t)i * J + j) * KP + kp]; };
  const int ijk_max[3] = {I, J, KP * 32};
  auto create_face = [&](int64_t index, const int ijk[3], int axis, bool upper_bit) {
    const int axis0 = (axis + 1) % 3, axis1 = (axis + 2) % 3;
    float v00[3], v01[3], v10[3], v11[3];
    const float plane = (float)ijk[axis] / (float)ijk_max[axis];
    v00[axis] = v01[axis] = v10[axis] = v11[axis] = plane;
    const float v0x = (float)ijk[axis0] / (float)ijk_max[axis0];
    const float v1x = (float)(ijk[axis0] + 1) / (float)ijk_max[axis0];
    const float vx0 = (float)ijk[axis1] / (float)ijk_max[axis1];
    const float vx1 = (float)(ijk[axis1] + 1) / (float)ijk_max[axis1];
    v00[axis0] = v0x, v00[axis1] = vx0;
    v01[axis0] = v0x, v01[axis1] = vx1;
    v10[axis0] = v1x, v10[axis1] = vx0;
    v11[axis0] = v1x, v11[axis1] = vx1;
    const int side = upper_bit ? 1 : 0;
    const float* face_color = colors + (axis * 2 + side) * 3;
    const float* triangles[2][3] = {{v00, upper_bit ? v01 : v10, upper_bit ? v10 : v01},
                                    {v11, upper_bit ? v10 : v01, upper_bit ? v01 : v10}};
    for (int t = 0; t < 2; ++t) {
      for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) verts[((index + t) * 3 + c) * 3 + a] = triangles[t][c][2 - a];
      for (int a = 0; a < 3; ++a) tri_colors[(index + t) * 3 + a] = face_color[a];
    }
  };
#pragma omp parallel for schedule(static)
  for (int i = 0; i <= I; ++i)
    for (int j = 0; j <= J; ++j)
      for (int kp = 0; kp <= KP; ++kp) {
        const bool il = i == I, jl = j == J, kl = kp == KP;
        uint32_t here = (il || jl || kl) ? 0u : OCC(i, j, kp);
        uint32_t minus_i = (jl || kl || i == 0) ? 0u : OCC(i - 1, j, kp);
        uint32_t minus_j = (il || kl || j == 0) ? 0u : OCC(i, j - 1, kp);
        bool minus_k = (il || jl || kp == 0) ? false : (OCC(i, j, kp - 1) & 0x80000000u) != 0;
        int64_t index = offsets[((int64_t)i * (J + 1) + j) * (KP + 1) + kp];
        int k = kp * 32;
        for (int bit = 0; bit < 32; ++bit, ++k) {
          const bool h = here & 1u, mi = minus_i & 1u, mj = minus_j & 1u;
          const int ijk[3] = {i, j, k};
          if (h != mi) create_face(index, ijk, 0, h), index += 2;
          if (h != mj) create_face(index, ijk, 1, h), index += 2;
          if (h != minus_k) create_face(index, ijk, 2, h), index += 2;
          minus_k = h;
          here >>= 1;
          minus_i >>= 1;
          minus_j >>= 1;
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
        for (int c = 0; c < 3; ++c) out_v[3 * vi + c] = vx.v0[c] + t * (vx.v1[a][c] - vx.v0[c]);
        for (int k = 0; k < C; ++k)
          for (int ch = 0; ch < 3; ++ch) {
            const float s0 = gsh[((int64_t)k * G + vx.i0) * 3 + ch];
            const float s1 = gsh[((int64_t)k * G + vx.i1[a]) * 3 + ch];
            out_sh[((int64_t)k * V + vi) * 3 + ch] = s0 + t * (s1 - s0);
          }
        out_sdf[vi] = vx.d0 + t * (vx.d1[a] - vx.d0);
        out_type[vi] = (uint8_t)a;
        vi++;
      }
    }
  }
}

// Where each triangle vertex comes from: origin corner, axis corner and the
// (detached) weight t of create_triangle_vertices.slang:80-96. Used by the
// finite-difference checks, which hold t fixed as the reference's adjoint does.
void or_triangle_vertex_sources(const float* gsdf, const int32_t* lower, int64_t G, const float* level_sets, int S,
                                const int32_t* voff, int32_t* out_i0, int32_t* out_i1, float* out_t) {
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    OracleVoxel vx;
    vx.i0 = lower[g];
    vx.d0 = gsdf[vx.i0];
    for (int a = 0; a < 3; ++a) {
      vx.i1[a] = lower[(a + 1) * G + g];
      vx.d1[a] = vx.i1[a] >= 0 ? gsdf[vx.i1[a]] : vx.d0;
    }
    for (int s = 0; s < S; ++s) {
      int64_t vi = voff[(int64_t)s * G + g];
      for (int a = 0; a < 3; ++a) {
        if (!should_compute_triangle_vertex(vx, a, level_sets[s])) continue;
        out_i0[vi] = vx.i0;
        out_i1[vi] = vx.i1[a];
        out_t[vi] = mc_weight(vx.d0, vx.d1[a], level_sets[s]);
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


// ===========================================================================
// Rasterization (triangle_rasterization/*.slang, sort_keys.cu)
// ===========================================================================
}  // extern "C"

namespace {

// `int(x)` on the GPU: truncation toward zero, saturating, NaN -> 0.
inline int f2i_rz(float x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x < -2147483648.0f) return (int)0x80000000u;
  return (int)x;
}

inline float dot2(float ax, float ay, float bx, float by) { return ax * bx + ay * by; }

// intersect_and_composite.slang:65-106 / intersect.slang:14-49, evaluated in
// full for every (pixel, triangle) pair as the reference does.
inline void barycentric(float p1x, float p1y, float p2x, float p2y, float p3x, float p3y, float px, float py,
                        float& u, float& v, float& w) {
  const float e12x = p2x - p1x, e12y = p2y - p1y;
  const float e23x = p3x - p2x, e23y = p3y - p2y;
  const float e13x = p3x - p1x, e13y = p3y - p1y;
  const float d_12_12 = dot2(e12x, e12y, e12x, e12y);
  const float d_12_23 = dot2(e12x, e12y, e23x, e23y);
  const float d_12_13 = dot2(e12x, e12y, e13x, e13y);
  const float d_13_13 = dot2(e13x, e13y, e13x, e13y);
  const float d_13_23 = dot2(e13x, e13y, e23x, e23y);
  const float d_23_23 = dot2(e23x, e23y, e23x, e23y);
  const float d_1x_12 = dot2(px - p1x, py - p1y, e12x, e12y);
  const float d_1x_13 = dot2(px - p1x, py - p1y, e13x, e13y);
  const float d_2x_12 = dot2(px - p2x, py - p2y, e12x, e12y);
  const float d_2x_13 = dot2(px - p2x, py - p2y, e13x, e13y);
  float denom = std::nanf("");  // the reference leaves it unset; only reachable with NaNs
  if (std::fabs(d_12_13) <= std::fabs(d_12_23) && std::fabs(d_12_13) <= std::fabs(d_13_23)) {
    denom = d_12_12 * d_13_13 - d_12_13 * d_12_13;
  } else if (std::fabs(d_12_23) <= std::fabs(d_12_13) && std::fabs(d_12_23) <= std::fabs(d_13_23)) {
    denom = d_12_12 * d_23_23 - d_12_23 * d_12_23;
  } else if (std::fabs(d_13_23) <= std::fabs(d_12_13) && std::fabs(d_13_23) <= std::fabs(d_12_23)) {
    denom = d_13_13 * d_23_23 - d_13_23 * d_13_23;
  }
  v = d_13_13 * d_1x_12 - d_12_13 * d_1x_13;
  w = d_12_12 * d_1x_13 - d_12_13 * d_1x_12;
  u = d_12_23 * d_2x_13 - d_13_23 * d_2x_12;
  const float eps = 1e-8f;
  v /= denom + eps;
  w /= denom + eps;
  u /= denom + eps;
}

// intersect_and_composite.slang:131-136 / intersect.slang:61-64.
inline bool accepted(float u, float v, float w) {
  const float sum = (u + v) + w;
  if (std::isnan(u) || std::isnan(v) || std::isnan(w) || u < 0 || u > 1 || v < 0 || v > 1 || w < 0 || w > 1 ||
      sum < 0.999f || sum > 1.001f)
    return false;
  return true;
}

inline float interp3(float u, float v, float w, float a, float b, float c) { return u * a + v * b + w * c; }

inline float sdf_to_cdf(float sdf, float s, float& e) {
  e = std::exp(-sdf * s);
  return 1.0f / (1.0f + e);
}

inline float alpha_raw(float oc, float ic) { return ((oc - ic) + 1e-5f) / (oc + 1e-5f); }
inline float clamp01(float x) { return std::min(std::max(x, 0.0f), 1.0f); }

const float kSH_C0 = 0.28209479177387814f;
const float kSH_C1 = 0.4886025119029199f;
const float kSH_C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
                         0.5462742152960396f};
const float kSH_C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f, 0.3731763325901154f,
                         -0.4570457994644658f, 1.445305721320277f, -0.5900435899266435f};

// evaluate_spherical_harmonics.slang:124-160 as basis functions of dir.
inline void sh_basis(float x, float y, float z, int n, float* basis) {
  basis[0] = kSH_C0;
  if (n <= 1) return;
  basis[1] = -kSH_C1 * y;
  basis[2] = kSH_C1 * z;
  basis[3] = -kSH_C1 * x;
  if (n <= 4) return;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  basis[4] = kSH_C2[0] * xy;
  basis[5] = kSH_C2[1] * yz;
  basis[6] = kSH_C2[2] * (2.0f * zz - xx - yy);
  basis[7] = kSH_C2[3] * xz;
  basis[8] = kSH_C2[4] * (xx - yy);
  if (n <= 9) return;
  basis[9] = kSH_C3[0] * y * (3.0f * xx - yy);
  basis[10] = kSH_C3[1] * xy * z;
  basis[11] = kSH_C3[2] * y * (4.0f * zz - xx - yy);
  basis[12] = kSH_C3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
  basis[13] = kSH_C3[4] * x * (4.0f * zz - xx - yy);
  basis[14] = kSH_C3[5] * z * (xx - yy);
  basis[15] = kSH_C3[6] * x * (xx - 3.0f * yy);
}

inline void view_dir(const float* v, const float* cam, float& x, float& y, float& z) {
  const float dx = v[0] - cam[0], dy = v[1] - cam[1], dz = v[2] - cam[2];
  const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
  x = dx / len;
  y = dy / len;
  z = dz / len;
}

struct Layout {
  int cam_off, cam_len, shell_off, shell_len, tile_off, tile_len, depth_off;
};
inline uint64_t fmask(int len) { return (uint64_t)((1u << len) - 1u); }

}  // namespace

extern "C" {

// torch.inverse(extrinsics)[:, :3, 3] (evaluate_spherical_harmonics.py:38),
// Gauss-Jordan with partial pivoting in double precision.
void or_camera_positions(const float* ext, int B, float* out) {
  for (int b = 0; b < B; ++b) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? (double)ext[16 * b + 4 * r + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
      int piv = c;
      for (int r = c + 1; r < 4; ++r)
        if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
      for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
      const double d = a[c][c];
      for (int k = 0; k < 8; ++k) a[c][k] /= d;
      for (int r = 0; r < 4; ++r)
        if (r != c) {
          const double f = a[r][c];
          for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 3; ++r) out[3 * b + r] = (float)a[r][4 + 3];
  }
}

// project_vertices.slang:51-92.
void or_project_vertices(const float* verts, int64_t V, const float* ext, const float* intr, int B, float* out_xy,
                         float* out_depth) {
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; ++v) {
    const float x = verts[3 * v], y = verts[3 * v + 1], z = verts[3 * v + 2];
    for (int b = 0; b < B; ++b) {
      const float* E = ext + 16 * b;
      const float* K = intr + 9 * b;
      float cam[3];
      for (int r = 0; r < 3; ++r) cam[r] = E[4 * r] * x + E[4 * r + 1] * y + E[4 * r + 2] * z + E[4 * r + 3] * 1.0f;
      const float kx = K[0] * cam[0] + K[1] * cam[1] + K[2] * cam[2];
      const float ky = K[3] * cam[0] + K[4] * cam[1] + K[5] * cam[2];
      const int64_t o = (int64_t)b * V + v;
      out_xy[2 * o] = kx / cam[2];
      out_xy[2 * o + 1] = ky / cam[2];
      out_depth[o] = cam[2];
    }
  }
}

// evaluate_spherical_harmonics.slang:187-228 (forward).
void or_evaluate_sh(const float* verts, int64_t V, const float* sh, int sh_degree, const float* campos, int B,
                    float* out) {
  const int n = (sh_degree + 1) * (sh_degree + 1);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; ++v) {
    for (int b = 0; b < B; ++b) {
      float x, y, z, basis[16];
      view_dir(verts + 3 * v, campos + 3 * b, x, y, z);
      sh_basis(x, y, z, n, basis);
      for (int c = 0; c < 3; ++c) {
        float rgb = basis[0] * sh[((int64_t)0 * V + v) * 3 + c];
        for (int k = 1; k < n; ++k) rgb += basis[k] * sh[((int64_t)k * V + v) * 3 + c];
        out[((int64_t)b * V + v) * 3 + c] = std::max(rgb + 0.5f, 0.0f);
      }
    }
  }
}

// evaluate_spherical_harmonics.slang:230-270 (backward, to the SH only).
void or_evaluate_sh_backward(const float* verts, int64_t V, int sh_degree, const float* campos, int B,
                             const float* colors, const float* dcolors, float* dsh) {
  const int n = (sh_degree + 1) * (sh_degree + 1);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; ++v) {
    for (int b = 0; b < B; ++b) {
      float x, y, z, basis[16];
      view_dir(verts + 3 * v, campos + 3 * b, x, y, z);
      sh_basis(x, y, z, n, basis);
      for (int c = 0; c < 3; ++c) {
        const int64_t o = ((int64_t)b * V + v) * 3 + c;
        const float g = colors[o] > 0.0f ? dcolors[o] : 0.0f;
        for (int k = 0; k < n; ++k) dsh[((int64_t)k * V + v) * 3 + c] += basis[k] * g;
      }
    }
  }
}

// bound_triangles.slang:62-192.
void or_bound_triangles(const float* xy, const float* depth, int64_t V, const int32_t* faces, int64_t F, int B,
                        int tile_h, int tile_w, int rows, int cols, float near, int32_t* out_min, int32_t* out_max,
                        int32_t* out_count) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)B * F; ++i) {
    const int b = (int)(i / F);
    const int64_t f = i % F;
    const int64_t base = (int64_t)b * V;
    const int64_t ia = base + faces[3 * f], ib = base + faces[3 * f + 1], ic = base + faces[3 * f + 2];
    const float ax = xy[2 * ia], ay = xy[2 * ia + 1], bx = xy[2 * ib], by = xy[2 * ib + 1];
    const float cx = xy[2 * ic], cy = xy[2 * ic + 1];
    int r0 = 0, r1 = 0, c0 = 0, c1 = 0;
    const float check = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    const float min_depth = std::fmin(std::fmin(depth[ia], depth[ib]), depth[ic]);
    if (!(check < 0) && !(min_depth < near)) {
      const float ymin = std::fmin(std::fmin(ay, by), cy), ymax = std::fmax(std::fmax(ay, by), cy);
      const float xmin = std::fmin(std::fmin(ax, bx), cx), xmax = std::fmax(std::fmax(ax, bx), cx);
      r0 = std::clamp(f2i_rz(ymin) / tile_h, 0, rows);
      r1 = std::clamp(f2i_rz(std::ceil(ymax / (float)tile_h)), 0, rows);
      c0 = std::clamp(f2i_rz(xmin) / tile_w, 0, cols);
      c1 = std::clamp(f2i_rz(std::ceil(xmax / (float)tile_w)), 0, cols);
    }
    out_min[2 * i] = r0;
    out_min[2 * i + 1] = c0;
    out_max[2 * i] = r1;
    out_max[2 * i + 1] = c1;
    out_count[i] = (r1 - r0) * (c1 - c0);
  }
}

// generate_keys.slang:4-68 with keys.slang:6-22. offsets: inclusive int64.
void or_generate_keys(const float* depth, int64_t V, const int32_t* faces, int64_t F, const int32_t* sfb, int S,
                      const int32_t* tmin, const int32_t* tmax, const int64_t* offsets, int B, int grid_width,
                      const int32_t* layout, int64_t* out_keys, int32_t* out_tri) {
  const Layout L{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], layout[6]};
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < F; ++f) {
    uint32_t shell = 0;
    for (; shell < (uint32_t)S; ++shell)
      if (f < sfb[shell]) break;
    for (int b = 0; b < B; ++b) {
      const int64_t oi = (int64_t)b * F + f;
      int64_t key_index = oi == 0 ? 0 : offsets[oi - 1];
      const int r0 = tmin[2 * oi], c0 = tmin[2 * oi + 1], r1 = tmax[2 * oi], c1 = tmax[2 * oi + 1];
      const int64_t base = (int64_t)b * V;
      const float mean = ((depth[base + faces[3 * f]] + depth[base + faces[3 * f + 1]]) + depth[base + faces[3 * f + 2]]) / 3.f;
      uint32_t bits;
      std::memcpy(&bits, &mean, 4);
      for (int row = r0; row < r1; ++row)
        for (int col = c0; col < c1; ++col) {
          const uint32_t tile = (uint32_t)(row * grid_width + col);
          const uint64_t key = (((uint64_t)b & fmask(L.cam_len)) << L.cam_off) |
                               (((uint64_t)shell & fmask(L.shell_len)) << L.shell_off) |
                               (((uint64_t)tile & fmask(L.tile_len)) << L.tile_off) | ((uint64_t)bits << L.depth_off);
          out_keys[key_index] = (int64_t)key;
          out_tri[key_index] = (int32_t)f;
          key_index++;
        }
    }
  }
}

// cub::DeviceRadixSort::SortPairs on signed int64 keys, bits [0, 64)
// (sort_keys.cu:241-267): a stable sort by signed key.
void or_sort_pairs(const int64_t* keys, const int32_t* vals, int64_t n, int64_t* out_keys, int32_t* out_vals) {
  std::vector<int64_t> idx((size_t)n);
  for (int64_t i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
  for (int64_t i = 0; i < n; ++i) {
    out_keys[i] = keys[idx[i]];
    out_vals[i] = vals[idx[i]];
  }
}

// delineate_tiles.slang:14-58 (output zero-filled first, delineate_tiles.py:40).
void or_delineate_tiles(const int64_t* keys, int64_t K, const int32_t* layout, int separate_shells, int B, int Sd,
                        int64_t T, int64_t* out) {
  const Layout L{layout[0], layout[1], layout[2], layout[3], layout[4], layout[5], layout[6]};
  std::memset(out, 0, sizeof(int64_t) * 2 * (size_t)B * Sd * T);
  auto index_of = [&](uint64_t key) {
    const int64_t cam = (int64_t)((key >> L.cam_off) & fmask(L.cam_len));
    const int64_t sh = separate_shells ? (int64_t)((key >> L.shell_off) & fmask(L.shell_len)) : 0;
    const int64_t tile = (int64_t)((key >> L.tile_off) & fmask(L.tile_len));
    return (cam * Sd + sh) * T + tile;
  };
  for (int64_t i = 0; i < K; ++i) {
    const int64_t here = index_of((uint64_t)keys[i]);
    if (i > 0) {
      const int64_t last = index_of((uint64_t)keys[i - 1]);
      if (here != last) {
        out[2 * last + 1] = i;
        out[2 * here] = i;
      }
    }
    if (i == K - 1) out[2 * here + 1] = K;
  }
}

// ---------------------------------------------------------------------------
// intersect_and_composite.slang:224-339 (forward) and :341-564 (backward).
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {
struct FusedScene {
  const float* xy;
  const float* colors;
  const float* sdf;
  int64_t V;
  const int32_t* faces;
  float s;
  const int64_t* keys;
  const int32_t* tri;
  const int64_t* bounds;
  int B, S, rows, cols, th, tw, H, W, shell_off, shell_len;
};

struct Hit {
  int64_t k;  // position in the sorted list
  int32_t f;
  int shell;
  float u, v, w;
};

// All hits of one pixel, in compositing order (the shell-monotone walk).
inline void walk(const FusedScene& a, int cam, int64_t tile, float px, float py, std::vector<Hit>& hits) {
  hits.clear();
  const int64_t T = (int64_t)a.rows * a.cols;
  const int64_t start = a.bounds[2 * (cam * T + tile)], end = a.bounds[2 * (cam * T + tile) + 1];
  int last_shell = -1;
  const float* xy = a.xy + (int64_t)cam * a.V * 2;
  for (int64_t k = start; k < end; ++k) {
    const int shell = (int)(((uint64_t)a.keys[k] >> a.shell_off) & fmask(a.shell_len));
    if (shell <= last_shell) continue;
    const int32_t f = a.tri[k];
    const int32_t ia = a.faces[3 * (int64_t)f], ib = a.faces[3 * (int64_t)f + 1], ic = a.faces[3 * (int64_t)f + 2];
    float u, v, w;
    barycentric(xy[2 * ia], xy[2 * ia + 1], xy[2 * ib], xy[2 * ib + 1], xy[2 * ic], xy[2 * ic + 1], px, py, u, v, w);
    if (!accepted(u, v, w)) continue;
    hits.push_back({k, f, shell, u, v, w});
    last_shell = shell;
    if (last_shell == a.S - 1) break;
  }
}

inline void sample(const FusedScene& a, int cam, const Hit& h, float* rgb, float& sdf) {
  const int32_t ia = a.faces[3 * (int64_t)h.f], ib = a.faces[3 * (int64_t)h.f + 1], ic = a.faces[3 * (int64_t)h.f + 2];
  const float* col = a.colors + (int64_t)cam * a.V * 3;
  for (int c = 0; c < 3; ++c) rgb[c] = interp3(h.u, h.v, h.w, col[3 * ia + c], col[3 * ib + c], col[3 * ic + c]);
  sdf = interp3(h.u, h.v, h.w, a.sdf[ia], a.sdf[ib], a.sdf[ic]);
}
}  // namespace

extern "C" {

void or_intersect_and_composite_forward(const float* xy, const float* colors, const float* sdf, int64_t V,
                                        const int32_t* faces, float sharpness, const int64_t* keys,
                                        const int32_t* tri, const int64_t* bounds, int B, int S, int rows, int cols,
                                        int th, int tw, int H, int W, int shell_off, int shell_len, float* out) {
  const FusedScene a{xy, colors, sdf, V, faces, sharpness, keys, tri, bounds, B, S, rows, cols, th, tw, H, W,
                     shell_off, shell_len};
  const int64_t T = (int64_t)rows * cols;
#pragma omp parallel
  {
    std::vector<Hit> hits;
#pragma omp for schedule(dynamic, 4)
    for (int64_t bt = 0; bt < B * T; ++bt) {
      const int cam = (int)(bt / T);
      const int64_t tile = bt % T;
      for (int ty = 0; ty < th; ++ty)
        for (int tx = 0; tx < tw; ++tx) {
          const int px = (int)(tile % cols) * tw + tx, py = (int)(tile / cols) * th + ty;
          if (px >= W || py >= H) continue;
          walk(a, cam, tile, (float)px + 0.5f, (float)py + 0.5f, hits);
          float acc[3] = {0.f, 0.f, 0.f}, Tr = 1.0f, e;
          float outer_cdf = sdf_to_cdf(1e10f, sharpness, e);
          for (const Hit& h : hits) {
            float rgb[3], s_in;
            sample(a, cam, h, rgb, s_in);
            const float inner_cdf = sdf_to_cdf(s_in, sharpness, e);
            const float alpha = clamp01(alpha_raw(outer_cdf, inner_cdf));
            for (int c = 0; c < 3; ++c) acc[c] = acc[c] + rgb[c] * Tr * alpha;
            Tr = Tr * (1.0f - alpha);
            outer_cdf = inner_cdf;
          }
          const int64_t plane = (int64_t)H * W;
          float* o = out + (int64_t)cam * 4 * plane + (int64_t)py * W + px;
          o[0] = acc[0];
          o[plane] = acc[1];
          o[2 * plane] = acc[2];
          o[3 * plane] = Tr;
        }
    }
  }
}

// The hits the fused walk accepts at every pixel, in compositing order
// (at most one per shell): face index (-1 = none) and barycentrics (u, v, w).
void or_fused_hits(const float* xy, int64_t V, const int32_t* faces, const int64_t* keys, const int32_t* tri,
                   const int64_t* bounds, int B, int S, int rows, int cols, int th, int tw, int H, int W,
                   int shell_off, int shell_len, int32_t* out_face, float* out_uvw) {
  const FusedScene a{xy, nullptr, nullptr, V, faces, 0.f, keys, tri, bounds, B, S, rows, cols, th, tw, H, W,
                     shell_off, shell_len};
  const int64_t T = (int64_t)rows * cols;
#pragma omp parallel
  {
    std::vector<Hit> hits;
#pragma omp for schedule(dynamic, 4)
    for (int64_t bt = 0; bt < B * T; ++bt) {
      const int cam = (int)(bt / T);
      const int64_t tile = bt % T;
      for (int ty = 0; ty < th; ++ty)
        for (int tx = 0; tx < tw; ++tx) {
          const int px = (int)(tile % cols) * tw + tx, py = (int)(tile / cols) * th + ty;
          if (px >= W || py >= H) continue;
          walk(a, cam, tile, (float)px + 0.5f, (float)py + 0.5f, hits);
          const int64_t base = (((int64_t)cam * H + py) * W + px) * S;
          for (int l = 0; l < S; ++l) {
            const bool have = l < (int)hits.size();
            out_face[base + l] = have ? hits[l].f : -1;
            out_uvw[3 * (base + l)] = have ? hits[l].u : 0.f;
            out_uvw[3 * (base + l) + 1] = have ? hits[l].v : 0.f;
            out_uvw[3 * (base + l) + 2] = have ? hits[l].w : 0.f;
          }
        }
    }
  }
}

// exact = 0: the reference's routing (outer hit's deferred gradient scattered
// with the current hit's weights); exact = 1: the true adjoint.
void or_intersect_and_composite_backward(const float* xy, const float* colors, const float* sdf, int64_t V,
                                         const int32_t* faces, float sharpness, const int64_t* keys,
                                         const int32_t* tri, const int64_t* bounds, int B, int S, int rows,
                                         int cols, int th, int tw, int H, int W, int shell_off, int shell_len,
                                         const float* out, const float* grad_out, float* grad_colors,
                                         float* grad_sdf, float* grad_sharpness, int exact) {
  const FusedScene a{xy, colors, sdf, V, faces, sharpness, keys, tri, bounds, B, S, rows, cols, th, tw, H, W,
                     shell_off, shell_len};
  const int64_t T = (int64_t)rows * cols;
  const float s = sharpness;
  double d_sharp_total = 0.0;
#pragma omp parallel reduction(+ : d_sharp_total)
  {
    std::vector<Hit> hits;
    auto scatter = [&](int cam, int32_t f, float u, float v, float w, const float* drgb, float dsdf) {
      const int32_t id[3] = {faces[3 * (int64_t)f], faces[3 * (int64_t)f + 1], faces[3 * (int64_t)f + 2]};
      const float wt[3] = {u, v, w};
      for (int q = 0; q < 3; ++q) {
        for (int c = 0; c < 3; ++c) {
#pragma omp atomic
          grad_colors[((int64_t)cam * V + id[q]) * 3 + c] += wt[q] * drgb[c];
        }
#pragma omp atomic
        grad_sdf[id[q]] += wt[q] * dsdf;
      }
    };
#pragma omp for schedule(dynamic, 4)
    for (int64_t bt = 0; bt < B * T; ++bt) {
      const int cam = (int)(bt / T);
      const int64_t tile = bt % T;
      for (int ty = 0; ty < th; ++ty)
        for (int tx = 0; tx < tw; ++tx) {
          const int px = (int)(tile % cols) * tw + tx, py = (int)(tile / cols) * th + ty;
          if (px >= W || py >= H) continue;
          walk(a, cam, tile, (float)px + 0.5f, (float)py + 0.5f, hits);
          const int64_t plane = (int64_t)H * W;
          const int64_t o = (int64_t)cam * 4 * plane + (int64_t)py * W + px;
          float final_rgb[3], dL[3];
          for (int c = 0; c < 3; ++c) {
            final_rgb[c] = out[o + c * plane];
            dL[c] = grad_out[o + c * plane];
          }
          const float final_T = out[o + 3 * plane], dLT = grad_out[o + 3 * plane];
          float acc[3] = {0.f, 0.f, 0.f}, Tr = 1.0f, e_out;
          float outer_cdf = sdf_to_cdf(1e10f, s, e_out), outer_sdf = 1e10f;
          float dp_rgb[3] = {0.f, 0.f, 0.f}, dp_sdf = 0.f;
          const Hit* prev = nullptr;
          for (const Hit& h : hits) {
            float rgb[3], s_in, e_in;
            sample(a, cam, h, rgb, s_in);
            const float inner_cdf = sdf_to_cdf(s_in, s, e_in);
            const float raw = alpha_raw(outer_cdf, inner_cdf);
            const float alpha = clamp01(raw);
            const float weight = alpha * Tr;
            const float inv = 1.0f / ((1.0f - alpha) + 1e-6f);
            float d_color[3], d_alpha = 0.f;
            for (int c = 0; c < 3; ++c) {
              acc[c] = acc[c] + weight * rgb[c];
              const float suffix = final_rgb[c] - acc[c];
              d_color[c] = weight * dL[c];
              d_alpha += dL[c] * (Tr * rgb[c] - suffix * inv);
            }
            d_alpha += -dLT * final_T * inv;
            const float d_raw = (raw > 0.0f && raw < 1.0f) ? d_alpha : 0.0f;
            const float den = outer_cdf + 1e-5f, num = (outer_cdf - inner_cdf) + 1e-5f;
            const float d_num = d_raw / den, d_den = -d_raw * num / (den * den);
            const float d_oc = d_num + d_den, d_ic = -d_num;
            const float ki = inner_cdf * inner_cdf * e_in, ko = outer_cdf * outer_cdf * e_out;
            d_sharp_total += (double)(d_ic * ki * s_in + d_oc * ko * outer_sdf);
            if (prev) {
              dp_sdf += d_oc * ko * s;
              if (exact)
                scatter(cam, prev->f, prev->u, prev->v, prev->w, dp_rgb, dp_sdf);
              else
                scatter(cam, prev->f, h.u, h.v, h.w, dp_rgb, dp_sdf);
            }
            for (int c = 0; c < 3; ++c) dp_rgb[c] = d_color[c];
            dp_sdf = d_ic * ki * s;
            prev = &h;
            Tr = Tr * (1.0f - alpha);
            outer_cdf = inner_cdf;
            outer_sdf = s_in;
            e_out = e_in;
          }
          if (prev) scatter(cam, prev->f, prev->u, prev->v, prev->w, dp_rgb, dp_sdf);
        }
    }
  }
  grad_sharpness[0] += (float)d_sharp_total;
}

// ---------------------------------------------------------------------------
// Explicit mode: intersect.slang:86-182, interpolate.slang:19-76,
// composite.slang:60-218.
// ---------------------------------------------------------------------------
void or_intersect(const float* xy, int64_t V, const int32_t* faces, const int32_t* tri, const int64_t* bounds, int B,
                  int S, int rows, int cols, int th, int tw, int H, int W, float* out_uv, int32_t* out_index) {
  const int64_t T = (int64_t)rows * cols;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t bt = 0; bt < (int64_t)B * S * T; ++bt) {
    const int64_t batch = bt / T, tile = bt % T;
    const int cam = (int)(batch / S);
    const float* p = xy + (int64_t)cam * V * 2;
    const int64_t start = bounds[2 * bt], end = bounds[2 * bt + 1];
    for (int ty = 0; ty < th; ++ty)
      for (int tx = 0; tx < tw; ++tx) {
        const int px = (int)(tile % cols) * tw + tx, py = (int)(tile / cols) * th + ty;
        if (px >= W || py >= H) continue;
        const int64_t o = (batch * H + py) * W + px;
        out_uv[2 * o] = 0.f;
        out_uv[2 * o + 1] = 0.f;
        out_index[o] = -1;
        for (int64_t k = start; k < end; ++k) {
          const int32_t f = tri[k];
          const int32_t ia = faces[3 * (int64_t)f], ib = faces[3 * (int64_t)f + 1], ic = faces[3 * (int64_t)f + 2];
          float u, v, w;
          barycentric(p[2 * ia], p[2 * ia + 1], p[2 * ib], p[2 * ib + 1], p[2 * ic], p[2 * ic + 1], (float)px + 0.5f,
                      (float)py + 0.5f, u, v, w);
          if (!accepted(u, v, w)) continue;
          out_uv[2 * o] = u;
          out_uv[2 * o + 1] = v;
          out_index[o] = f;
          break;
        }
      }
  }
}

void or_interpolate(const float* uv, const int32_t* index, int B, int S, int H, int W, const int32_t* faces,
                    const float* sdf, const float* colors, int64_t V, float* out_sdf, float* out_colors) {
  const int64_t HW = (int64_t)H * W, total = (int64_t)B * S * HW;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < total; ++i) {
    const int32_t f = index[i];
    if (f < 0) {
      out_sdf[i] = 0.f;
      for (int c = 0; c < 3; ++c) out_colors[3 * i + c] = 0.f;
      continue;
    }
    const int64_t b = (i / HW) / S;
    const float u = uv[2 * i], v = uv[2 * i + 1], w = (1.0f - u) - v;
    const int32_t ia = faces[3 * (int64_t)f], ib = faces[3 * (int64_t)f + 1], ic = faces[3 * (int64_t)f + 2];
    const float* col = colors + b * V * 3;
    for (int c = 0; c < 3; ++c) out_colors[3 * i + c] = interp3(u, v, w, col[3 * ia + c], col[3 * ib + c], col[3 * ic + c]);
    out_sdf[i] = interp3(u, v, w, sdf[ia], sdf[ib], sdf[ic]);
  }
}

void or_interpolate_backward(const float* uv, const int32_t* index, int B, int S, int H, int W, const int32_t* faces,
                             int64_t V, const float* gsdf_out, const float* gcol_out, float* gsdf, float* gcol) {
  const int64_t HW = (int64_t)H * W, total = (int64_t)B * S * HW;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < total; ++i) {
    const int32_t f = index[i];
    if (f < 0) continue;
    const int64_t b = (i / HW) / S;
    const float u = uv[2 * i], v = uv[2 * i + 1], w = (1.0f - u) - v;
    const int32_t id[3] = {faces[3 * (int64_t)f], faces[3 * (int64_t)f + 1], faces[3 * (int64_t)f + 2]};
    const float wt[3] = {u, v, w};
    for (int q = 0; q < 3; ++q) {
      if (gsdf_out) {
#pragma omp atomic
        gsdf[id[q]] += wt[q] * gsdf_out[i];
      }
      if (gcol_out)
        for (int c = 0; c < 3; ++c) {
#pragma omp atomic
          gcol[(b * V + id[q]) * 3 + c] += wt[q] * gcol_out[3 * i + c];
        }
    }
  }
}

void or_composite(const float* sdf, const float* colors, const uint8_t* mask, int64_t P, int S, float sharpness,
                  float* out_colors, float* out_T) {
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < P; ++p) {
    float acc[3] = {0.f, 0.f, 0.f}, Tr = 1.0f, e;
    float outer_cdf = sdf_to_cdf(1e10f, sharpness, e);
    for (int l = 0; l < S; ++l) {
      if (!mask[p * S + l]) continue;
      const float inner_cdf = sdf_to_cdf(sdf[p * S + l], sharpness, e);
      const float alpha = clamp01(alpha_raw(outer_cdf, inner_cdf));
      for (int c = 0; c < 3; ++c) acc[c] = acc[c] + colors[(p * S + l) * 3 + c] * Tr * alpha;
      Tr = Tr * (1.0f - alpha);
      outer_cdf = inner_cdf;
    }
    for (int c = 0; c < 3; ++c) out_colors[3 * p + c] = acc[c];
    out_T[p] = Tr;
  }
}

void or_composite_backward(const float* sdf, const float* colors, const uint8_t* mask, int64_t P, int S,
                           float sharpness, const float* out_colors, const float* out_T, const float* gcol_out,
                           const float* gT_out, float* gsdf, float* gcol, float* gsharp, int exact) {
  const float s = sharpness;
  double total = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : total)
  for (int64_t p = 0; p < P; ++p) {
    const float dL[3] = {gcol_out ? gcol_out[3 * p] : 0.f, gcol_out ? gcol_out[3 * p + 1] : 0.f,
                         gcol_out ? gcol_out[3 * p + 2] : 0.f};
    const float dLT = gT_out ? gT_out[p] : 0.f;
    float acc[3] = {0.f, 0.f, 0.f}, Tr = 1.0f, e_out;
    float outer_cdf = sdf_to_cdf(1e10f, s, e_out), outer_sdf = 1e10f, d_partial = 0.f;
    int prev_shell = -1;
    for (int l = 0; l < S; ++l) {
      if (!mask[p * S + l]) continue;
      const float inner = sdf[p * S + l];
      float e_in;
      const float inner_cdf = sdf_to_cdf(inner, s, e_in);
      const float raw = alpha_raw(outer_cdf, inner_cdf), alpha = clamp01(raw);
      const float weight = alpha * Tr, inv = 1.0f / ((1.0f - alpha) + 1e-6f);
      float d_alpha = 0.f;
      for (int c = 0; c < 3; ++c) {
        const float col = colors[(p * S + l) * 3 + c];
        acc[c] = acc[c] + weight * col;
        d_alpha += dL[c] * (Tr * col - (out_colors[3 * p + c] - acc[c]) * inv);
        gcol[(p * S + l) * 3 + c] += weight * dL[c];
      }
      d_alpha += -dLT * out_T[p] * inv;
      const float d_raw = (raw > 0.0f && raw < 1.0f) ? d_alpha : 0.0f;
      const float den = outer_cdf + 1e-5f, num = (outer_cdf - inner_cdf) + 1e-5f;
      const float d_num = d_raw / den, d_den = -d_raw * num / (den * den);
      const float d_oc = d_num + d_den, d_ic = -d_num;
      const float ki = inner_cdf * inner_cdf * e_in, ko = outer_cdf * outer_cdf * e_out;
      total += (double)(d_ic * ki * inner + d_oc * ko * outer_sdf);
      if (prev_shell >= 0) {
        d_partial += d_oc * ko * s;
        gsdf[p * S + (exact ? prev_shell : l - 1)] += d_partial;
      }
      d_partial = d_ic * ki * s;
      Tr = Tr * (1.0f - alpha);
      outer_cdf = inner_cdf;
      outer_sdf = inner;
      e_out = e_in;
      prev_shell = l;
    }
    if (prev_shell >= 0) gsdf[p * S + (exact ? prev_shell : S - 1)] += d_partial;
  }
  gsharp[0] += (float)total;
}

}  // extern "C"
