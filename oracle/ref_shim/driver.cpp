// Grid emulation and C ABI for the reference's kernels compiled on the host.
//
// TEST INFRASTRUCTURE ONLY. Includes the rewritten reference sources that
// oracle/build_ref.py writes into oracle/_ref/ (one namespace per kernel
// file and compile-time configuration) and exposes each kernel as an
// extern "C" function that launches it over the same grid as the reference's
// Python wrapper. Kernels without barriers run their blocks in parallel;
// kernels with CTA barriers run one block at a time, each emulated thread on
// its own OS thread, synchronised by a std::barrier.

#include <cstdlib>
#include <functional>
#include <thread>
#include <vector>

#include "slang.h"

// ---------------------------------------------------------------------------
// Grid emulation
// ---------------------------------------------------------------------------
namespace {

uint3 ceil_grid(uint3 n, uint3 b) { return uint3((n.x + b.x - 1) / b.x, (n.y + b.y - 1) / b.y, (n.z + b.z - 1) / b.z); }

void run_grid(uint3 grid, uint3 block, const std::function<void()>& kernel) {
  const int64_t blocks = (int64_t)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t bi = 0; bi < blocks; ++bi) {
    g_block_idx = uint3(bi % grid.x, (bi / grid.x) % grid.y, bi / ((int64_t)grid.x * grid.y));
    g_block_dim = block;
    g_block_barrier = nullptr;
    for (uint tz = 0; tz < block.z; ++tz)
      for (uint ty = 0; ty < block.y; ++ty)
        for (uint tx = 0; tx < block.x; ++tx) {
          g_thread_idx = uint3(tx, ty, tz);
          kernel();
        }
  }
}

// Blocks one at a time; every thread of a block on its own OS thread.
void run_grid_with_barriers(uint3 grid, uint3 block, const std::function<void()>& kernel) {
  const uint threads = block.x * block.y * block.z;
  for (int64_t bi = 0; bi < (int64_t)grid.x * grid.y * grid.z; ++bi) {
    const uint3 bidx(bi % grid.x, (bi / grid.x) % grid.y, bi / ((int64_t)grid.x * grid.y));
    std::barrier<> sync((std::ptrdiff_t)threads);
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (uint t = 0; t < threads; ++t) {
      pool.emplace_back([&, t]() {
        g_block_idx = bidx;
        g_block_dim = block;
        g_thread_idx = uint3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
        g_block_barrier = &sync;
        kernel();
      });
    }
    for (auto& th : pool) th.join();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Rewritten reference sources
// ---------------------------------------------------------------------------
namespace k_vertex_occupancy {
#include "triangle_extraction__compute_vertex_occupancy.inc"
}
namespace k_count_occupancy {
#include "triangle_extraction__count_occupancy.inc"
}
namespace k_create_voxels {
#include "triangle_extraction__create_voxels.inc"
}
namespace k_dilate {
#include "triangle_extraction__dilate_occupancy.inc"
}
namespace k_count_vertices {
#include "triangle_extraction__count_triangle_vertices.inc"
}
#define NUM_SPHERICAL_HARMONICS 1
namespace k_create_vertices_1 {
#include "triangle_extraction__create_triangle_vertices.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 4
namespace k_create_vertices_4 {
#include "triangle_extraction__create_triangle_vertices.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 9
namespace k_create_vertices_9 {
#include "triangle_extraction__create_triangle_vertices.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 16
namespace k_create_vertices_16 {
#include "triangle_extraction__create_triangle_vertices.inc"
}
#undef NUM_SPHERICAL_HARMONICS
namespace k_count_faces {
#include "triangle_extraction__count_triangle_faces.inc"
}
namespace k_create_faces {
#include "triangle_extraction__create_triangle_faces.inc"
}
namespace k_regularizers {
#include "triangle_extraction__compute_sdf_regularizers.inc"
}
namespace k_write_occupancy {
#include "triangle_extraction__write_occupancy.inc"
}
namespace k_upscale_occupancy {
#include "triangle_extraction__upscale_occupancy.inc"
}
#define NUM_SPHERICAL_HARMONICS 1
namespace k_upscale_parameters_1 {
#include "triangle_extraction__upscale_parameters.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 4
namespace k_upscale_parameters_4 {
#include "triangle_extraction__upscale_parameters.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 9
namespace k_upscale_parameters_9 {
#include "triangle_extraction__upscale_parameters.inc"
}
#undef NUM_SPHERICAL_HARMONICS
#define NUM_SPHERICAL_HARMONICS 16
namespace k_upscale_parameters_16 {
#include "triangle_extraction__upscale_parameters.inc"
}
#undef NUM_SPHERICAL_HARMONICS
namespace k_occupancy_mesh {
#include "triangle_extraction__get_occupancy_mesh.inc"
}
namespace k_project {
#include "triangle_rasterization__project_vertices.inc"
}
namespace k_bound {
#include "triangle_rasterization__bound_triangles.inc"
}

// Fused key layout, MSB first: camera(6) | tile(20) | depth(32) | shell(6).
#define CAMERA_BIT_OFFSET 58
#define CAMERA_BIT_LENGTH 6
#define TILE_BIT_OFFSET 38
#define TILE_BIT_LENGTH 20
#define DEPTH_BIT_OFFSET 6
#define DEPTH_BIT_LENGTH 32
#define SHELL_BIT_OFFSET 0
#define SHELL_BIT_LENGTH 6
namespace k_keys_fused {
#include "triangle_rasterization__generate_keys.inc"
}
namespace k_delineate_fused {
#include "triangle_rasterization__delineate_tiles.inc"
}
#define TILE_HEIGHT 16
#define TILE_WIDTH 16
namespace k_fused_16 {
#include "triangle_rasterization__intersect_and_composite.inc"
}
#undef TILE_HEIGHT
#undef TILE_WIDTH
#undef CAMERA_BIT_OFFSET
#undef CAMERA_BIT_LENGTH
#undef TILE_BIT_OFFSET
#undef TILE_BIT_LENGTH
#undef DEPTH_BIT_OFFSET
#undef DEPTH_BIT_LENGTH
#undef SHELL_BIT_OFFSET
#undef SHELL_BIT_LENGTH

// Explicit key layout, MSB first: camera(6) | shell(6) | tile(20) | depth(32).
#define CAMERA_BIT_OFFSET 58
#define CAMERA_BIT_LENGTH 6
#define SHELL_BIT_OFFSET 52
#define SHELL_BIT_LENGTH 6
#define TILE_BIT_OFFSET 32
#define TILE_BIT_LENGTH 20
#define DEPTH_BIT_OFFSET 0
#define DEPTH_BIT_LENGTH 32
namespace k_keys_explicit {
#include "triangle_rasterization__generate_keys.inc"
}
namespace k_delineate_explicit {
#include "triangle_rasterization__delineate_tiles.inc"
}
#define TILE_HEIGHT 16
#define TILE_WIDTH 16
namespace k_intersect_16 {
#include "triangle_rasterization__intersect.inc"
}
#undef TILE_HEIGHT
#undef TILE_WIDTH

#define SH_DEGREE 0
namespace k_sh_0 {
#include "triangle_rasterization__evaluate_spherical_harmonics.inc"
}
#undef SH_DEGREE
#define SH_DEGREE 1
namespace k_sh_1 {
#include "triangle_rasterization__evaluate_spherical_harmonics.inc"
}
#undef SH_DEGREE
#define SH_DEGREE 2
namespace k_sh_2 {
#include "triangle_rasterization__evaluate_spherical_harmonics.inc"
}
#undef SH_DEGREE
#define SH_DEGREE 3
namespace k_sh_3 {
#include "triangle_rasterization__evaluate_spherical_harmonics.inc"
}
#undef SH_DEGREE
namespace k_interpolate {
#include "triangle_rasterization__interpolate.inc"
}
namespace k_composite {
#include "triangle_rasterization__composite.inc"
}

// ---------------------------------------------------------------------------
// C ABI: each function launches the kernel over the reference wrapper's grid.
// ---------------------------------------------------------------------------
extern "C" {

// compute_vertex_occupancy.py:47-56
void ref_compute_vertex_occupancy(int32_t* occ, int I, int J, int KP, int32_t* vocc, int32_t* vcounts) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> v(vocc, {(uint64_t)I + 1, (uint64_t)J + 1, (uint64_t)KP + 1});
  TensorView<int> c(vcounts, {(uint64_t)I + 1, (uint64_t)J + 1, (uint64_t)KP + 1});
  run_grid(ceil_grid(uint3(I + 1, J + 1, KP + 1), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_vertex_occupancy::compute_vertex_occupancy(o, v, c); });
  vcounts[(int64_t)(I + 1) * (J + 1) * (KP + 1)] = 0;
}

// count_occupancy.py:33-44 (output zero-filled by the caller)
void ref_count_occupancy(int32_t* occ, int I, int J, int KP, int32_t* counts) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> c(counts, {(uint64_t)I + 1, (uint64_t)J + 1, (uint64_t)KP + 1});
  run_grid(ceil_grid(uint3(I, J, KP), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_count_occupancy::count_occupancy(o, c); });
}

// create_voxels.py:66-88
void ref_create_voxels(int32_t* occ, int32_t* xoff, int32_t* vocc, int32_t* voff, int I, int J, int KP, int64_t Nv,
                       int64_t G, float* vertices, int32_t* neighbors, int32_t* lower, int32_t* upper,
                       int32_t* indices) {
  if (Nv <= 0) return;
  const uint64_t i1 = I + 1, j1 = J + 1, k1 = KP + 1;
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> xo(xoff, {i1, j1, k1}), vo(vocc, {i1, j1, k1}), vf(voff, {i1, j1, k1});
  TensorView<float> ve(vertices, {(uint64_t)G, 3});
  TensorView<int> nb(neighbors, {7, (uint64_t)Nv}), lc(lower, {4, (uint64_t)G}), uc(upper, {4, (uint64_t)Nv});
  TensorView<int> ix(indices, {(uint64_t)Nv});
  run_grid(ceil_grid(uint3(I + 1, J + 1, KP + 1), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_create_voxels::create_voxels(o, xo, vo, vf, ve, nb, lc, uc, ix); });
}

// dilate_occupancy.py:36-46
void ref_dilate_occupancy(int32_t* occ, int I, int J, int KP, int d, int32_t* out) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP}), n(out, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  run_grid(ceil_grid(uint3(I, J, KP), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_dilate::dilate_occupancy(o, n, d); });
}

// write_occupancy.py:30-44 (grid zero-filled by the caller)
void ref_write_occupancy(int32_t* voxel_indices, int64_t n, int32_t* occ, int64_t words) {
  TensorView<int> o(occ, {(uint64_t)words}), v(voxel_indices, {(uint64_t)n});
  run_grid(uint3((uint)((n + 255) / 256), 1, 1), uint3(256, 1, 1),
           [&] { k_write_occupancy::write_occupancy(o, v, 0, 1); });
}

// upscale_occupancy.py:42-52
void ref_upscale_occupancy(int32_t* occ, int I, int J, int KP, int I2, int J2, int KP2, int32_t* out) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> n(out, {(uint64_t)I2, (uint64_t)J2, (uint64_t)KP2});
  run_grid(ceil_grid(uint3(I2, J2, KP2), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_upscale_occupancy::upscale_occupancy(o, n); });
}

// upscale_parameters.py:77-93
void ref_upscale_parameters(int C, int32_t* ovocc, int32_t* ovoff, float* osdf, float* osh, int64_t Vold, int I1,
                            int J1, int KP1, int32_t* nvocc, int32_t* nvoff, int I1n, int J1n, int KP1n,
                            int64_t Vnew, float* nsdf, float* nsh) {
  TensorView<int> ov(ovocc, {(uint64_t)I1, (uint64_t)J1, (uint64_t)KP1});
  TensorView<int> oo(ovoff, {(uint64_t)I1, (uint64_t)J1, (uint64_t)KP1});
  TensorView<float> od(osdf, {(uint64_t)Vold}), osv(osh, {(uint64_t)C, (uint64_t)Vold, 3});
  TensorView<int> nv(nvocc, {(uint64_t)I1n, (uint64_t)J1n, (uint64_t)KP1n});
  TensorView<int> no(nvoff, {(uint64_t)I1n, (uint64_t)J1n, (uint64_t)KP1n});
  TensorView<float> nd(nsdf, {(uint64_t)Vnew}), nsv(nsh, {(uint64_t)C, (uint64_t)Vnew, 3});
  const uint3 grid = ceil_grid(uint3(I1n, J1n, KP1n), uint3(32, 32, 1)), block(32, 32, 1);
  switch (C) {
    case 1: run_grid(grid, block, [&] { k_upscale_parameters_1::upscale_parameters(ov, oo, od, osv, nv, no, nd, nsv); }); break;
    case 4: run_grid(grid, block, [&] { k_upscale_parameters_4::upscale_parameters(ov, oo, od, osv, nv, no, nd, nsv); }); break;
    case 9: run_grid(grid, block, [&] { k_upscale_parameters_9::upscale_parameters(ov, oo, od, osv, nv, no, nd, nsv); }); break;
    case 16: run_grid(grid, block, [&] { k_upscale_parameters_16::upscale_parameters(ov, oo, od, osv, nv, no, nd, nsv); }); break;
    default: std::abort();
  }
}

// get_occupancy_mesh.py:43-56 (counts zero-filled by the caller)
void ref_count_occupancy_mesh_triangles(int32_t* occ, int I, int J, int KP, int32_t* counts) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> c(counts, {(uint64_t)I + 1, (uint64_t)J + 1, (uint64_t)KP + 1});
  run_grid(ceil_grid(uint3(I + 1, J + 1, KP + 1), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_occupancy_mesh::count_triangles(o, c); });
}

// get_occupancy_mesh.py:66-78
void ref_create_occupancy_mesh_triangles(int32_t* occ, int I, int J, int KP, int32_t* offsets, int64_t T,
                                         float* verts, float* tri_colors, float* colors) {
  TensorView<int> o(occ, {(uint64_t)I, (uint64_t)J, (uint64_t)KP});
  TensorView<int> off(offsets, {(uint64_t)I + 1, (uint64_t)J + 1, (uint64_t)KP + 1});
  TensorView<float> tv(verts, {(uint64_t)T, 3, 3}), tc(tri_colors, {(uint64_t)T, 3}), col(colors, {3, 2, 3});
  run_grid(ceil_grid(uint3(I + 1, J + 1, KP + 1), uint3(32, 32, 1)), uint3(32, 32, 1),
           [&] { k_occupancy_mesh::create_triangles(o, off, tv, tc, col); });
}

// count_triangle_vertices.py:31-50
void ref_count_triangle_vertices(float* sdf, int32_t* lower, int64_t G, float* level_sets, int S, int32_t* counts) {
  TensorView<float> d(sdf, {(uint64_t)G}), ls(level_sets, {(uint64_t)S});
  TensorView<int> lc(lower, {4, (uint64_t)G}), c(counts, {(uint64_t)S, (uint64_t)G});
  run_grid(uint3((G + 255) / 256, 1, 1), uint3(256, 1, 1),
           [&] { k_count_vertices::countTriangleVertices(d, lc, ls, c); });
  counts[(int64_t)S * G] = 0;
}

// create_triangle_vertices.py:51-84 (forward)
void ref_create_triangle_vertices(float* gv, float* gsdf, float* gsh, int C, int32_t* lower, int64_t G,
                                  float* level_sets, int S, int32_t* voff, int64_t V, float* out_v, float* out_sdf,
                                  float* out_sh, uint8_t* out_type) {
  TensorView<float> v(gv, {(uint64_t)G, 3}), d(gsdf, {(uint64_t)G}), sh(gsh, {(uint64_t)C, (uint64_t)G, 3});
  TensorView<int> lc(lower, {4, (uint64_t)G}), vo(voff, {(uint64_t)S, (uint64_t)G});
  TensorView<float> ls(level_sets, {(uint64_t)S});
  TensorView<float> ov(out_v, {(uint64_t)V, 3}), od(out_sdf, {(uint64_t)V}), osh(out_sh, {(uint64_t)C, (uint64_t)V, 3});
  TensorView<uint8_t> ot(out_type, {(uint64_t)V});
  const uint3 grid((G + 255) / 256, 1, 1), block(256, 1, 1);
  if (C == 1)
    run_grid(grid, block, [&] { k_create_vertices_1::create_triangle_vertices_forward(v, d, sh, lc, vo, ls, ov, od, osh, ot); });
  else if (C == 4)
    run_grid(grid, block, [&] { k_create_vertices_4::create_triangle_vertices_forward(v, d, sh, lc, vo, ls, ov, od, osh, ot); });
  else if (C == 9)
    run_grid(grid, block, [&] { k_create_vertices_9::create_triangle_vertices_forward(v, d, sh, lc, vo, ls, ov, od, osh, ot); });
  else if (C == 16)
    run_grid(grid, block, [&] { k_create_vertices_16::create_triangle_vertices_forward(v, d, sh, lc, vo, ls, ov, od, osh, ot); });
  else
    std::abort();
}

// compute_sdf_regularizers.py:47-71 (forward).
void ref_compute_sdf_regularizers(float* sdf, int64_t G, int32_t* neighbors, int32_t* lower, int32_t* upper,
                                  int64_t Nv, int vx, int vy, int vz, float* pos, float* neg, float* curv) {
  DiffTensorView d(TensorView<float>(sdf, {(uint64_t)G}));
  TensorView<int> nb(neighbors, {7, (uint64_t)Nv}), lc(lower, {4, (uint64_t)G}), uc(upper, {4, (uint64_t)Nv});
  DiffTensorView p(TensorView<float>(pos, {(uint64_t)Nv})), n(TensorView<float>(neg, {(uint64_t)Nv}));
  DiffTensorView c(TensorView<float>(curv, {(uint64_t)Nv}));
  run_grid(uint3((uint)((Nv + 255) / 256), 1, 1), uint3(256, 1, 1),
           [&] { k_regularizers::compute_sdf_regularizers(d, nb, lc, uc, vx, vy, vz, p, n, c); });
}

// count_triangle_faces.py:48-61
void ref_count_triangle_faces(float* sdf, int32_t* lower, int64_t G, int32_t* upper, int64_t Nv, float* level_sets,
                              int S, int32_t* counts, uint8_t* codes) {
  TensorView<float> d(sdf, {(uint64_t)G}), ls(level_sets, {(uint64_t)S});
  TensorView<int> lc(lower, {4, (uint64_t)G}), uc(upper, {4, (uint64_t)Nv}), c(counts, {(uint64_t)S, (uint64_t)Nv});
  TensorView<uint8_t> cc(codes, {(uint64_t)S, (uint64_t)Nv});
  run_grid(uint3((Nv + 255) / 256, 1, 1), uint3(256, 1, 1),
           [&] { k_count_faces::count_triangle_faces(d, lc, uc, ls, c, cc); });
  counts[(int64_t)S * Nv] = 0;
}

// create_triangle_faces.py:46-63
void ref_create_triangle_faces(float* sdf, int64_t G, int32_t* neighbors, int32_t* indices, int64_t Nv,
                               int32_t* voff, uint8_t* types, int64_t V, uint8_t* codes, float* level_sets, int S,
                               int32_t* foff, int32_t* faces, int32_t* voxel_indices, int64_t F) {
  TensorView<float> d(sdf, {(uint64_t)G}), ls(level_sets, {(uint64_t)S});
  TensorView<int> nb(neighbors, {7, (uint64_t)Nv}), ix(indices, {(uint64_t)Nv});
  TensorView<int> vo(voff, {(uint64_t)S * G + 1});
  TensorView<uint8_t> ty(types, {(uint64_t)V}), cc(codes, {(uint64_t)S, (uint64_t)Nv});
  TensorView<int> fo(foff, {(uint64_t)S * Nv + 1}), fa(faces, {(uint64_t)F, 3}), vi(voxel_indices, {(uint64_t)F});
  run_grid(uint3((Nv + 255) / 256, 1, 1), uint3(256, 1, 1),
           [&] { k_create_faces::create_triangle_faces(d, nb, ix, vo, ty, cc, ls, fa, vi, (int)G, fo); });
}

// project_vertices.py:44-54
void ref_project_vertices(float* ext, float* intr, int B, float* verts, int64_t V, float* out_xy, float* out_depth) {
  TensorView<float> e(ext, {(uint64_t)B, 4, 4}), k(intr, {(uint64_t)B, 3, 3}), v(verts, {(uint64_t)V, 3});
  TensorView<float> xy(out_xy, {(uint64_t)B, (uint64_t)V, 2}), dp(out_depth, {(uint64_t)B, (uint64_t)V});
  run_grid(uint3((V + 255) / 256, 1, 1), uint3(256, 1, 1), [&] { k_project::project_vertices(e, k, v, xy, dp); });
}

// bound_triangles.py:51-69
void ref_bound_triangles(float* xy, float* depth, int B, int64_t V, int32_t* faces, int64_t F, int tile_h, int tile_w,
                         int rows, int cols, float near, int32_t* out_min, int32_t* out_max, int32_t* out_count) {
  TensorView<float> v(xy, {(uint64_t)B, (uint64_t)V, 2}), d(depth, {(uint64_t)B, (uint64_t)V});
  TensorView<int> f(faces, {(uint64_t)F, 3});
  TensorView<int> mn(out_min, {(uint64_t)B, (uint64_t)F, 2}), mx(out_max, {(uint64_t)B, (uint64_t)F, 2});
  TensorView<int> ct(out_count, {(uint64_t)B, (uint64_t)F});
  run_grid(uint3((F + 255) / 256, 1, 1), uint3(256, 1, 1), [&] {
    k_bound::bound_triangles(v, d, f, tile_h, tile_w, 0, 0, rows, cols, near, mn, mx, ct);
  });
}

// generate_keys.py:52-68; offsets are the inclusive int64 cumsum.
void ref_generate_keys(int explicit_layout, float* depth, int B, int64_t V, int32_t* faces, int64_t F, int32_t* sfb,
                       int S, int32_t* tmin, int32_t* tmax, int64_t* offsets, int grid_width, int64_t K,
                       int64_t* out_keys, int32_t* out_tri) {
  TensorView<float> d(depth, {(uint64_t)B, (uint64_t)V});
  TensorView<int> f(faces, {(uint64_t)F, 3}), s(sfb, {(uint64_t)S});
  TensorView<int> mn(tmin, {(uint64_t)B, (uint64_t)F, 2}), mx(tmax, {(uint64_t)B, (uint64_t)F, 2});
  TensorView<int64_t> of(offsets, {(uint64_t)B * F}), ok(out_keys, {(uint64_t)K});
  TensorView<int> ot(out_tri, {(uint64_t)K});
  const uint3 grid((F + 255) / 256, 1, 1), block(256, 1, 1);
  if (explicit_layout)
    run_grid(grid, block, [&] { k_keys_explicit::generate_keys(d, f, s, mn, mx, of, grid_width, ok, ot); });
  else
    run_grid(grid, block, [&] { k_keys_fused::generate_keys(d, f, s, mn, mx, of, grid_width, ok, ot); });
}

// delineate_tiles.py:40-53 (output zero-filled by the caller)
void ref_delineate_tiles(int explicit_layout, int64_t* keys, int64_t K, int B, int Sd, int64_t T, int separate,
                         int64_t* out) {
  int64_t num_keys = K;
  TensorView<int64_t> k(keys, {(uint64_t)K}), n(&num_keys, {1}), o(out, {(uint64_t)B, (uint64_t)Sd, (uint64_t)T, 2});
  const uint3 grid((K + 255) / 256, 1, 1), block(256, 1, 1);
  if (explicit_layout)
    run_grid(grid, block, [&] { k_delineate_explicit::delineate_tiles(k, n, o, separate != 0, 1e-8f); });
  else
    run_grid(grid, block, [&] { k_delineate_fused::delineate_tiles(k, n, o, separate != 0, 1e-8f); });
}

// evaluate_spherical_harmonics.py:42-53; camera positions given.
void ref_evaluate_sh(int degree, float* verts, int64_t V, float* sh, int C, float* campos, int B, float* out) {
  TensorView<float> v(verts, {(uint64_t)V, 3}), s(sh, {(uint64_t)C, (uint64_t)V, 3}), c(campos, {(uint64_t)B, 3});
  TensorView<float> o(out, {(uint64_t)B, (uint64_t)V, 3});
  const uint3 grid((V + 255) / 256, 1, 1), block(256, 1, 1);
  switch (degree) {
    case 0: run_grid(grid, block, [&] { k_sh_0::evaluate_spherical_harmonics_forward(v, s, c, o); }); break;
    case 1: run_grid(grid, block, [&] { k_sh_1::evaluate_spherical_harmonics_forward(v, s, c, o); }); break;
    case 2: run_grid(grid, block, [&] { k_sh_2::evaluate_spherical_harmonics_forward(v, s, c, o); }); break;
    default: run_grid(grid, block, [&] { k_sh_3::evaluate_spherical_harmonics_forward(v, s, c, o); }); break;
  }
}

// intersect_and_composite.py:46-63 (tile 16x16, fused layout).
void ref_intersect_and_composite_forward(float* xy, float* colors, float* sdf, int B, int64_t V, int32_t* faces,
                                         int64_t F, float sharpness, int64_t* keys, int32_t* tri, int64_t K,
                                         int64_t* bounds, int num_shells, int rows, int cols, int H, int W,
                                         float* out) {
  TensorView<float> v(xy, {(uint64_t)B, (uint64_t)V, 2}), c(colors, {(uint64_t)B, (uint64_t)V, 3});
  TensorView<float> d(sdf, {(uint64_t)V}), s(&sharpness, {1});
  TensorView<int> f(faces, {(uint64_t)F, 3}), t(tri, {(uint64_t)K});
  TensorView<int64_t> k(keys, {(uint64_t)K}), bd(bounds, {(uint64_t)B, (uint64_t)rows * cols, 2});
  TensorView<float> o(out, {(uint64_t)B, 4, (uint64_t)H, (uint64_t)W});
  run_grid_with_barriers(uint3((uint)(rows * cols * B), 1, 1), uint3(256, 1, 1), [&] {
    k_fused_16::intersect_and_composite_forward(t, bd, v, c, d, f, s, num_shells, rows, cols, o, k);
  });
}

// intersect_and_composite.py:82-147 (tile 16x16, fused layout). Gradient
// buffers are zero-filled by the caller, as torch.zeros_like there.
void ref_intersect_and_composite_backward(float* xy, float* colors, float* sdf, int B, int64_t V, int32_t* faces,
                                          int64_t F, float sharpness, int64_t* keys, int32_t* tri, int64_t K,
                                          int64_t* bounds, int num_shells, int rows, int cols, int H, int W,
                                          float* out, float* grad_out, float* grad_colors, float* grad_sdf,
                                          float* grad_sharpness) {
  TensorView<float> v(xy, {(uint64_t)B, (uint64_t)V, 2});
  DiffTensorView c(TensorView<float>(colors, {(uint64_t)B, (uint64_t)V, 3}), grad_colors);
  DiffTensorView d(TensorView<float>(sdf, {(uint64_t)V}), grad_sdf);
  DiffTensorView s(TensorView<float>(&sharpness, {1}), grad_sharpness);
  TensorView<int> f(faces, {(uint64_t)F, 3}), t(tri, {(uint64_t)K});
  TensorView<int64_t> k(keys, {(uint64_t)K}), bd(bounds, {(uint64_t)B, (uint64_t)rows * cols, 2});
  DiffTensorView o(TensorView<float>(out, {(uint64_t)B, 4, (uint64_t)H, (uint64_t)W}), grad_out);
  run_grid_with_barriers(uint3((uint)(rows * cols * B), 1, 1), uint3(256, 1, 1), [&] {
    k_fused_16::intersect_and_composite_backward(t, bd, v, c, d, f, s, num_shells, rows, cols, o, k);
  });
}

// intersect.py:50-63 (tile 16x16).
void ref_intersect(float* xy, int B, int64_t V, int32_t* faces, int64_t F, int32_t* tri, int64_t K, int64_t* bounds,
                   int S, int rows, int cols, int H, int W, float* out_uv, int32_t* out_index) {
  TensorView<float> v(xy, {(uint64_t)B, (uint64_t)V, 2});
  TensorView<int> f(faces, {(uint64_t)F, 3}), t(tri, {(uint64_t)K});
  TensorView<int64_t> bd(bounds, {(uint64_t)B, (uint64_t)S, (uint64_t)rows * cols, 2});
  TensorView<float> uv(out_uv, {(uint64_t)B * S, (uint64_t)H, (uint64_t)W, 2});
  TensorView<int> ix(out_index, {(uint64_t)B * S, (uint64_t)H, (uint64_t)W});
  run_grid_with_barriers(uint3((uint)(rows * cols * B * S), 1, 1), uint3(256, 1, 1), [&] {
    k_intersect_16::intersect(t, bd, v, f, rows, cols, H, W, uv, ix);
  });
}

// interpolate.py:40-58
void ref_interpolate(float* uv, int32_t* index, int B, int S, int H, int W, int32_t* faces, int64_t F, float* sdf,
                     float* colors, int64_t V, float* out_sdf, float* out_colors) {
  const uint64_t bs = (uint64_t)B * S;
  TensorView<float> u(uv, {bs, (uint64_t)H, (uint64_t)W, 2});
  TensorView<int> ix(index, {bs, (uint64_t)H, (uint64_t)W}), f(faces, {(uint64_t)F, 3});
  TensorView<float> d(sdf, {(uint64_t)V}), c(colors, {(uint64_t)B, (uint64_t)V, 3});
  TensorView<float> od(out_sdf, {bs, (uint64_t)H, (uint64_t)W}), oc(out_colors, {bs, (uint64_t)H, (uint64_t)W, 3});
  run_grid(uint3((W + 15) / 16, (H + 15) / 16, (uint)bs), uint3(16, 16, 1),
           [&] { k_interpolate::interpolate(u, ix, f, d, c, od, oc, S); });
}

// composite.py:36-50
void ref_composite_forward(float* sdf, float* colors, uint8_t* mask, int64_t P, int S, float sharpness,
                           float* out_colors, float* out_T) {
  TensorView<float> d(sdf, {(uint64_t)P, (uint64_t)S}), c(colors, {(uint64_t)P, (uint64_t)S, 3});
  TensorView<bool> m(reinterpret_cast<bool*>(mask), {(uint64_t)P, (uint64_t)S});
  TensorView<float> s(&sharpness, {1}), oc(out_colors, {(uint64_t)P, 3}), ot(out_T, {(uint64_t)P});
  run_grid(uint3((P + 255) / 256, 1, 1), uint3(256, 1, 1),
           [&] { k_composite::composite_forward(d, c, m, s, oc, ot); });
}

// composite.py:63-99. Gradient buffers zero-filled by the caller.
void ref_composite_backward(float* sdf, float* colors, uint8_t* mask, int64_t P, int S, float sharpness,
                            float* out_colors, float* out_T, float* grad_colors_out, float* grad_T_out,
                            float* grad_sdf, float* grad_colors, float* grad_sharpness) {
  DiffTensorView d(TensorView<float>(sdf, {(uint64_t)P, (uint64_t)S}), grad_sdf);
  DiffTensorView c(TensorView<float>(colors, {(uint64_t)P, (uint64_t)S, 3}), grad_colors);
  TensorView<bool> m(reinterpret_cast<bool*>(mask), {(uint64_t)P, (uint64_t)S});
  DiffTensorView s(TensorView<float>(&sharpness, {1}), grad_sharpness);
  DiffTensorView oc(TensorView<float>(out_colors, {(uint64_t)P, 3}), grad_colors_out);
  DiffTensorView ot(TensorView<float>(out_T, {(uint64_t)P}), grad_T_out);
  run_grid(uint3((P + 255) / 256, 1, 1), uint3(256, 1, 1),
           [&] { k_composite::composite_backward(d, c, m, s, oc, ot); });
}

}  // extern "C"
