/*
 * meshtryoshka_gb300 — C ABI of the GB300 (sm_103a) implementation of
 * Meshtryoshka's per-step render path: marching-cubes level-set extraction
 * from a sparse voxel SDF, and tile-based multi-shell triangle rasterization
 * with NeuS-style compositing (forward and backward).
 *
 * Conventions shared by every entry point:
 *   - All pointers are DEVICE pointers to dense, row-major (C-contiguous)
 *     arrays, except where a parameter is documented as host memory.
 *   - Sizes are element counts, never bytes, unless the name says "bytes".
 *   - Every call only enqueues work on `stream`; none synchronizes, and none
 *     allocates memory. Temporary storage is passed in by the caller as a
 *     `workspace` whose size is given by the matching *_workspace_bytes().
 *   - Every call returns an mt_status; MT_OK (0) means the work was enqueued.
 *   - Device-side failures (a bounded spin-wait that gave up) are recorded in
 *     the int32 status word at byte 0 of the workspace. The caller may read it
 *     after synchronizing; 0 means ok, otherwise it holds an mt_status.
 *   - float32 / int32 / int64 / uint8 are the only element types.
 *
 * Each function cites the reference interface it replaces (paths relative to
 * the reference repository dcharatan/meshtryoshka).
 */
#ifndef MESHTRYOSHKA_GB300_H
#define MESHTRYOSHKA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MT_API __attribute__((visibility("default")))
#else
#define MT_API
#endif

/* Same underlying type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* mt_stream_t;

enum mt_status {
  MT_OK = 0,
  MT_ERR_INVALID_ARGUMENT = 1,  /* bad size / pointer / parameter */
  MT_ERR_CUDA = 2,              /* a kernel launch failed */
  MT_ERR_WORKSPACE_TOO_SMALL = 3,
  MT_ERR_KEY_OVERFLOW = 4,      /* a key field does not fit its bit budget */
  MT_ERR_DEVICE_TIMEOUT = 5,    /* a bounded device spin-wait gave up */
  MT_ERR_CAPACITY = 6           /* an output buffer is smaller than needed */
};

/* Human-readable name of a status code (static string, never NULL). */
MT_API const char* mt_status_string(int status);

/* Library ABI version: (major << 16) | minor. */
MT_API int mt_version(void);

/* ------------------------------------------------------------------------
 * Scans (replace triangle_extraction/compute_exclusive_cumsum.cu:8-39, which
 * wraps cub::DeviceScan::ExclusiveSum, and the int64 torch.cumsum of
 * triangle_rasterization/generate_keys.py:48). Single-pass decoupled
 * look-back scans; in place where the reference is in place.
 * ---------------------------------------------------------------------- */

/* Bytes of workspace needed by any scan over n elements. */
MT_API size_t mt_scan_workspace_bytes(int64_t n);

/* data[0..n) <- exclusive prefix sum of data[0..n), in place. */
MT_API int mt_exclusive_scan_i32(int32_t* data, int64_t n, void* workspace,
                          size_t workspace_bytes, mt_stream_t stream);

/* data[0..n) <- exclusive prefix sum of data[0..n), in place (int64). */
MT_API int mt_exclusive_scan_i64(int64_t* data, int64_t n, void* workspace,
                          size_t workspace_bytes, mt_stream_t stream);

/* out[0..n) <- inclusive prefix sum of in[0..n), widened to int64
 * (torch.cumsum(in, dtype=torch.int64)). */
MT_API int mt_inclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n,
                                 void* workspace, size_t workspace_bytes,
                                 mt_stream_t stream);

/* ------------------------------------------------------------------------
 * Voxel extraction (triangle_extraction/__init__.py:31-62 extract_voxels).
 * Packed occupancy: int32 words [I, J, KP]; bit b of word (i, j, kp) is
 * voxel (i, j, 32*kp + b).
 * ---------------------------------------------------------------------- */

/* triangle_extraction/compute_vertex_occupancy.slang:9-68.
 * vertex_occupancy: [I+1, J+1, KP+1]; vertex_counts: (I+1)(J+1)(KP+1)+1
 * (popcount per word, last entry set to 0). */
MT_API int mt_compute_vertex_occupancy(const int32_t* occupancy, int32_t I, int32_t J,
                                int32_t KP, int32_t* vertex_occupancy,
                                int32_t* vertex_counts, mt_stream_t stream);

/* triangle_extraction/count_occupancy.slang:3-20 (+ count_occupancy.py:30).
 * voxel_counts: (I+1)(J+1)(KP+1)+1 entries; popcount of occupied words,
 * zero everywhere else. */
MT_API int mt_count_occupancy(const int32_t* occupancy, int32_t I, int32_t J,
                       int32_t KP, int32_t* voxel_counts, mt_stream_t stream);

/* triangle_extraction/create_voxels.slang:3-276. The offsets are the
 * exclusive scans of the two count arrays above, viewed as [I+1, J+1, KP+1].
 * Outputs: vertices [G,3] f32, neighbors [7,Nv], lower_corners [4,G],
 * upper_corners [4,Nv], indices [Nv] (G = num_vertices, Nv = num_voxels). */
MT_API int mt_create_voxels(const int32_t* occupancy, const int32_t* voxel_offsets,
                     const int32_t* vertex_occupancy,
                     const int32_t* vertex_offsets, int32_t I, int32_t J,
                     int32_t KP, int64_t num_voxels, int64_t num_vertices,
                     float* vertices, int32_t* neighbors,
                     int32_t* lower_corners, int32_t* upper_corners,
                     int32_t* indices, mt_stream_t stream);

/* triangle_extraction/dilate_occupancy.slang:9-94: box dilation of the packed
 * grid by `dilation` voxels (0 < dilation < 32). out must not alias in. */
MT_API int mt_dilate_occupancy(const int32_t* occupancy, int32_t I, int32_t J,
                        int32_t KP, int32_t dilation, int32_t* out,
                        mt_stream_t stream);

/* ------------------------------------------------------------------------
 * Per-step marching cubes (triangle_extraction/__init__.py:75-157
 * tessellate_voxels). G = voxels + subvoxels, Nv = voxels, S = level sets,
 * C = spherical-harmonic coefficients per colour channel.
 * ---------------------------------------------------------------------- */

/* triangle_extraction/count_triangle_vertices.slang:3-37.
 * counts: S*G+1 int32, level-set-major; the last entry is set to 0. */
MT_API int mt_count_triangle_vertices(const float* signed_distances,
                               const int32_t* lower_corners, int64_t G,
                               const float* level_sets, int32_t S,
                               int32_t* counts, mt_stream_t stream);

/* triangle_extraction/create_triangle_vertices.slang:145-199 (forward).
 * vertex_offsets: exclusive scan of the counts above (S*G+1 entries).
 * grid_sh [C,G,3]; outputs vertices [V,3], signed_distances [V],
 * spherical_harmonics [C,V,3], vertex_types [V] (uint8 axis 0/1/2). */
MT_API int mt_create_triangle_vertices(const float* grid_vertices,
                                const float* grid_signed_distances,
                                const float* grid_spherical_harmonics,
                                int32_t C, const int32_t* lower_corners,
                                int64_t G, const float* level_sets, int32_t S,
                                const int32_t* vertex_offsets, int64_t V,
                                float* vertices, float* signed_distances,
                                float* spherical_harmonics,
                                uint8_t* vertex_types, mt_stream_t stream);

/* triangle_extraction/create_triangle_vertices.slang:201-291 (backward).
 * Accumulates (+=) into grad_grid_vertices [G,3], grad_grid_signed_distances
 * [G], grad_grid_spherical_harmonics [C,G,3]; callers zero them first.
 * grad_vertices may be NULL (treated as zero). The MC weight t is detached,
 * as in the reference. */
MT_API int mt_create_triangle_vertices_backward(
    const float* grid_signed_distances, int32_t C,
    const int32_t* lower_corners, int64_t G, const float* level_sets,
    int32_t S, const int32_t* vertex_offsets, const float* grad_vertices,
    const float* grad_signed_distances, const float* grad_spherical_harmonics,
    int64_t V, float* grad_grid_vertices, float* grad_grid_signed_distances,
    float* grad_grid_spherical_harmonics, mt_stream_t stream);

/* triangle_extraction/count_triangle_faces.slang:15-50.
 * face_counts: S*Nv+1 int32 (3 x triangles; last entry 0);
 * cell_codes: [S, Nv] uint8 cube codes. */
MT_API int mt_count_triangle_faces(const float* signed_distances,
                            const int32_t* lower_corners, int64_t G,
                            const int32_t* upper_corners, int64_t Nv,
                            const float* level_sets, int32_t S,
                            int32_t* face_counts, uint8_t* cell_codes,
                            mt_stream_t stream);

/* triangle_extraction/create_triangle_faces.slang:5-78. face_offsets is the
 * exclusive scan of face_counts. Outputs faces [F,3] int32 (reversed slot
 * order as in the reference) and voxel_indices [F]. */
MT_API int mt_create_triangle_faces(const int32_t* neighbors, const int32_t* indices,
                             int64_t Nv, int64_t G,
                             const int32_t* vertex_offsets,
                             const uint8_t* vertex_types,
                             const uint8_t* cell_codes, int32_t S,
                             const int32_t* face_offsets, int64_t F,
                             int32_t* faces, int32_t* voxel_indices,
                             mt_stream_t stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* MESHTRYOSHKA_GB300_H */
