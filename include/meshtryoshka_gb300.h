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
  MT_ERR_CAPACITY = 6,          /* an output buffer is smaller than needed */
  MT_ERR_TOO_LARGE = 7          /* size exceeds a fixed static-scratch limit */
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

/* Test support for the bounded device waits (no counterpart in the
 * reference): one warp looks back from tile 1 of a scan whose tile 0 never
 * publishes, gives up after spin_limit polls (1..2^20), records
 * MT_ERR_DEVICE_TIMEOUT in the workspace status word (byte 0, as every scan
 * does) and writes the prefix it fell back to (0) to prefix_out[0] (device).
 * The workspace needs at least 272 bytes. */
MT_API int mt_test_lookback_timeout(int32_t spin_limit, int64_t* prefix_out, void* workspace,
                             size_t workspace_bytes, mt_stream_t stream);

/* Allocation-free exclusive scan (no counterpart in the reference). Same
 * result as mt_exclusive_scan_i32, for callers that cannot allocate device
 * memory for scratch: a plain C/C++ host with no device allocator of its own,
 * or code whose host framework forbids new device allocations. Its scratch is
 * a fixed 87,640-byte __device__ array inside this library, resident on
 * every GPU that loads it until the process exits. Limits: n <=
 * mt_exclusive_scan_i32_static_max_elements() (2^26); larger n returns
 * MT_ERR_TOO_LARGE. All calls on a device share the array, so calls whose
 * work overlaps on the GPU race; issue them on one stream. The first call in
 * a CUDA context (that context current) looks up the array's address and
 * caches it under the context's id, so a device reset or another context
 * gets a fresh lookup; make that first call before any stream capture in the
 * context. data and stream must belong to the current context. A look-back
 * wait that gave up leaves MT_ERR_DEVICE_TIMEOUT in the array's status word
 * (read it with mt_exclusive_scan_i32_static_status); each call clears it. */
MT_API int mt_exclusive_scan_i32_static(int32_t* data, int64_t n, mt_stream_t stream);

/* Copies the status word of the last mt_exclusive_scan_i32_static call in the
 * current context (MT_OK or MT_ERR_DEVICE_TIMEOUT, 4 bytes) to status_out,
 * device or host memory, in stream order; read host memory after the stream
 * has been synchronised. Allocates nothing. */
MT_API int mt_exclusive_scan_i32_static_status(int32_t* status_out, mt_stream_t stream);

/* Largest n accepted by mt_exclusive_scan_i32_static. */
MT_API int64_t mt_exclusive_scan_i32_static_max_elements(void);

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
 * Coarse-to-fine subdivision (meshtryoshka/model/tesseract.py:396-486).
 * ---------------------------------------------------------------------- */

/* write_occupancy.py:22-46 / write_occupancy.slang:1-20: sets bit v & 31 of
 * word v >> 5 for each of the n voxel indices (atomic OR into a caller-zeroed
 * grid of `words` int32). Indices outside [0, 32 words) are skipped. */
MT_API int mt_write_occupancy(const int32_t* voxel_indices, int64_t n,
                       int32_t* occupancy, int64_t words, mt_stream_t stream);

/* upscale_occupancy.py:24-54 / upscale_occupancy.slang:1-74: [I, J, KP] ->
 * [I2, J2, KP2] (every new extent >= the old one). `mask` (nullable, same
 * shape as `occupancy`) is AND-ed into every old word read, which is the
 * `old_occupancy & occupancy_to_upscale` of upscale_parameters.py:49. */
MT_API int mt_upscale_occupancy(const int32_t* occupancy, const int32_t* mask,
                         int32_t I, int32_t J, int32_t KP, int32_t I2,
                         int32_t J2, int32_t KP2, int32_t* out,
                         mt_stream_t stream);

/* upscale_parameters.slang:129-198 (launch at upscale_parameters.py:77-93):
 * trilinear resampling of [Vold] signed distances and [C, Vold, 3] SH from
 * the old vertex grid ([I1, J1, KP1] vertex occupancy + exclusive per-word
 * vertex offsets, as compute_vertex_occupancy + scan give) onto the new one
 * ([I1n, J1n, KP1n]); writes Vnew entries. */
MT_API int mt_upscale_parameters(
    const int32_t* old_vertex_occupancy, const int32_t* old_vertex_offsets,
    const float* old_signed_distances, const float* old_spherical_harmonics,
    int32_t C, int64_t Vold, int32_t I1, int32_t J1, int32_t KP1,
    const int32_t* new_vertex_occupancy, const int32_t* new_vertex_offsets,
    int32_t I1n, int32_t J1n, int32_t KP1n, int64_t Vnew,
    float* new_signed_distances, float* new_spherical_harmonics,
    mt_stream_t stream);

/* get_occupancy_mesh.slang:1-54 count_triangles: counts[(I+1)(J+1)(KP+1)+1]
 * int32, 2 x boundary faces owned per entry (last entry set to 0, ready for
 * an exclusive scan). */
MT_API int mt_count_occupancy_mesh_triangles(const int32_t* occupancy, int32_t I,
                                      int32_t J, int32_t KP, int32_t* counts,
                                      mt_stream_t stream);

/* get_occupancy_mesh.slang:122-220 create_triangles: writes T triangles,
 * vertices [T, 3, 3] and triangle_colors [T, 3] from colors [3, 2, 3]
 * (axis, side, rgb), at the scanned offsets. */
MT_API int mt_create_occupancy_mesh_triangles(const int32_t* occupancy, int32_t I,
                                       int32_t J, int32_t KP,
                                       const int32_t* offsets, int64_t T,
                                       const float* colors, float* vertices,
                                       float* triangle_colors,
                                       mt_stream_t stream);

/* index_vertices.py:17-21: quantized[3V] = int64(round(points * inv_tol))
 * (round half to even) and *max_abs = max |quantized| (device uint64). */
MT_API int mt_quantize_points(const float* points, int64_t V, float inv_tol,
                       int64_t* quantized, uint64_t* max_abs,
                       mt_stream_t stream);

/* index_vertices.py:23-25: keys[v] = (x << 2 shift) | (y << shift) | z,
 * values[v] = v. */
MT_API int mt_pack_point_keys(const int64_t* quantized, int64_t V, int32_t shift,
                       int64_t* keys, int32_t* values, mt_stream_t stream);

/* values[v] = v for v < n. */
MT_API int mt_iota_i32(int64_t n, int32_t* values, mt_stream_t stream);

/* index_vertices.py:30-51 index_keys, after a stable sort of (key, v):
 * out[order[p]] = order[first position of p's run of equal keys]. */
MT_API int mt_index_sorted_runs(const int64_t* sorted_keys, const int32_t* order,
                         int64_t n, int32_t* out, mt_stream_t stream);

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
 * spherical_harmonics [C,V,3], vertex_types [V] (uint8 axis 0/1/2), and
 * vertex_sources [3,V] int32: origin corner, axis corner and the float bits
 * of the (detached) weight t of every vertex. num_vertices: NULL, or a
 * device int32 (the last vertex offset); V is then the buffers' capacity
 * (the row stride of spherical_harmonics) and vertices past it are dropped.
 * spherical_harmonics NULL (grid_sh may then be NULL too): the SH rows are
 * not formed (mt_grid_sh_colors evaluates colours from the grid directly). */
MT_API int mt_create_triangle_vertices(const float* grid_vertices,
                                const float* grid_signed_distances,
                                const float* grid_spherical_harmonics,
                                int32_t C, const int32_t* lower_corners,
                                int64_t G, const float* level_sets, int32_t S,
                                const int32_t* vertex_offsets, int64_t V,
                                const int32_t* num_vertices,
                                float* vertices, float* signed_distances,
                                float* spherical_harmonics,
                                uint8_t* vertex_types, int32_t* vertex_sources,
                                mt_stream_t stream);

/* triangle_extraction/create_triangle_vertices.slang:201-291 (backward).
 * Writes (=) every entry of grad_grid_vertices [G,3] (may be NULL when
 * grad_vertices is NULL), grad_grid_signed_distances [G] and
 * grad_grid_spherical_harmonics [C,G,3]; no zero-filled outputs needed.
 * corner_inverse: scratch of 4*G int32. A NULL input gradient counts as
 * zero. The MC weight t is detached, as in the reference. workspace: see
 * mt_create_triangle_vertices_backward_workspace_bytes (may be NULL). */
MT_API int mt_create_triangle_vertices_backward(
    const float* grid_signed_distances, int32_t C,
    const int32_t* lower_corners, int64_t G, const float* level_sets,
    int32_t S, const int32_t* vertex_offsets, const float* grad_vertices,
    const float* grad_signed_distances, const float* grad_spherical_harmonics,
    int64_t V, int32_t* corner_inverse, float* grad_grid_vertices,
    float* grad_grid_signed_distances, float* grad_grid_spherical_harmonics,
    void* workspace, size_t workspace_bytes, mt_stream_t stream);

/* Opt-in live marching-cubes weight (not in the reference, which detaches t
 * at create_triangle_vertices.slang:92-96). Adds (+=) to
 * grad_grid_signed_distances [G] the gradient that flows through
 * t = (iso - d0) / (d1 - d0) when t is live: for every vertex with
 * 0 < t < 1 and d0 != d1, dL/dt = grad_vertices . (p1 - p0) +
 * sum_k grad_spherical_harmonics[k] . (sh1_k - sh0_k), scattered as
 * -dL/dt (1 - t) / (d1 - d0) to the origin corner and -dL/dt t / (d1 - d0) to
 * the axis corner. vertex_sources: the [3, V] (origin, axis corner, t bits)
 * record written by mt_create_triangle_vertices; num_vertices: optional
 * device count of live rows (NULL = V). Either gradient may be NULL. With t
 * live the vertex SDF is the level set itself, so a caller combining this
 * with mt_create_triangle_vertices_backward passes it no SDF gradient. */
MT_API int mt_create_triangle_vertices_live_t_backward(
    const float* grid_vertices, const float* grid_signed_distances,
    const float* grid_spherical_harmonics, int32_t C, int64_t G,
    const int32_t* vertex_sources, int64_t V, const int32_t* num_vertices,
    const float* grad_vertices, const float* grad_spherical_harmonics,
    float* grad_grid_signed_distances, mt_stream_t stream);

/* Workspace for mt_create_triangle_vertices_backward's list form (S <= 21:
 * per-grid-vertex contribution lists, then a coalesced SH gather). With a
 * NULL or smaller workspace the single-pass gather runs instead; both give
 * the same results. */
MT_API size_t mt_create_triangle_vertices_backward_workspace_bytes(int64_t G, int64_t V);

/* ------------------------------------------------------------------------
 * Grid SH straight to vertex colours (not in the reference, which forms the
 * per-vertex SH rows [C,V,3] in create_triangle_vertices.slang:145-199 and
 * evaluates them in evaluate_spherical_harmonics.slang:4-270; these entry
 * points give the same bits without the rows, forward and backward).
 * ---------------------------------------------------------------------- */

/* The backward of create_triangle_vertices.slang:201-291 as a gather needs,
 * per grid vertex, the list of its contributions (vertex, t, origin or axis
 * corner), enumerated in a fixed order. This builds it ahead of the
 * backward: corner_inverse [4,G] (scratch), list_offsets [G+1] (CSR offsets)
 * and list [2V, 2] int32 (vertex | origin flag << 31, float bits of t). At
 * most mt_vertex_grad_list_max_shells() level sets and V < 2^31
 * (MT_ERR_TOO_LARGE otherwise). */
MT_API int mt_vertex_grad_list_max_shells(void);
MT_API size_t mt_build_vertex_grad_list_workspace_bytes(int64_t G);
MT_API int mt_build_vertex_grad_list(const float* grid_signed_distances,
                                     const int32_t* lower_corners, int64_t G,
                                     const float* level_sets, int32_t S,
                                     const int32_t* vertex_offsets, int64_t V,
                                     int32_t* corner_inverse, int32_t* list_offsets,
                                     int32_t* list, void* workspace,
                                     size_t workspace_bytes, mt_stream_t stream);

/* create_triangle_vertices.slang:201-291 (backward) for the vertex positions
 * and signed distances from a prebuilt list: the same sums, in the same
 * order, as mt_create_triangle_vertices_backward. Every grid entry written. */
MT_API int mt_vertex_grads_from_list(const int32_t* list_offsets, const int32_t* list,
                                     int64_t G, const float* grad_vertices,
                                     const float* grad_signed_distances,
                                     float* grad_grid_vertices,
                                     float* grad_grid_signed_distances,
                                     mt_stream_t stream);

/* out_colors [B,V,3] = evaluate_spherical_harmonics(vertices, the SH rows
 * that mt_create_triangle_vertices would interpolate from grid_sh [C,G,3]
 * with vertex_sources [3,V]), rows in registers. num_vertices: NULL or the
 * device live count; rows past it are not written. */
MT_API int mt_grid_sh_colors(const float* grid_spherical_harmonics, int32_t C, int64_t G,
                             const int32_t* vertex_sources, int64_t V,
                             const int32_t* num_vertices, const float* vertices,
                             int32_t sh_degree, const float* camera_positions,
                             int32_t B, float* out_colors, mt_stream_t stream);

/* Backward of mt_grid_sh_colors: grad_grid_sh [C,G,3] (every entry written)
 * from grad_colors [B,V,3] through the list of mt_build_vertex_grad_list.
 * The per-vertex SH gradient of mt_evaluate_spherical_harmonics_backward is
 * formed once per vertex into workspace (at least
 * mt_grid_sh_colors_backward_workspace_bytes(V) bytes, 16-byte aligned) and
 * summed per grid vertex, or, with workspace NULL, on the fly per list
 * entry; either way the result equals that call followed by
 * mt_create_triangle_vertices_backward bit for bit. num_vertices: NULL or the
 * device live vertex count. */
MT_API size_t mt_grid_sh_colors_backward_workspace_bytes(int64_t V);
MT_API int mt_grid_sh_colors_backward(const int32_t* list_offsets, const int32_t* list,
                                      int64_t G, int64_t V, const float* vertices,
                                      int32_t C, int32_t sh_degree,
                                      const float* camera_positions, int32_t B,
                                      const float* out_colors, const float* grad_colors,
                                      float* grad_grid_spherical_harmonics,
                                      const int32_t* num_vertices, void* workspace,
                                      size_t workspace_bytes, mt_stream_t stream);

/* triangle_extraction/compute_sdf_regularizers.slang:18-128 (forward) and its
 * automatic derivative (backward). Per voxel: eikonal_loss_pos / _neg [Nv]
 * (squared excess / deficit of the trilinear SDF's gradient norm at the
 * voxel centre, scaled by the grid size voxel_x/y/z, over 1) and
 * curvature_loss [Nv] (squared Laplacian at the +xyz corner). The backward
 * writes (=) every entry of grad_grid_signed_distances [G]; any of the three
 * input gradients may be NULL (zero). */
MT_API int mt_compute_sdf_regularizers(
    const float* grid_signed_distances, const int32_t* voxel_neighbors,
    const int32_t* voxel_lower_corners, int64_t G, const int32_t* voxel_upper_corners,
    int64_t Nv, int32_t voxel_x, int32_t voxel_y, int32_t voxel_z,
    float* eikonal_loss_pos, float* eikonal_loss_neg, float* curvature_loss,
    mt_stream_t stream);

MT_API int mt_compute_sdf_regularizers_backward(
    const float* grid_signed_distances, const int32_t* voxel_neighbors,
    const int32_t* voxel_lower_corners, int64_t G, const int32_t* voxel_upper_corners,
    int64_t Nv, int32_t voxel_x, int32_t voxel_y, int32_t voxel_z,
    const float* grad_eikonal_loss_pos, const float* grad_eikonal_loss_neg,
    const float* grad_curvature_loss, float* grad_grid_signed_distances,
    mt_stream_t stream);

/* triangle_extraction/count_triangle_faces.slang:15-50.
 * face_counts: S*Nv+1 int32 (3 x triangles; last entry 0);
 * cell_codes: [S, Nv] uint8 cube codes. */
MT_API int mt_count_triangle_faces(const float* signed_distances,
                            const int32_t* lower_corners, int64_t G,
                            const int32_t* upper_corners, int64_t Nv,
                            const float* level_sets, int32_t S,
                            int32_t* face_counts, uint8_t* cell_codes,
                            mt_stream_t stream);

/* The shell boundaries of triangle_extraction/__init__.py:145-146 from the
 * two scanned count arrays (vertex_offsets: S*G + 1 entries, face_offsets:
 * S*Nv + 1): vertex_boundaries[s] = vertex_offsets[(s + 1) G],
 * face_boundaries[s] = face_offsets[(s + 1) Nv] / 3, and (num_faces
 * nullable) *num_faces = face_offsets[S Nv] / 3 (:131). One launch for what
 * the reference does with four tensor ops. */
MT_API int mt_shell_boundaries(const int32_t* vertex_offsets, int64_t G,
                               const int32_t* face_offsets, int64_t Nv, int32_t S,
                               int32_t* vertex_boundaries, int32_t* face_boundaries,
                               int32_t* num_faces, mt_stream_t stream);

/* Not in the reference (capacity-sized buffers of a captured step):
 * *overflow = 1 when a live count exceeds its capacity (num_vertices >
 * vertex_capacity, num_faces > face_capacity or num_keys > key_capacity;
 * a NULL count is skipped), else 0. Device scalars in, one byte out. */
MT_API int mt_capacity_overflow(const int32_t* num_vertices, int64_t vertex_capacity,
                                const int32_t* num_faces, int64_t face_capacity,
                                const int64_t* num_keys, int64_t key_capacity,
                                uint8_t* overflow, mt_stream_t stream);

/* triangle_extraction/create_triangle_faces.slang:5-78. face_offsets is the
 * exclusive scan of face_counts. Outputs faces [F,3] int32 (reversed slot
 * order as in the reference) and voxel_indices [F]. V is the length of
 * vertex_types. F and V may be capacities: faces past F are not written and
 * no vertex past V is looked up. */
MT_API int mt_create_triangle_faces(const int32_t* neighbors, const int32_t* indices,
                             int64_t Nv, int64_t G, int64_t V,
                             const int32_t* vertex_offsets,
                             const uint8_t* vertex_types,
                             const uint8_t* cell_codes, int32_t S,
                             const int32_t* face_offsets, int64_t F,
                             int32_t* faces, int32_t* voxel_indices,
                             mt_stream_t stream);


/* ------------------------------------------------------------------------
 * Key sort (triangle_rasterization/sort_keys.cu:215-270, which calls
 * cub::DeviceRadixSort::SortPairs over bits [0, 64) of int64 keys).
 * Stable LSD radix sort in SIGNED int64 key order over bits
 * [begin_bit, end_bit); keys_out/values_out must not alias the inputs.
 * ---------------------------------------------------------------------- */

MT_API size_t mt_sort_pairs_workspace_bytes(int64_t n);

/* n is the capacity of the buffers (and sizes the workspace). count: NULL,
 * or a device int64 holding how many leading pairs to sort (clamped to n);
 * with a device count the sort makes no host synchronisation and can be
 * captured in a CUDA graph. Outputs past the count are left unchanged. */
MT_API int mt_sort_pairs_i64_i32(const int64_t* keys_in, const int32_t* values_in,
                                 int64_t* keys_out, int32_t* values_out, int64_t n,
                                 const int64_t* count, int32_t begin_bit,
                                 int32_t end_bit, void* workspace,
                                 size_t workspace_bytes, mt_stream_t stream);

/* ------------------------------------------------------------------------
 * Rasterization front end. B = cameras, V = triangle vertices, F = faces.
 * Key layout arrays are int32[7]: camera offset, camera length, shell
 * offset, shell length, tile offset, tile length, depth offset (depth is
 * always 32 bits); see triangle_rasterization/keys.py:4-22.
 * ---------------------------------------------------------------------- */

/* inverse(extrinsics)[:, :3, 3] (evaluate_spherical_harmonics.py:38).
 * extrinsics [B,4,4] world->camera; out [B,3]. */
MT_API int mt_camera_positions(const float* extrinsics, int32_t B, float* out,
                               mt_stream_t stream);

/* triangle_rasterization/project_vertices.slang:51-92.
 * out_xy [B,V,2] pixels (unnormalised, no +0.5), out_depth [B,V]. */
MT_API int mt_project_vertices(const float* vertices, int64_t V,
                               const float* extrinsics, const float* intrinsics,
                               int32_t B, float* out_xy, float* out_depth,
                               mt_stream_t stream);

/* triangle_rasterization/evaluate_spherical_harmonics.slang:187-228.
 * spherical_harmonics [C,V,3] (C >= (sh_degree+1)^2), camera_positions [B,3],
 * out_colors [B,V,3] = max(SH(dir) + 0.5, 0). */
MT_API int mt_evaluate_spherical_harmonics(const float* vertices, int64_t V,
                                           const float* spherical_harmonics,
                                           int32_t C, int32_t sh_degree,
                                           const float* camera_positions, int32_t B,
                                           float* out_colors, mt_stream_t stream);

/* evaluate_spherical_harmonics.slang:230-270 (backward to the SH only).
 * Writes (=) every entry of grad_spherical_harmonics [C,V,3]; rows beyond
 * (sh_degree+1)^2 are zero. */
MT_API int mt_evaluate_spherical_harmonics_backward(
    const float* vertices, int64_t V, int32_t C, int32_t sh_degree,
    const float* camera_positions, int32_t B, const float* out_colors,
    const float* grad_colors, float* grad_spherical_harmonics, mt_stream_t stream);

/* triangle_rasterization/bound_triangles.slang:144-192.
 * out_min / out_max [B,F,2] (row, col) tile bounds [min, max); out_count
 * [B,F] = tiles touched (0 for back-facing or near-plane-culled faces).
 * num_faces: NULL, or a device int32; rows at or past it touch no tile (F is
 * then the capacity). A face naming a vertex outside [0, V) touches no tile.
 * cameras: NULL, or the ragged camera table of the compositing entry points
 * (each camera clamps to its own rows x cols grid). */
MT_API int mt_bound_triangles(const float* xy, const float* depth, int64_t V,
                              const int32_t* faces, int64_t F,
                              const int32_t* num_faces, int32_t B,
                              int32_t tile_h, int32_t tile_w, int32_t rows,
                              int32_t cols, const int64_t* cameras,
                              float near_plane, int32_t* out_min,
                              int32_t* out_max, int32_t* out_count,
                              mt_stream_t stream);

/* triangle_rasterization/generate_keys.slang:4-68. offsets [B*F] is the
 * inclusive int64 prefix sum of out_count; K = offsets[B*F-1]. Writes one
 * key per (camera, face, tile) in (camera, face, row, col) order. cameras:
 * NULL (tile = row * grid_width + col), or the ragged camera table (each
 * camera's own grid width). */
MT_API int mt_generate_keys(const float* depth, int64_t V, const int32_t* faces,
                            int64_t F, const int32_t* shell_face_boundaries,
                            int32_t S, const int32_t* tile_min,
                            const int32_t* tile_max, const int64_t* offsets,
                            int32_t B, int32_t grid_width, const int64_t* cameras,
                            const int32_t* layout, int64_t K, int64_t* out_keys,
                            int32_t* out_triangles, mt_stream_t stream);

/* mt_bound_triangles + the int64 inclusive scan of its counts +
 * mt_generate_keys, for callers that give a key capacity K instead of reading
 * the key count back (replaces the chain
 * triangle_rasterization/__init__.py:218-236 when nothing may synchronise,
 * e.g. inside a CUDA graph). Three kernels: tile rectangles and per-chunk key
 * counts, a scan of the chunk counts, keys.
 * The keys written, and their order, equal the three-stage chain's; keys past
 * K are dropped. *out_num_keys (device int64) receives the live key count,
 * which may exceed K. xy must be 8-byte aligned. workspace (16-byte
 * aligned): at least mt_bound_and_generate_keys_workspace_bytes(B * F) bytes
 * (about 20 bytes per item; it holds each item's tile rectangle and key depth
 * between the kernels). */
MT_API size_t mt_bound_and_generate_keys_workspace_bytes(int64_t items);
MT_API int mt_bound_and_generate_keys(
    const float* xy, const float* depth, int64_t V, const int32_t* faces,
    int64_t F, const int32_t* num_faces, const int32_t* shell_face_boundaries,
    int32_t S, int32_t B, int32_t tile_h, int32_t tile_w, int32_t rows,
    int32_t cols, const int64_t* cameras, float near_plane,
    const int32_t* layout, int64_t K, int64_t* out_keys, int32_t* out_triangles,
    int64_t* out_num_keys, void* workspace, size_t workspace_bytes,
    mt_stream_t stream);

/* triangle_rasterization/delineate_tiles.slang:14-58 (+ the zero fill of
 * delineate_tiles.py:40, done here). out_boundaries [B, shell_dim,
 * num_tiles, 2] int64; shell_dim = S when separate_shells, else 1.
 * num_keys: NULL (all K keys), or a device int64 count of live keys. */
MT_API int mt_delineate_tiles(const int64_t* sorted_keys, int64_t K,
                              const int64_t* num_keys,
                              const int32_t* layout, int32_t separate_shells,
                              int32_t B, int32_t shell_dim, int64_t num_tiles,
                              int64_t* out_boundaries, mt_stream_t stream);

/* sort_keys.cu:241-267 (stable signed-key sort) followed by
 * delineate_tiles.slang:14-58, for keys made by mt_generate_keys: keys are
 * counted and scattered into their (camera, [shell,] tile) bins and each bin
 * is sorted by its low key bits and original index, which gives the stable
 * sort's order. Same outputs as mt_sort_pairs_i64_i32 + mt_delineate_tiles.
 * Applicable when mt_sort_keys_by_tile_supported() returns 1 (the key
 * layout is the fused or explicit one, no camera sets the key's sign bit,
 * and the composite of low bits and index fits in 63 bits). Part of the work
 * runs on a helper stream that this library keeps per (device, stream); it
 * is forked from `stream` and joined back to it with events, so the outputs
 * are ordered on `stream` as usual (and the call can be graph-captured once
 * it has run on that stream outside capture). */
MT_API int mt_sort_keys_by_tile_supported(const int32_t* layout, int32_t separate_shells,
                                   int32_t B, int64_t K);
MT_API size_t mt_sort_keys_by_tile_workspace_bytes(int64_t K, int64_t num_bins);
MT_API int mt_sort_keys_by_tile(const int64_t* keys, const int32_t* triangles, int64_t K,
                         const int64_t* num_keys, const int32_t* layout,
                         int32_t separate_shells, int32_t B, int32_t shell_dim,
                         int64_t num_tiles, int64_t* sorted_keys,
                         int32_t* sorted_triangles, int64_t* out_boundaries,
                         void* workspace, size_t workspace_bytes, mt_stream_t stream);

/* ------------------------------------------------------------------------
 * Fused multi-shell compositing
 * (triangle_rasterization/intersect_and_composite.slang:224-564).
 * xy [B,V,2], colors [B,V,3], signed_distances [V], faces [F,3],
 * sharpness: device scalar; sorted keys / triangles [K]; tile_boundaries
 * [B, rows*cols, 2]; layout: host int32[7] key layout (as mt_generate_keys);
 * out [B,4,H,W] = (rgb, transmittance). One CTA of tile_h*tile_w (<= 1024)
 * threads per (camera, tile); its warps work independently.
 * warp_masks [K] uint32 is scratch written by the forward (per key, the warps
 * of its tile the triangle can cover) and read by the backward.
 * num_keys: NULL (all K keys live), or a device int64 count of live keys
 * (K is then the capacity of the key buffers).
 * Cameras of different sizes (not in the reference): cameras = NULL (every
 * camera rows x cols tiles of H x W pixels, out [B,4,H,W]), or a device table
 * int64 [B, 6] = (rows, cols, height, width, first tile, first output
 * element) per camera, with camera_tiles = the total of rows x cols over
 * cameras; each camera's output is then [4, height, width] at its first
 * output element, tile_boundaries stay [B, rows*cols, 2] with rows / cols /
 * H / W the maxima, and keys carry the camera-local tile index.
 * work_counter: one uint64 of device scratch (reset here): the kernel's
 * persistent warps pull (camera, tile, warp) work items from it.
 * Optional MSE epilogue (not in the reference, where the trainer blends,
 * clips and takes the loss with separate tensor ops): with target != NULL
 * ([B,3,H,W], or each camera's [3,h,w] back to back for ragged cameras) and
 * background [3], the forward also sets the device scalar *loss_sum =
 * loss_scale x sum over pixels and channels of
 * (clip(rgb + T * background, 0, 1) - target)^2, and the backward takes
 * d L / d loss from the device scalar grad_loss instead of grad_out.
 * hit_bits (not in the reference; NULL = off): a hit-bit store of
 * hit_bits_bytes bytes, 128-byte aligned; mt_composite_hit_bits_bytes gives
 * the size that holds a number of batches. Each warp work item of the
 * forward counts the keys it will walk, reserves ceil(count / 32) batches of
 * the store and writes, per batch, the bits of the triangles each of its
 * pixels hits, as long as the store has room (a 128-byte line per batch); a
 * backward on the same inputs given the same buffer reads them instead of
 * testing those batches again, and tests the rest (same bits, same
 * gradients). Batches for K keys never exceed
 * K * ceil(tile_h * tile_w / 32) / 32 + camera_tiles * ceil(tile_h * tile_w / 32).
 * camera_tiles: the total tiles over cameras (B * rows * cols for a uniform
 * grid). cta_threads (not in the reference, which runs one tile of
 * TILE_H x TILE_W threads per CTA): 128, 256 or 512 threads per CTA of
 * persistent warps (0 = 256); the results do not depend on it.
 * ---------------------------------------------------------------------- */
MT_API size_t mt_composite_hit_bits_bytes(int64_t camera_tiles, int32_t tile_h, int32_t tile_w,
                                          int64_t batches);

MT_API int mt_intersect_and_composite_forward(
    const float* xy, const float* colors, const float* signed_distances, int64_t V,
    const int32_t* faces, const float* sharpness, const int64_t* sorted_keys,
    const int32_t* sorted_triangles, int64_t K, const int64_t* num_keys,
    const int64_t* tile_boundaries, int32_t B, int32_t num_shells, int32_t rows,
    int32_t cols, int32_t tile_h, int32_t tile_w, int32_t H, int32_t W,
    const int32_t* layout, const int64_t* cameras, int64_t camera_tiles,
    uint32_t* warp_masks, uint64_t* work_counter, float* out, const float* target,
    const float* background, float loss_scale, float* loss_sum, void* hit_bits, size_t hit_bits_bytes,
    int32_t* tile_order, size_t tile_order_bytes, int32_t cta_threads, mt_stream_t stream);

/* Backward: accumulates (+=) into grad_colors [B,V,3], grad_signed_distances
 * [V], grad_sharpness [1]. warp_masks as written by the forward call on the
 * same keys. ssaa (1 = none): with ssaa > 1 (uniform cameras, H and W
 * multiples of ssaa) target is the factor written by mt_ssaa_loss and every
 * sub-pixel takes 1 / ssaa^2 of its output pixel's d L / d image.
 * staging (not in the reference; NULL = off), 128-byte aligned, of at least
 * mt_composite_staging_bytes(B, V) bytes: the backward packs every (camera,
 * vertex) into a 32-byte record there, and each warp brings the vertex
 * records of its next batch of triangles into shared memory with bulk copies
 * (cp.async.bulk on an mbarrier) while it composites the current batch;
 * same gradients. A bounded wait that gives up leaves MT_ERR_DEVICE_TIMEOUT
 * in the staging status word. exact_adjoint = 0 reproduces the reference's gradient routing
 * (the outer hit's deferred gradient is scattered with the current hit's
 * barycentric weights); 1 uses the outer hit's own weights. */
MT_API int mt_intersect_and_composite_backward(
    const float* xy, const float* colors, const float* signed_distances, int64_t V,
    const int32_t* faces, const float* sharpness, const int64_t* sorted_keys,
    const int32_t* sorted_triangles, int64_t K, const int64_t* tile_boundaries,
    int32_t B, int32_t num_shells, int32_t rows, int32_t cols, int32_t tile_h,
    int32_t tile_w, int32_t H, int32_t W, const int32_t* layout,
    const int64_t* cameras, int64_t camera_tiles, const uint32_t* warp_masks,
    uint64_t* work_counter, const float* out, const float* grad_out,
    const float* target, const float* background, float loss_scale,
    const float* grad_loss, int32_t ssaa, float* grad_colors, float* grad_signed_distances,
    float* grad_sharpness, int32_t exact_adjoint, const void* hit_bits, size_t hit_bits_bytes,
    void* staging, size_t staging_bytes, const int32_t* tile_order, size_t tile_order_bytes,
    int32_t cta_threads, mt_stream_t stream);

/* Bytes of the optional tile order of the compositing kernels (not in the
 * reference, whose CTAs take tiles in grid order): int32 bucket counts and
 * cursors, then one global tile index per tile (camera_tiles of them). With
 * a tile order the forward sorts the tiles by descending key count (buckets
 * of 8 keys) and its persistent warps take the tiles' work items in that
 * order, so the few expensive tiles start first instead of last; the
 * backward, given the same buffer after the forward on the same keys, takes
 * the items in the same order. NULL: launch order. Results do not depend on
 * the order (the gradients' atomic sums may round in another order). */
MT_API size_t mt_composite_tile_order_bytes(int64_t camera_tiles);

/* Bytes of the backward's optional staging scratch for B cameras and V
 * vertices: a 128-byte header (a device status word at byte 0) and one
 * 32-byte record (x, y, r, g, b, signed distance) per (camera, vertex). */
MT_API size_t mt_composite_staging_bytes(int32_t B, int64_t V);

/* MSE epilogue with SSAA (not in the reference, where the trainer applies
 * triangle_rasterization/__init__.py:274-287 and the loss as tensor ops):
 * raw [B,4,H,W] compositing output at the supersampled size; per output
 * pixel of [B,3,H/ssaa,W/ssaa], the mean of rgb + T * background over its
 * ssaa x ssaa sub-pixels, clipped to [0,1], against target. Sets the device
 * scalar *loss = loss_scale x sum of squared errors and writes factor
 * [B,3,H/ssaa,W/ssaa] = 2 (image - target) where the clip passes the
 * gradient (else 0), for the compositing backward's ssaa mode. */
MT_API int mt_ssaa_loss(const float* raw, int32_t B, int32_t H, int32_t W, int32_t ssaa,
                        const float* background, const float* target, float loss_scale, float* loss,
                        float* factor, mt_stream_t stream);

/* ------------------------------------------------------------------------
 * Explicit mode (triangle_rasterization/__init__.py:22-164).
 * ---------------------------------------------------------------------- */

/* intersect.slang:86-182: first hit per (camera, shell, pixel).
 * tile_boundaries [B,S,rows*cols,2]; out_uv [B*S,H,W,2]; out_index
 * [B*S,H,W] (-1 = miss, uv = 0). */
MT_API int mt_intersect(const float* xy, int64_t V, const int32_t* faces,
                        const int32_t* sorted_triangles,
                        const int64_t* tile_boundaries, int32_t B, int32_t S,
                        int32_t rows, int32_t cols, int32_t tile_h, int32_t tile_w,
                        int32_t H, int32_t W, float* out_uv, int32_t* out_index,
                        mt_stream_t stream);

/* interpolate.slang:22-76: out_signed_distances [B*S,H,W], out_colors
 * [B*S,H,W,3] with weights (u, v, 1-u-v); misses are 0. */
MT_API int mt_interpolate(const float* uv, const int32_t* index, int32_t B,
                          int32_t S, int32_t H, int32_t W, const int32_t* faces,
                          const float* signed_distances, const float* colors,
                          int64_t V, float* out_signed_distances,
                          float* out_colors, mt_stream_t stream);

/* Backward of mt_interpolate; accumulates (+=) into grad_signed_distances [V]
 * and grad_colors [B,V,3]. Either grad_out pointer may be NULL (zero). */
MT_API int mt_interpolate_backward(const float* uv, const int32_t* index,
                                   int32_t B, int32_t S, int32_t H, int32_t W,
                                   const int32_t* faces, int64_t V,
                                   const float* grad_out_signed_distances,
                                   const float* grad_out_colors,
                                   float* grad_signed_distances,
                                   float* grad_colors, mt_stream_t stream);

/* composite.slang:60-120: signed_distances [P,S], colors [P,S,3], mask [P,S]
 * (bytes, non-zero = hit) -> out_colors [P,3], out_transmittances [P]. */
MT_API int mt_composite(const float* signed_distances, const float* colors,
                        const uint8_t* mask, int64_t P, int32_t S,
                        const float* sharpness, float* out_colors,
                        float* out_transmittances, mt_stream_t stream);

/* composite.slang:122-218; accumulates (+=) into grad_signed_distances [P,S],
 * grad_colors [P,S,3], grad_sharpness [1]. exact_adjoint = 0 reproduces the
 * reference's slot routing (shell_index - 1, and num_shells - 1 for the
 * last hit); 1 routes to the previous / last hit shell. */
MT_API int mt_composite_backward(const float* signed_distances, const float* colors,
                                 const uint8_t* mask, int64_t P, int32_t S,
                                 const float* sharpness, const float* out_colors,
                                 const float* out_transmittances,
                                 const float* grad_out_colors,
                                 const float* grad_out_transmittances,
                                 float* grad_signed_distances, float* grad_colors,
                                 float* grad_sharpness, int32_t exact_adjoint,
                                 mt_stream_t stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* MESHTRYOSHKA_GB300_H */
