// Fused multi-shell intersect + composite, forward and backward, for sm_103a.
//
// Follows triangle_rasterization/intersect_and_composite.slang:1-564. One CTA
// per (camera, tile), one thread per pixel. Each tile's depth-sorted triangle
// list is staged through shared memory in chunks of up to 256 triangles; the
// staging thread computes the triangle-only part of the barycentric solve
// (edge vectors, the six edge dot products, the chosen denominator) once,
// with the same operations the per-pixel formula uses, so every per-pixel
// result is bit-identical to evaluating the full formula per pixel.
//
// Work reduction without changing any decision:
//   * warps cover compact 8x4 pixel blocks and build, per chunk, a compacted
//     list (ballot + popcount) of the triangles whose conservative accept box
//     overlaps their pixels (bary.cuh: cull_box);
//   * per pixel, the three barycentric numerators reject most remaining
//     triangles before any division (bary.cuh: hit_test).
//
// Backward re-walks the list, recomputes hits and applies the suffix trick
// of the reference. Per-triangle gradients are summed in shared memory per
// chunk (12 floats per staged triangle) and flushed with one global atomic
// per non-zero scalar; gradients for triangles of an earlier chunk go to
// global memory directly. Two routings:
//   reference (exact_adjoint = 0): the deferred gradient of the previous
//     (outer) hit is scattered to the previous triangle's vertices with the
//     *current* hit's barycentric weights (intersect_and_composite.slang:
//     487-509), as the reference does;
//   exact (exact_adjoint = 1): with the previous hit's own weights.
// The sharpness gradient is reduced per CTA before one global atomic.

#include "bary.cuh"
#include "mt_common.cuh"

namespace mt {
namespace {

constexpr int kMaxChunk = 256;

struct TriAttr {
  float ca[3], cb[3], cc[3];
  float sa, sb, sc;
};

struct CompositeArgs {
  const float* xy;      // [B, V, 2]
  const float* colors;  // [B, V, 3]
  const float* sdf;     // [V]
  int64_t V;
  const int32_t* faces;  // [F, 3]
  const float* sharpness;
  const uint64_t* keys;   // sorted keys
  const int32_t* tri;     // sorted triangle indices
  const int64_t* bounds;  // [B, T, 2]
  int B, S, rows, cols, tile_h, tile_w, H, W;
  int shell_off, shell_len;
  const float* out;  // forward output [B, 4, H, W] (input to backward)
};

struct CompositeGrads {
  const float* grad_out;  // [B, 4, H, W]
  float* grad_colors;     // [B, V, 3]
  float* grad_sdf;        // [V]
  float* grad_sharpness;  // [1]
  int exact;
};

// Shared-memory carve-up for one chunk of `chunk` staged triangles.
struct Smem {
  TriGeom* geo;
  TriAttr* attr;
  CullBox* box;
  int3* vids;        // backward only
  float* gslot;      // backward only: [chunk][12]
  uint8_t* wlist;    // [warps][chunk]
};

__device__ __forceinline__ Smem carve(void* base, int chunk, int warps, bool backward) {
  char* p = static_cast<char*>(base);
  Smem s;
  s.geo = reinterpret_cast<TriGeom*>(p);
  p += sizeof(TriGeom) * chunk;
  s.attr = reinterpret_cast<TriAttr*>(p);
  p += sizeof(TriAttr) * chunk;
  s.box = reinterpret_cast<CullBox*>(p);
  p += sizeof(CullBox) * chunk;
  s.vids = nullptr;
  s.gslot = nullptr;
  if (backward) {
    s.vids = reinterpret_cast<int3*>(p);
    p += sizeof(int3) * chunk;
    s.gslot = reinterpret_cast<float*>(p);
    p += sizeof(float) * 12 * chunk;
  }
  s.wlist = reinterpret_cast<uint8_t*>(p);
  return s;
}

size_t smem_bytes(int chunk, int warps, bool backward) {
  size_t b = (sizeof(TriGeom) + sizeof(TriAttr) + sizeof(CullBox)) * (size_t)chunk;
  if (backward) b += (sizeof(int3) + 12 * sizeof(float)) * (size_t)chunk;
  return b + (size_t)warps * chunk;
}

// Stages triangle `k` of the sorted list into slot `slot`.
__device__ __forceinline__ void stage(const CompositeArgs& a, int cam, int64_t k, const Smem& sm, int slot) {
  const int32_t f = __ldg(a.tri + k);
  const uint64_t key = __ldg(reinterpret_cast<const unsigned long long*>(a.keys) + k);
  const int32_t ia = __ldg(a.faces + 3 * (int64_t)f), ib = __ldg(a.faces + 3 * (int64_t)f + 1),
                ic = __ldg(a.faces + 3 * (int64_t)f + 2);
  const float2* xy = reinterpret_cast<const float2*>(a.xy) + (int64_t)cam * a.V;
  const float2 pa = __ldg(xy + ia), pb = __ldg(xy + ib), pc = __ldg(xy + ic);
  TriGeom g;
  setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, g);
  g.shell = (int)((key >> a.shell_off) & (uint64_t)((1u << a.shell_len) - 1u));
  sm.geo[slot] = g;
  sm.box[slot] = cull_box(g, pa.x, pa.y, pb.x, pb.y, pc.x, pc.y);
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
  sm.attr[slot] = t;
  if (sm.vids) sm.vids[slot] = make_int3(ia, ib, ic);
}

// Builds this warp's list of staged triangles whose accept box overlaps the
// warp's pixels; returns its length.
__device__ __forceinline__ int build_warp_list(const Smem& sm, int n, int chunk, int warp, int lane, float rx0,
                                               float rx1, float ry0, float ry1) {
  uint8_t* list = sm.wlist + warp * chunk;
  int count = 0;
  for (int base = 0; base < n; base += 32) {
    const int i = base + lane;
    const bool keep = i < n && box_overlaps(sm.box[i], rx0, rx1, ry0, ry1);
    const uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (keep) list[count + __popc(m & lanemask_lt())] = (uint8_t)i;
    count += __popc(m);
  }
  __syncwarp();
  return count;
}

struct PixelSetup {
  int cam;
  int64_t tile;
  int px, py;
  bool in_image;
  float fx, fy;
  float rx0, rx1, ry0, ry1;
};

__device__ __forceinline__ PixelSetup setup_pixel(const CompositeArgs& a) {
  PixelSetup p;
  const int64_t T = (int64_t)a.rows * a.cols;
  p.tile = blockIdx.x % T;
  p.cam = (int)(blockIdx.x / T);
  const int tid = threadIdx.x;
  const int numel = a.tile_h * a.tile_w;
  int lx = 0, ly = 0;
  tile_pixel(tid, a.tile_w, a.tile_h, lx, ly);
  const bool in_tile = tid < numel;
  p.px = (int)(p.tile % a.cols) * a.tile_w + lx;
  p.py = (int)(p.tile / a.cols) * a.tile_h + ly;
  p.in_image = in_tile && p.px < a.W && p.py < a.H;
  p.fx = (float)p.px + 0.5f;
  p.fy = (float)p.py + 0.5f;
  const float nan = __int_as_float(0x7fffffff);
  warp_rect(in_tile ? p.fx : nan, in_tile ? p.fy : nan, p.rx0, p.rx1, p.ry0, p.ry1);
  return p;
}

template <int kMaxThreads>
__global__ void __launch_bounds__(kMaxThreads) composite_forward_kernel(CompositeArgs a, float* __restrict__ out) {
  extern __shared__ float4 smem_f4[];
  const int bs = blockDim.x;
  const int chunk = bs < kMaxChunk ? bs : kMaxChunk;
  const Smem sm = carve(smem_f4, chunk, bs >> 5, false);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const PixelSetup px = setup_pixel(a);
  const int64_t T = (int64_t)a.rows * a.cols;
  const float s = *a.sharpness;

  float acc[3] = {0.f, 0.f, 0.f};
  float T_ = 1.0f;
  bool active = px.in_image;
  int last_shell = -1;
  float e_dummy;
  float outer_cdf = sdf_to_cdf(1e10f, s, e_dummy);  // dummy outer sample

  const int64_t start = a.bounds[2 * ((int64_t)px.cam * T + px.tile)];
  const int64_t end = a.bounds[2 * ((int64_t)px.cam * T + px.tile) + 1];
  for (int64_t c0 = start; c0 < end; c0 += chunk) {
    if (__syncthreads_count(active) == 0) break;
    const int n = (int)min((int64_t)chunk, end - c0);
    if (tid < n) stage(a, px.cam, c0 + tid, sm, tid);
    __syncthreads();
    const int len = build_warp_list(sm, n, chunk, warp, lane, px.rx0, px.rx1, px.ry0, px.ry1);
    if (active) {
      const uint8_t* list = sm.wlist + warp * chunk;
      for (int j = 0; j < len; ++j) {
        const int i = list[j];
        const TriGeom& g = sm.geo[i];
        if (g.shell <= last_shell) continue;
        float u, v, w;
        if (!hit_test(g, px.fx, px.fy, u, v, w)) continue;
        const TriAttr& t = sm.attr[i];
        const float sdf_in = interp(u, v, w, t.sa, t.sb, t.sc);
        float e_in;
        const float inner_cdf = sdf_to_cdf(sdf_in, s, e_in);
        const float alpha = clamp01(alpha_raw(outer_cdf, inner_cdf));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float rgb = interp(u, v, w, t.ca[c], t.cb[c], t.cc[c]);
          acc[c] = __fmaf_rn(__fmul_rn(rgb, T_), alpha, acc[c]);
        }
        T_ = __fmul_rn(T_, __fsub_rn(1.0f, alpha));
        outer_cdf = inner_cdf;
        last_shell = g.shell;
        if (last_shell == a.S - 1) {
          active = false;
          break;
        }
      }
    }
  }
  if (px.in_image) {
    const int64_t plane = (int64_t)a.H * a.W;
    float* o = out + (int64_t)px.cam * 4 * plane + (int64_t)px.py * a.W + px.px;
    o[0] = acc[0];
    o[plane] = acc[1];
    o[2 * plane] = acc[2];
    o[3 * plane] = T_;
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

template <int kMaxThreads>
__global__ void __launch_bounds__(kMaxThreads) composite_backward_kernel(CompositeArgs a, CompositeGrads gr) {
  extern __shared__ float4 smem_f4[];
  __shared__ float s_red[32];
  const int bs = blockDim.x;
  const int chunk = bs < kMaxChunk ? bs : kMaxChunk;
  const Smem sm = carve(smem_f4, chunk, bs >> 5, true);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const PixelSetup px = setup_pixel(a);
  const int64_t T = (int64_t)a.rows * a.cols;
  const float s = *a.sharpness;
  const int cam = px.cam;

  float final_rgb[3] = {0.f, 0.f, 0.f}, dL_rgb[3] = {0.f, 0.f, 0.f};
  float final_T = 0.f, dL_T = 0.f;
  if (px.in_image) {
    const int64_t plane = (int64_t)a.H * a.W;
    const int64_t o = (int64_t)cam * 4 * plane + (int64_t)px.py * a.W + px.px;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      final_rgb[c] = a.out[o + c * plane];
      dL_rgb[c] = gr.grad_out[o + c * plane];
    }
    final_T = a.out[o + 3 * plane];
    dL_T = gr.grad_out[o + 3 * plane];
  }
  for (int i = tid; i < chunk * 12; i += bs) sm.gslot[i] = 0.f;

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
  int64_t prev_k = -1;
  int3 prev_vid = make_int3(0, 0, 0);
  float pu = 0.f, pv = 0.f, pw = 0.f;

  const int64_t start = a.bounds[2 * ((int64_t)cam * T + px.tile)];
  const int64_t end = a.bounds[2 * ((int64_t)cam * T + px.tile) + 1];
  for (int64_t c0 = start; c0 < end; c0 += chunk) {
    if (__syncthreads_count(active) == 0) break;
    const int n = (int)min((int64_t)chunk, end - c0);
    if (tid < n) stage(a, cam, c0 + tid, sm, tid);
    __syncthreads();
    const int len = build_warp_list(sm, n, chunk, warp, lane, px.rx0, px.rx1, px.ry0, px.ry1);
    if (active) {
      const uint8_t* list = sm.wlist + warp * chunk;
      for (int j = 0; j < len; ++j) {
        const int i = list[j];
        const TriGeom& g = sm.geo[i];
        if (g.shell <= last_shell) continue;
        float u, v, w;
        if (!hit_test(g, px.fx, px.fy, u, v, w)) continue;
        const TriAttr& t = sm.attr[i];
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
          acc[c] = __fmaf_rn(weight, rgb, acc[c]);
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
          if (prev_k >= c0)
            scatter_slot(sm.gslot + 12 * (prev_k - c0), su, sv, sw, dp_rgb, dp_sdf);
          else
            scatter_global(a, gr, cam, prev_vid, su, sv, sw, dp_rgb, dp_sdf);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) dp_rgb[c] = d_color[c];
        dp_sdf = d_ic * ki * s;
        prev_k = c0 + i;
        prev_vid = sm.vids[i];
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
    // Flush this chunk's per-triangle sums (thread t owns slot t).
    __syncthreads();
    if (tid < n) {
      float* slot = sm.gslot + 12 * tid;
      const int3 vid = sm.vids[tid];
      const int id[3] = {vid.x, vid.y, vid.z};
      float* gc = gr.grad_colors + (int64_t)cam * a.V * 3;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float x = slot[4 * q + c];
          if (x != 0.f) atomicAdd(gc + 3 * (int64_t)id[q] + c, x);
          slot[4 * q + c] = 0.f;
        }
        const float y = slot[4 * q + 3];
        if (y != 0.f) atomicAdd(gr.grad_sdf + id[q], y);
        slot[4 * q + 3] = 0.f;
      }
    }
  }
  if (px.in_image && last_shell != -1) scatter_global(a, gr, cam, prev_vid, pu, pv, pw, dp_rgb, dp_sdf);

  // Block reduction of the sharpness gradient, one atomic per CTA.
  float x = px.in_image ? d_sharp : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if (lane == 0) s_red[warp] = x;
  __syncthreads();
  if (tid < 32) {
    const int nw = bs >> 5;
    float y = tid < nw ? s_red[tid] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    if (tid == 0 && y != 0.f) atomicAdd(gr.grad_sharpness, y);
  }
}

int check_args(const CompositeArgs& a) {
  if (a.B < 0 || a.S < 1 || a.rows < 0 || a.cols < 0 || a.tile_h < 1 || a.tile_w < 1 || a.H < 0 || a.W < 0)
    return MT_ERR_INVALID_ARGUMENT;
  if ((int64_t)a.tile_h * a.tile_w > 1024) return MT_ERR_INVALID_ARGUMENT;
  if ((int64_t)a.rows * a.tile_h < a.H || (int64_t)a.cols * a.tile_w < a.W) return MT_ERR_INVALID_ARGUMENT;
  if (a.shell_len < 1 || a.shell_len > 31 || a.shell_off < 0 || a.shell_off + a.shell_len > 64)
    return MT_ERR_INVALID_ARGUMENT;
  return MT_OK;
}

inline int block_threads(const CompositeArgs& a) { return (a.tile_h * a.tile_w + 31) / 32 * 32; }

template <typename K>
int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
      return MT_ERR_CUDA;
  }
  return MT_OK;
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

int mt_intersect_and_composite_forward(const float* xy, const float* colors, const float* signed_distances,
                                       int64_t V, const int32_t* faces, const float* sharpness,
                                       const int64_t* sorted_keys, const int32_t* sorted_triangles,
                                       const int64_t* tile_boundaries, int32_t B, int32_t num_shells,
                                       int32_t rows, int32_t cols, int32_t tile_h, int32_t tile_w, int32_t H,
                                       int32_t W, int32_t shell_bit_offset, int32_t shell_bit_length,
                                       float* out, mt_stream_t stream) {
  CompositeArgs a{xy, colors, signed_distances, V, faces, sharpness,
                  reinterpret_cast<const uint64_t*>(sorted_keys), sorted_triangles, tile_boundaries,
                  B, num_shells, rows, cols, tile_h, tile_w, H, W, shell_bit_offset, shell_bit_length, nullptr};
  int rc = check_args(a);
  if (rc != MT_OK) return rc;
  const int64_t blocks = (int64_t)B * rows * cols;
  if (blocks == 0 || H == 0 || W == 0) return MT_OK;
  MT_REQUIRE(xy && colors && signed_distances && faces && sharpness && tile_boundaries && out);
  MT_REQUIRE(blocks < ((int64_t)1 << 31));
  const int bs = block_threads(a);
  const int chunk = bs < kMaxChunk ? bs : kMaxChunk;
  const size_t smem = smem_bytes(chunk, bs / 32, false);
  if (bs <= 256) {
    rc = set_smem(composite_forward_kernel<256>, smem);
    if (rc != MT_OK) return rc;
    composite_forward_kernel<256><<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, out);
  } else {
    rc = set_smem(composite_forward_kernel<1024>, smem);
    if (rc != MT_OK) return rc;
    composite_forward_kernel<1024><<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, out);
  }
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_intersect_and_composite_backward(const float* xy, const float* colors, const float* signed_distances,
                                        int64_t V, const int32_t* faces, const float* sharpness,
                                        const int64_t* sorted_keys, const int32_t* sorted_triangles,
                                        const int64_t* tile_boundaries, int32_t B, int32_t num_shells,
                                        int32_t rows, int32_t cols, int32_t tile_h, int32_t tile_w, int32_t H,
                                        int32_t W, int32_t shell_bit_offset, int32_t shell_bit_length,
                                        const float* out, const float* grad_out, float* grad_colors,
                                        float* grad_signed_distances, float* grad_sharpness, int32_t exact_adjoint,
                                        mt_stream_t stream) {
  CompositeArgs a{xy, colors, signed_distances, V, faces, sharpness,
                  reinterpret_cast<const uint64_t*>(sorted_keys), sorted_triangles, tile_boundaries,
                  B, num_shells, rows, cols, tile_h, tile_w, H, W, shell_bit_offset, shell_bit_length, out};
  int rc = check_args(a);
  if (rc != MT_OK) return rc;
  const int64_t blocks = (int64_t)B * rows * cols;
  if (blocks == 0 || H == 0 || W == 0) return MT_OK;
  MT_REQUIRE(xy && colors && signed_distances && faces && sharpness && tile_boundaries && out && grad_out);
  MT_REQUIRE(grad_colors && grad_signed_distances && grad_sharpness);
  MT_REQUIRE(blocks < ((int64_t)1 << 31));
  CompositeGrads gr{grad_out, grad_colors, grad_signed_distances, grad_sharpness, exact_adjoint ? 1 : 0};
  const int bs = block_threads(a);
  const int chunk = bs < kMaxChunk ? bs : kMaxChunk;
  const size_t smem = smem_bytes(chunk, bs / 32, true);
  if (bs <= 256) {
    rc = set_smem(composite_backward_kernel<256>, smem);
    if (rc != MT_OK) return rc;
    composite_backward_kernel<256><<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, gr);
  } else {
    rc = set_smem(composite_backward_kernel<1024>, smem);
    if (rc != MT_OK) return rc;
    composite_backward_kernel<1024><<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, gr);
  }
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
