// Fused multi-shell intersect + composite, forward and backward, for sm_103a.
//
// Follows triangle_rasterization/intersect_and_composite.slang:1-564. One CTA
// per (camera, tile), one thread per pixel. Each tile's depth-sorted triangle
// list is staged through shared memory in CTA-sized chunks; per-triangle
// quantities of the barycentric solve (edge vectors, the six edge dot
// products, the chosen denominator) are computed once by the staging thread
// instead of once per pixel, with the same operations, so every per-pixel
// result is bit-identical to evaluating the full formula per pixel.
//
// Per pixel, the three barycentric numerators decide most misses exactly
// before any division: with a positive, finite denominator d, a numerator
// below -d * 2^-100 yields a quotient below -2^-100 after rounding, which the
// reference test rejects as "< 0". Only the remaining candidates pay for the
// three IEEE divisions and the full acceptance test.
//
// Backward re-walks the list, recomputes hits, and applies the suffix trick
// of the reference. Gradient routing has two modes:
//   kReference  (default) exactly the reference's routing: the deferred
//               gradient of the previous (outer) hit is scattered to the
//               previous triangle's vertices with the *current* triangle's
//               barycentric weights (intersect_and_composite.slang:487-509);
//   kExact      the adjoint of the forward: the previous hit's own weights.
// Sharpness gradients are reduced per CTA before one global atomic.

#include "bary.cuh"
#include "mt_common.cuh"

namespace mt {
namespace {

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
  const uint64_t* keys;    // sorted keys
  const int32_t* tri;      // sorted triangle indices
  const int64_t* bounds;   // [B, T, 2]
  int B, S, rows, cols, tile_h, tile_w, H, W;
  int shell_off, shell_len;
  const float* out;  // forward output [B, 4, H, W] (input to backward)
};

// Stages triangle `k` of the sorted list into slot `slot`.
__device__ __forceinline__ void stage(const CompositeArgs& a, int cam, int64_t k, TriGeom* geo, TriAttr* attr,
                                      int3* vids, int slot) {
  const int32_t f = a.tri[k];
  const uint64_t key = a.keys[k];
  const int32_t ia = a.faces[3 * (int64_t)f], ib = a.faces[3 * (int64_t)f + 1], ic = a.faces[3 * (int64_t)f + 2];
  const float2* xy = reinterpret_cast<const float2*>(a.xy) + (int64_t)cam * a.V;
  const float2 pa = xy[ia], pb = xy[ib], pc = xy[ic];
  TriGeom g;
  setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, g);
  g.shell = (int)((key >> a.shell_off) & (uint64_t)((1u << a.shell_len) - 1u));
  geo[slot] = g;
  if (attr) {
    const float* col = a.colors + (int64_t)cam * a.V * 3;
    TriAttr t;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      t.ca[c] = col[3 * (int64_t)ia + c];
      t.cb[c] = col[3 * (int64_t)ib + c];
      t.cc[c] = col[3 * (int64_t)ic + c];
    }
    t.sa = a.sdf[ia];
    t.sb = a.sdf[ib];
    t.sc = a.sdf[ic];
    attr[slot] = t;
  }
  if (vids) vids[slot] = make_int3(ia, ib, ic);
}

__global__ void composite_forward_kernel(CompositeArgs a, float* __restrict__ out) {
  extern __shared__ float4 smem_f4[];
  const int bs = blockDim.x;
  TriGeom* geo = reinterpret_cast<TriGeom*>(smem_f4);
  TriAttr* attr = reinterpret_cast<TriAttr*>(geo + bs);

  const int64_t T = (int64_t)a.rows * a.cols;
  const int64_t tile = blockIdx.x % T;
  const int cam = (int)(blockIdx.x / T);
  const int tid = threadIdx.x;
  const int px = (int)(tile % a.cols) * a.tile_w + tid % a.tile_w;
  const int py = (int)(tile / a.cols) * a.tile_h + tid / a.tile_w;
  const bool in_image = px < a.W && py < a.H;
  const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
  const float s = *a.sharpness;

  float acc[3] = {0.f, 0.f, 0.f};
  float T_ = 1.0f;
  bool active = in_image;
  int last_shell = -1;
  float e_dummy;
  float outer_cdf = sdf_to_cdf(1e10f, s, e_dummy);  // dummy outer sample

  const int64_t start = a.bounds[2 * ((int64_t)cam * T + tile)];
  const int64_t end = a.bounds[2 * ((int64_t)cam * T + tile) + 1];
  for (int64_t chunk = start; chunk < end; chunk += bs) {
    if (__syncthreads_count(active) == 0) break;
    if (chunk + tid < end) stage(a, cam, chunk + tid, geo, attr, nullptr, tid);
    __syncthreads();
    if (active) {
      const int n = (int)min((int64_t)bs, end - chunk);
      for (int i = 0; i < n; ++i) {
        const int shell = geo[i].shell;
        if (shell <= last_shell) continue;
        float u, v, w;
        if (!hit_test(geo[i], fx, fy, u, v, w)) continue;
        const TriAttr& t = attr[i];
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
        last_shell = shell;
        if (last_shell == a.S - 1) {
          active = false;
          break;
        }
      }
    }
  }
  if (in_image) {
    const int64_t plane = (int64_t)a.H * a.W;
    float* o = out + (int64_t)cam * 4 * plane + (int64_t)py * a.W + px;
    o[0] = acc[0];
    o[plane] = acc[1];
    o[2 * plane] = acc[2];
    o[3 * plane] = T_;
  }
}

struct CompositeGrads {
  const float* grad_out;  // [B, 4, H, W]
  float* grad_colors;     // [B, V, 3]
  float* grad_sdf;        // [V]
  float* grad_sharpness;  // [1]
  int exact;
};

__device__ __forceinline__ void scatter(const CompositeArgs& a, const CompositeGrads& gr, int cam, int3 vid,
                                        float u, float v, float w, const float (&drgb)[3], float dsdf) {
  float* gc = gr.grad_colors + (int64_t)cam * a.V * 3;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    atomicAdd(gc + 3 * (int64_t)vid.x + c, u * drgb[c]);
    atomicAdd(gc + 3 * (int64_t)vid.y + c, v * drgb[c]);
    atomicAdd(gc + 3 * (int64_t)vid.z + c, w * drgb[c]);
  }
  atomicAdd(gr.grad_sdf + vid.x, u * dsdf);
  atomicAdd(gr.grad_sdf + vid.y, v * dsdf);
  atomicAdd(gr.grad_sdf + vid.z, w * dsdf);
}

__global__ void composite_backward_kernel(CompositeArgs a, CompositeGrads gr) {
  extern __shared__ float4 smem_f4[];
  const int bs = blockDim.x;
  TriGeom* geo = reinterpret_cast<TriGeom*>(smem_f4);
  TriAttr* attr = reinterpret_cast<TriAttr*>(geo + bs);
  int3* vids = reinterpret_cast<int3*>(attr + bs);
  __shared__ float s_red[32];

  const int64_t T = (int64_t)a.rows * a.cols;
  const int64_t tile = blockIdx.x % T;
  const int cam = (int)(blockIdx.x / T);
  const int tid = threadIdx.x;
  const int px = (int)(tile % a.cols) * a.tile_w + tid % a.tile_w;
  const int py = (int)(tile / a.cols) * a.tile_h + tid / a.tile_w;
  const bool in_image = px < a.W && py < a.H;
  const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
  const float s = *a.sharpness;

  float final_rgb[3] = {0.f, 0.f, 0.f}, dL_rgb[3] = {0.f, 0.f, 0.f};
  float final_T = 0.f, dL_T = 0.f;
  if (in_image) {
    const int64_t plane = (int64_t)a.H * a.W;
    const int64_t o = (int64_t)cam * 4 * plane + (int64_t)py * a.W + px;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      final_rgb[c] = a.out[o + c * plane];
      dL_rgb[c] = gr.grad_out[o + c * plane];
    }
    final_T = a.out[o + 3 * plane];
    dL_T = gr.grad_out[o + 3 * plane];
  }

  float acc[3] = {0.f, 0.f, 0.f};
  float T_ = 1.0f;
  bool active = in_image;
  int last_shell = -1;
  float e_out;
  float outer_cdf = sdf_to_cdf(1e10f, s, e_out);
  float outer_sdf = 1e10f;
  float d_sharp = 0.f;
  float dp_rgb[3] = {0.f, 0.f, 0.f};
  float dp_sdf = 0.f;
  int3 prev_vid = make_int3(0, 0, 0);
  float pu = 0.f, pv = 0.f, pw = 0.f;

  const int64_t start = a.bounds[2 * ((int64_t)cam * T + tile)];
  const int64_t end = a.bounds[2 * ((int64_t)cam * T + tile) + 1];
  for (int64_t chunk = start; chunk < end; chunk += bs) {
    if (__syncthreads_count(active) == 0) break;
    if (chunk + tid < end) stage(a, cam, chunk + tid, geo, attr, vids, tid);
    __syncthreads();
    if (active) {
      const int n = (int)min((int64_t)bs, end - chunk);
      for (int i = 0; i < n; ++i) {
        const int shell = geo[i].shell;
        if (shell <= last_shell) continue;
        float u, v, w;
        if (!hit_test(geo[i], fx, fy, u, v, w)) continue;
        const TriAttr& t = attr[i];
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

        // compute_alpha backward: clamp passes the gradient strictly inside.
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
        const float d_sdf_in = d_ic * ki * s;
        const float d_sdf_out = d_oc * ko * s;
        d_sharp += d_ic * ki * sdf_in + d_oc * ko * outer_sdf;

        if (last_shell != -1) {
          dp_sdf += d_sdf_out;
          if (gr.exact)
            scatter(a, gr, cam, prev_vid, pu, pv, pw, dp_rgb, dp_sdf);
          else
            scatter(a, gr, cam, prev_vid, u, v, w, dp_rgb, dp_sdf);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) dp_rgb[c] = d_color[c];
        dp_sdf = d_sdf_in;
        prev_vid = vids[i];
        pu = u;
        pv = v;
        pw = w;

        T_ = __fmul_rn(T_, __fsub_rn(1.0f, alpha));
        outer_cdf = inner_cdf;
        outer_sdf = sdf_in;
        e_out = e_in;
        last_shell = shell;
        if (last_shell == a.S - 1) {
          active = false;
          break;
        }
      }
    }
  }
  if (in_image && last_shell != -1) scatter(a, gr, cam, prev_vid, pu, pv, pw, dp_rgb, dp_sdf);

  // Block reduction of the sharpness gradient, one atomic per CTA.
  float x = in_image ? d_sharp : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((tid & 31) == 0) s_red[tid >> 5] = x;
  __syncthreads();
  if (tid < 32) {
    const int nw = (bs + 31) >> 5;
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

size_t forward_smem(int bs) { return (size_t)bs * (sizeof(TriGeom) + sizeof(TriAttr)); }
size_t backward_smem(int bs) { return (size_t)bs * (sizeof(TriGeom) + sizeof(TriAttr) + sizeof(int3)) + 16; }

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
  const int bs = tile_h * tile_w;
  const size_t smem = forward_smem(bs);
  rc = set_smem(composite_forward_kernel, smem);
  if (rc != MT_OK) return rc;
  composite_forward_kernel<<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, out);
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
  const int bs = tile_h * tile_w;
  const size_t smem = backward_smem(bs);
  rc = set_smem(composite_backward_kernel, smem);
  if (rc != MT_OK) return rc;
  composite_backward_kernel<<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(a, gr);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
