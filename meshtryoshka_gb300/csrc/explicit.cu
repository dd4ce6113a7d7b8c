// Explicit render mode for sm_103a: per-shell first-hit rasterization,
// barycentric interpolation (forward / backward) and the per-pixel shell
// compositing loop (forward / backward).
//
// Follows triangle_rasterization/intersect.slang:86-182,
// interpolate.slang:19-76 and composite.slang:60-218. The hit test is the
// same fixed-order barycentric solve as the fused kernel (bary.cuh).
//
// composite backward has the same two gradient-routing modes as the fused
// kernel: the reference's (the outer sample's signed-distance gradient goes
// to slot shell_index - 1 and the last one to slot num_shells - 1,
// composite.slang:197,212) or the exact adjoint (the previous and last *hit*
// shells).

#include "bary.cuh"
#include "mt_common.cuh"

namespace mt {
namespace {

struct ExplicitFace {
  TriGeom g;
  int32_t face;
};

__global__ void intersect_kernel(const float* __restrict__ xy, int64_t V, const int32_t* __restrict__ faces,
                                 const int32_t* __restrict__ tri, const int64_t* __restrict__ bounds, int B, int S,
                                 int rows, int cols, int tile_h, int tile_w, int H, int W, float* __restrict__ out_uv,
                                 int32_t* __restrict__ out_index) {
  extern __shared__ float4 smem_f4[];
  ExplicitFace* sf = reinterpret_cast<ExplicitFace*>(smem_f4);
  const int bs = blockDim.x;
  const int64_t T = (int64_t)rows * cols;
  const int64_t tile = blockIdx.x % T;
  const int64_t batch = blockIdx.x / T;  // camera * S + shell
  const int cam = (int)(batch / S);
  const int tid = threadIdx.x;
  const int px = (int)(tile % cols) * tile_w + tid % tile_w;
  const int py = (int)(tile / cols) * tile_h + tid / tile_w;
  const bool in_image = px < W && py < H;
  const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
  bool active = in_image;
  const int64_t start = bounds[2 * (batch * T + tile)];
  const int64_t end = bounds[2 * (batch * T + tile) + 1];
  const float2* xyc = reinterpret_cast<const float2*>(xy) + (int64_t)cam * V;
  for (int64_t chunk = start; chunk < end; chunk += bs) {
    if (__syncthreads_count(active) == 0) break;
    if (chunk + tid < end) {
      const int32_t f = tri[chunk + tid];
      const float2 pa = xyc[faces[3 * (int64_t)f]], pb = xyc[faces[3 * (int64_t)f + 1]],
                   pc = xyc[faces[3 * (int64_t)f + 2]];
      ExplicitFace e;
      setup_geometry(pa.x, pa.y, pb.x, pb.y, pc.x, pc.y, e.g);
      e.face = f;
      sf[tid] = e;
    }
    __syncthreads();
    if (active) {
      const int n = (int)min((int64_t)bs, end - chunk);
      for (int i = 0; i < n; ++i) {
        float u, v, w;
        if (!hit_test(sf[i].g, fx, fy, u, v, w)) continue;
        active = false;
        const int64_t o = (batch * H + py) * W + px;
        out_uv[2 * o] = u;
        out_uv[2 * o + 1] = v;
        out_index[o] = sf[i].face;
        break;
      }
    }
  }
  if (active) {
    const int64_t o = (batch * H + py) * W + px;
    out_uv[2 * o] = 0.f;
    out_uv[2 * o + 1] = 0.f;
    out_index[o] = -1;
  }
}

// interpolate.slang:22-76. (u, v, w = 1 - u - v) weights of the hit face.
__global__ void interpolate_forward_kernel(const float* __restrict__ uv, const int32_t* __restrict__ index,
                                           const int32_t* __restrict__ faces, const float* __restrict__ sdf,
                                           const float* __restrict__ colors, int64_t V, int S, int64_t BS,
                                           int64_t HW, float* __restrict__ out_sdf, float* __restrict__ out_colors) {
  const int64_t total = BS * HW;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t f = index[i];
    if (f < 0) {
      out_colors[3 * i] = 0.f;
      out_colors[3 * i + 1] = 0.f;
      out_colors[3 * i + 2] = 0.f;
      out_sdf[i] = 0.f;
      continue;
    }
    const int64_t b = (i / HW) / S;
    const float u = uv[2 * i], v = uv[2 * i + 1];
    const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
    const int32_t ia = faces[3 * (int64_t)f], ib = faces[3 * (int64_t)f + 1], ic = faces[3 * (int64_t)f + 2];
    const float* col = colors + b * V * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      out_colors[3 * i + c] = interp(u, v, w, col[3 * (int64_t)ia + c], col[3 * (int64_t)ib + c],
                                     col[3 * (int64_t)ic + c]);
    out_sdf[i] = interp(u, v, w, sdf[ia], sdf[ib], sdf[ic]);
  }
}

__global__ void interpolate_backward_kernel(const float* __restrict__ uv, const int32_t* __restrict__ index,
                                            const int32_t* __restrict__ faces, int64_t V, int S, int64_t BS,
                                            int64_t HW, const float* __restrict__ grad_sdf_out,
                                            const float* __restrict__ grad_colors_out,
                                            float* __restrict__ grad_sdf, float* __restrict__ grad_colors) {
  const int64_t total = BS * HW;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t f = index[i];
    if (f < 0) continue;
    const float gs = grad_sdf_out ? grad_sdf_out[i] : 0.f;
    const float g0 = grad_colors_out ? grad_colors_out[3 * i] : 0.f;
    const float g1 = grad_colors_out ? grad_colors_out[3 * i + 1] : 0.f;
    const float g2 = grad_colors_out ? grad_colors_out[3 * i + 2] : 0.f;
    if (gs == 0.f && g0 == 0.f && g1 == 0.f && g2 == 0.f) continue;
    const int64_t b = (i / HW) / S;
    const float u = uv[2 * i], v = uv[2 * i + 1];
    const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
    const int32_t id[3] = {faces[3 * (int64_t)f], faces[3 * (int64_t)f + 1], faces[3 * (int64_t)f + 2]};
    const float wt[3] = {u, v, w};
    float* gc = grad_colors + b * V * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (gs != 0.f) atomicAdd(grad_sdf + id[k], wt[k] * gs);
      atomicAdd(gc + 3 * (int64_t)id[k], wt[k] * g0);
      atomicAdd(gc + 3 * (int64_t)id[k] + 1, wt[k] * g1);
      atomicAdd(gc + 3 * (int64_t)id[k] + 2, wt[k] * g2);
    }
  }
}

// composite.slang:60-120: front-to-back over the masked shells of a pixel.
__global__ void shell_composite_forward_kernel(const float* __restrict__ sdf, const float* __restrict__ colors,
                                               const uint8_t* __restrict__ mask, int64_t P, int S,
                                               const float* __restrict__ sharpness, float* __restrict__ out_colors,
                                               float* __restrict__ out_T) {
  const float s = *sharpness;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    float acc[3] = {0.f, 0.f, 0.f};
    float T = 1.0f;
    float e;
    float outer_cdf = sdf_to_cdf(1e10f, s, e);
    for (int l = 0; l < S; ++l) {
      if (!mask[p * S + l]) continue;
      const float inner = sdf[p * S + l];
      const float inner_cdf = sdf_to_cdf(inner, s, e);
      const float alpha = clamp01(alpha_raw(outer_cdf, inner_cdf));
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] = over(acc[c], colors[(p * S + l) * 3 + c], T, alpha);
      T = __fmul_rn(T, __fsub_rn(1.0f, alpha));
      outer_cdf = inner_cdf;
    }
    out_colors[3 * p] = acc[0];
    out_colors[3 * p + 1] = acc[1];
    out_colors[3 * p + 2] = acc[2];
    out_T[p] = T;
  }
}

// composite.slang:122-218 (suffix trick, per-pixel sequential shells).
__global__ void shell_composite_backward_kernel(const float* __restrict__ sdf, const float* __restrict__ colors,
                                                const uint8_t* __restrict__ mask, int64_t P, int S,
                                                const float* __restrict__ sharpness,
                                                const float* __restrict__ out_colors, const float* __restrict__ out_T,
                                                const float* __restrict__ grad_colors_out,
                                                const float* __restrict__ grad_T_out, float* __restrict__ grad_sdf,
                                                float* __restrict__ grad_colors, float* __restrict__ grad_sharpness,
                                                int exact) {
  __shared__ float s_red[32];
  const float s = *sharpness;
  float d_sharp_total = 0.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    const float final_rgb[3] = {out_colors[3 * p], out_colors[3 * p + 1], out_colors[3 * p + 2]};
    const float final_T = out_T[p];
    const float dL[3] = {grad_colors_out ? grad_colors_out[3 * p] : 0.f,
                         grad_colors_out ? grad_colors_out[3 * p + 1] : 0.f,
                         grad_colors_out ? grad_colors_out[3 * p + 2] : 0.f};
    const float dLT = grad_T_out ? grad_T_out[p] : 0.f;
    float acc[3] = {0.f, 0.f, 0.f};
    float T = 1.0f;
    float e_out;
    float outer_cdf = sdf_to_cdf(1e10f, s, e_out);
    float outer_sdf = 1e10f;
    bool first = true;
    int prev_shell = -1;
    float d_partial = 0.f;
    for (int l = 0; l < S; ++l) {
      if (!mask[p * S + l]) continue;
      const float inner = sdf[p * S + l];
      float e_in;
      const float inner_cdf = sdf_to_cdf(inner, s, e_in);
      const float raw = alpha_raw(outer_cdf, inner_cdf);
      const float alpha = clamp01(raw);
      const float weight = __fmul_rn(alpha, T);
      const float inv = __fdiv_rn(1.0f, __fadd_rn(__fsub_rn(1.0f, alpha), 1e-6f));
      float d_alpha = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float col = colors[(p * S + l) * 3 + c];
        acc[c] = __fadd_rn(acc[c], __fmul_rn(weight, col));
        const float suffix = final_rgb[c] - acc[c];
        d_alpha += dL[c] * (T * col - suffix * inv);
        grad_colors[(p * S + l) * 3 + c] += weight * dL[c];
      }
      d_alpha += -dLT * final_T * inv;
      const float d_raw = (raw > 0.0f && raw < 1.0f) ? d_alpha : 0.0f;
      const float den = outer_cdf + 1e-5f;
      const float num = (outer_cdf - inner_cdf) + 1e-5f;
      const float d_num = d_raw / den;
      const float d_den = -d_raw * num / (den * den);
      const float d_oc = d_num + d_den;
      const float d_ic = -d_num;
      const float ki = inner_cdf * inner_cdf * e_in;
      const float ko = outer_cdf * outer_cdf * e_out;
      d_sharp_total += d_ic * ki * inner + d_oc * ko * outer_sdf;
      if (!first) {
        d_partial += d_oc * ko * s;
        const int slot = exact ? prev_shell : l - 1;
        grad_sdf[p * S + slot] += d_partial;
      }
      d_partial = d_ic * ki * s;
      T = __fmul_rn(T, __fsub_rn(1.0f, alpha));
      outer_cdf = inner_cdf;
      outer_sdf = inner;
      e_out = e_in;
      first = false;
      prev_shell = l;
    }
    if (!first) grad_sdf[p * S + (exact ? prev_shell : S - 1)] += d_partial;
  }
  float x = d_sharp_total;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = (blockDim.x + 31) >> 5;
    float y = threadIdx.x < nw ? s_red[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    if (threadIdx.x == 0 && y != 0.f) atomicAdd(grad_sharpness, y);
  }
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" {

int mt_intersect(const float* xy, int64_t V, const int32_t* faces, const int32_t* sorted_triangles,
                 const int64_t* tile_boundaries, int32_t B, int32_t S, int32_t rows, int32_t cols, int32_t tile_h,
                 int32_t tile_w, int32_t H, int32_t W, float* out_uv, int32_t* out_index, mt_stream_t stream) {
  MT_REQUIRE(B >= 0 && S >= 1 && rows >= 0 && cols >= 0 && tile_h > 0 && tile_w > 0 && H >= 0 && W >= 0);
  MT_REQUIRE((int64_t)tile_h * tile_w <= 1024);
  MT_REQUIRE((int64_t)rows * tile_h >= H && (int64_t)cols * tile_w >= W);
  const int64_t blocks = (int64_t)B * S * rows * cols;
  if (blocks == 0 || H == 0 || W == 0) return MT_OK;
  MT_REQUIRE(xy && faces && tile_boundaries && out_uv && out_index);
  MT_REQUIRE(blocks < ((int64_t)1 << 31));
  const int bs = tile_h * tile_w;
  const size_t smem = (size_t)bs * sizeof(ExplicitFace);
  if (set_smem<intersect_kernel>(smem) != MT_OK) return MT_ERR_CUDA;
  intersect_kernel<<<(unsigned)blocks, bs, smem, as_stream(stream)>>>(xy, V, faces, sorted_triangles,
                                                                      tile_boundaries, B, S, rows, cols, tile_h,
                                                                      tile_w, H, W, out_uv, out_index);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_interpolate(const float* uv, const int32_t* index, int32_t B, int32_t S, int32_t H, int32_t W,
                   const int32_t* faces, const float* signed_distances, const float* colors, int64_t V,
                   float* out_signed_distances, float* out_colors, mt_stream_t stream) {
  MT_REQUIRE(B >= 0 && S >= 1 && H >= 0 && W >= 0 && V >= 0);
  const int64_t total = (int64_t)B * S * H * W;
  if (total == 0) return MT_OK;
  MT_REQUIRE(uv && index && faces && signed_distances && colors && out_signed_distances && out_colors);
  interpolate_forward_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(
      uv, index, faces, signed_distances, colors, V, S, (int64_t)B * S, (int64_t)H * W, out_signed_distances,
      out_colors);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_interpolate_backward(const float* uv, const int32_t* index, int32_t B, int32_t S, int32_t H, int32_t W,
                            const int32_t* faces, int64_t V, const float* grad_out_signed_distances,
                            const float* grad_out_colors, float* grad_signed_distances, float* grad_colors,
                            mt_stream_t stream) {
  MT_REQUIRE(B >= 0 && S >= 1 && H >= 0 && W >= 0 && V >= 0);
  const int64_t total = (int64_t)B * S * H * W;
  if (total == 0) return MT_OK;
  MT_REQUIRE(uv && index && faces && grad_signed_distances && grad_colors);
  interpolate_backward_kernel<<<grid_stride_blocks(total, 256), 256, 0, as_stream(stream)>>>(
      uv, index, faces, V, S, (int64_t)B * S, (int64_t)H * W, grad_out_signed_distances, grad_out_colors,
      grad_signed_distances, grad_colors);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_composite(const float* signed_distances, const float* colors, const uint8_t* mask, int64_t P, int32_t S,
                 const float* sharpness, float* out_colors, float* out_transmittances, mt_stream_t stream) {
  MT_REQUIRE(P >= 0 && S >= 0);
  if (P == 0) return MT_OK;
  MT_REQUIRE(sharpness && out_colors && out_transmittances);
  MT_REQUIRE(S == 0 || (signed_distances && colors && mask));
  shell_composite_forward_kernel<<<grid_stride_blocks(P, 256), 256, 0, as_stream(stream)>>>(
      signed_distances, colors, mask, P, S, sharpness, out_colors, out_transmittances);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

int mt_composite_backward(const float* signed_distances, const float* colors, const uint8_t* mask, int64_t P,
                          int32_t S, const float* sharpness, const float* out_colors,
                          const float* out_transmittances, const float* grad_out_colors,
                          const float* grad_out_transmittances, float* grad_signed_distances, float* grad_colors,
                          float* grad_sharpness, int32_t exact_adjoint, mt_stream_t stream) {
  MT_REQUIRE(P >= 0 && S >= 0);
  if (P == 0 || S == 0) return MT_OK;
  MT_REQUIRE(signed_distances && colors && mask && sharpness && out_colors && out_transmittances);
  MT_REQUIRE(grad_signed_distances && grad_colors && grad_sharpness);
  shell_composite_backward_kernel<<<grid_stride_blocks(P, 256), 256, 0, as_stream(stream)>>>(
      signed_distances, colors, mask, P, S, sharpness, out_colors, out_transmittances, grad_out_colors,
      grad_out_transmittances, grad_signed_distances, grad_colors, grad_sharpness, exact_adjoint ? 1 : 0);
  MT_CHECK_LAUNCH();
  return MT_OK;
}

}  // extern "C"
