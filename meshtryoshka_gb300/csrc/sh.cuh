// Real spherical harmonics up to degree 3 and the vertex view direction
// (triangle_rasterization/evaluate_spherical_harmonics.slang:4-270), shared by
// the SH evaluation kernels and the fused grid-SH colour kernels. Units that
// include this header compile without FMA contraction, so every user
// evaluates the same operations with the same roundings.
#pragma once

#include "mt_common.cuh"

namespace mt {
namespace {

// rgb = max(sum_k basis_k(dir) sh_k + 0.5, 0).
__constant__ float kShC0 = 0.28209479177387814f;
__constant__ float kShC1 = 0.4886025119029199f;
__constant__ float kShC2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                               -1.0925484305920792f, 0.5462742152960396f};
__constant__ float kShC3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                               0.3731763325901154f,  -0.4570457994644658f, 1.445305721320277f,
                               -0.5900435899266435f};

__device__ __forceinline__ void sh_basis(float x, float y, float z, int n, float (&basis)[16]) {
  basis[0] = kShC0;
  if (n <= 1) return;
  basis[1] = -kShC1 * y;
  basis[2] = kShC1 * z;
  basis[3] = -kShC1 * x;
  if (n <= 4) return;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  basis[4] = kShC2[0] * xy;
  basis[5] = kShC2[1] * yz;
  basis[6] = kShC2[2] * (2.0f * zz - xx - yy);
  basis[7] = kShC2[3] * xz;
  basis[8] = kShC2[4] * (xx - yy);
  if (n <= 9) return;
  basis[9] = kShC3[0] * y * (3.0f * xx - yy);
  basis[10] = kShC3[1] * xy * z;
  basis[11] = kShC3[2] * y * (4.0f * zz - xx - yy);
  basis[12] = kShC3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
  basis[13] = kShC3[4] * x * (4.0f * zz - xx - yy);
  basis[14] = kShC3[5] * z * (xx - yy);
  basis[15] = kShC3[6] * x * (xx - 3.0f * yy);
}

// normalize(p - camera) = d / sqrt(dot(d, d)) for a position held in
// registers.
__device__ __forceinline__ void view_dir_at(float px, float py, float pz, const float* __restrict__ cam, float& x,
                                            float& y, float& z) {
  const float dx = __fsub_rn(px, cam[0]), dy = __fsub_rn(py, cam[1]), dz = __fsub_rn(pz, cam[2]);
  const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  x = __fdiv_rn(dx, len);
  y = __fdiv_rn(dy, len);
  z = __fdiv_rn(dz, len);
}

__device__ __forceinline__ void view_dir(const float* __restrict__ verts, int64_t v, const float* __restrict__ cam,
                                         float& x, float& y, float& z) {
  view_dir_at(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2], cam, x, y, z);
}

// Colours of vertex v for every camera from its coefficients (in
// registers): rgb_b = max(sum_k basis_k(dir_b) coef_k + 0.5, 0), terms added
// in k order. out: [B, V, 3].
template <int kCoeff>
__device__ __forceinline__ void sh_colors(const float* __restrict__ verts, int64_t V, const float (&coef)[kCoeff][3],
                                          const float* __restrict__ campos, int B, int64_t v,
                                          float* __restrict__ out) {
  for (int b = 0; b < B; ++b) {
    float x, y, z;
    view_dir(verts, v, campos + 3 * b, x, y, z);
    float basis[16];
    sh_basis(x, y, z, kCoeff, basis);
    float rgb[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[c] = __fmul_rn(basis[0], coef[0][c]);
#pragma unroll
    for (int k = 1; k < kCoeff; ++k) {
#pragma unroll
      for (int c = 0; c < 3; ++c) rgb[c] = __fadd_rn(rgb[c], __fmul_rn(basis[k], coef[k][c]));
    }
    float* o = out + ((int64_t)b * V + v) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = fmaxf(__fadd_rn(rgb[c], 0.5f), 0.0f);
  }
}

}  // namespace
}  // namespace mt
