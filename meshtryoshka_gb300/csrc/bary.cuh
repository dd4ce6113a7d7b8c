// Barycentric solve shared by the fused and explicit rasterization kernels
// (triangle_rasterization/intersect_and_composite.slang:65-136 and the
// identical intersect.slang:14-67), plus the NeuS alpha helpers
// (intersect_and_composite.slang:153-163, composite.slang:33-46).
//
// The operation order is fixed (explicit __fmaf_rn / __fmul_rn / __fdiv_rn,
// so nvcc cannot re-contract), which lets the CPU restatement reproduce every
// hit decision bit for bit.
#pragma once

#include "mt_common.cuh"

namespace mt {

struct TriGeom {
  float p1x, p1y, p2x, p2y;    // first two corners
  float e12x, e12y, e13x, e13y;  // edge vectors p2 - p1, p3 - p1
  float d1212, d1213, d1313, d1223;
  float d1323, dd, thr;  // dd = denom + 1e-8; thr = fast-reject threshold (or -inf)
  int shell;
};

__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) {
  return __fmaf_rn(ay, by, __fmul_rn(ax, bx));
}

// intersect_and_composite.slang:65-106 (triangle-only part) for one staged
// triangle.
__device__ __forceinline__ void setup_geometry(float p1x, float p1y, float p2x, float p2y, float p3x, float p3y,
                                               TriGeom& g) {
  const float e12x = __fsub_rn(p2x, p1x), e12y = __fsub_rn(p2y, p1y);
  const float e13x = __fsub_rn(p3x, p1x), e13y = __fsub_rn(p3y, p1y);
  const float e23x = __fsub_rn(p3x, p2x), e23y = __fsub_rn(p3y, p2y);
  const float d1212 = dot2(e12x, e12y, e12x, e12y);
  const float d1223 = dot2(e12x, e12y, e23x, e23y);
  const float d1213 = dot2(e12x, e12y, e13x, e13y);
  const float d1313 = dot2(e13x, e13y, e13x, e13y);
  const float d1323 = dot2(e13x, e13y, e23x, e23y);
  const float d2323 = dot2(e23x, e23y, e23x, e23y);
  const float a = fabsf(d1213), b = fabsf(d1223), c = fabsf(d1323);
  float denom;
  if (a <= b && a <= c) {
    denom = __fmaf_rn(d1212, d1313, -__fmul_rn(d1213, d1213));
  } else if (b <= a && b <= c) {
    denom = __fmaf_rn(d1212, d2323, -__fmul_rn(d1223, d1223));
  } else if (c <= a && c <= b) {
    denom = __fmaf_rn(d1313, d2323, -__fmul_rn(d1323, d1323));
  } else {
    denom = __int_as_float(0x7fffffff);  // only reachable with a NaN product: the sample is rejected anyway
  }
  const float dd = __fadd_rn(denom, 1e-8f);
  g.p1x = p1x;
  g.p1y = p1y;
  g.p2x = p2x;
  g.p2y = p2y;
  g.e12x = e12x;
  g.e12y = e12y;
  g.e13x = e13x;
  g.e13y = e13y;
  g.d1212 = d1212;
  g.d1213 = d1213;
  g.d1313 = d1313;
  g.d1223 = d1223;
  g.d1323 = d1323;
  g.dd = dd;
  const bool fast = dd > 0x1p-20f && dd < __int_as_float(0x7f800000);
  g.thr = fast ? -__fmul_rn(dd, 0x1p-100f) : __int_as_float(0xff800000);
}

// Barycentric solve and acceptance test (intersect_and_composite.slang:65-136).
__device__ __forceinline__ bool hit_test(const TriGeom& g, float px, float py, float& u, float& v, float& w) {
  const float q1x = __fsub_rn(px, g.p1x), q1y = __fsub_rn(py, g.p1y);
  const float q2x = __fsub_rn(px, g.p2x), q2y = __fsub_rn(py, g.p2y);
  const float d1x12 = dot2(q1x, q1y, g.e12x, g.e12y);
  const float d1x13 = dot2(q1x, q1y, g.e13x, g.e13y);
  const float d2x12 = dot2(q2x, q2y, g.e12x, g.e12y);
  const float d2x13 = dot2(q2x, q2y, g.e13x, g.e13y);
  const float vn = __fmaf_rn(g.d1313, d1x12, -__fmul_rn(g.d1213, d1x13));
  const float wn = __fmaf_rn(g.d1212, d1x13, -__fmul_rn(g.d1213, d1x12));
  const float un = __fmaf_rn(g.d1223, d2x13, -__fmul_rn(g.d1323, d2x12));
  if (un < g.thr || vn < g.thr || wn < g.thr) return false;
  u = __fdiv_rn(un, g.dd);
  v = __fdiv_rn(vn, g.dd);
  w = __fdiv_rn(wn, g.dd);
  const float sum = __fadd_rn(__fadd_rn(u, v), w);
  if (isnan(u) || isnan(v) || isnan(w)) return false;
  if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f || w < 0.0f || w > 1.0f) return false;
  if (sum < 0.999f || sum > 1.001f) return false;
  return true;
}

__device__ __forceinline__ float interp(float u, float v, float w, float a, float b, float c) {
  return __fmaf_rn(w, c, __fmaf_rn(v, b, __fmul_rn(u, a)));
}

// sdf_to_cdf (intersect_and_composite.slang:153-156); also returns exp(-sdf s).
__device__ __forceinline__ float sdf_to_cdf(float sdf, float s, float& e) {
  e = expf(__fmul_rn(-sdf, s));
  return __fdiv_rn(1.0f, __fadd_rn(1.0f, e));
}

__device__ __forceinline__ float alpha_raw(float oc, float ic) {
  return __fdiv_rn(__fadd_rn(__fsub_rn(oc, ic), 1e-5f), __fadd_rn(oc, 1e-5f));
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }


}  // namespace mt
