// Barycentric solve shared by the fused and explicit rasterization kernels
// (triangle_rasterization/intersect_and_composite.slang:65-136 and the
// identical intersect.slang:14-67), plus the NeuS alpha helpers
// (intersect_and_composite.slang:153-163, composite.slang:33-46).
//
// Every operation is the reference source's, in its order and without
// contraction (explicit __fmul_rn / __fadd_rn / __fsub_rn / __fdiv_rn, which
// nvcc never fuses), so hit decisions equal the reference kernel evaluated
// operation by operation in IEEE-754 single precision.
#pragma once

#include "mt_common.cuh"

namespace mt {

// 64 bytes, 16-byte aligned: a staged triangle loads as four 16-byte words.
struct alignas(16) TriGeom {
  float p1x, p1y, p2x, p2y;    // first two corners
  float e12x, e12y, e13x, e13y;  // edge vectors p2 - p1, p3 - p1
  float d1212, d1213, d1313, d1223;
  float d1323, dd, thr;  // dd = denom + 1e-8; thr = fast-reject threshold (or -inf)
  int shell;
};

// A staged triangle read from shared memory as four 16-byte loads.
__device__ __forceinline__ TriGeom load_geom(const TriGeom* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = q[0], b = q[1], c = q[2], d = q[3];
  TriGeom g;
  g.p1x = a.x; g.p1y = a.y; g.p2x = a.z; g.p2y = a.w;
  g.e12x = b.x; g.e12y = b.y; g.e13x = b.z; g.e13y = b.w;
  g.d1212 = c.x; g.d1213 = c.y; g.d1313 = c.z; g.d1223 = c.w;
  g.d1323 = d.x; g.dd = d.y; g.thr = d.z; g.shell = __float_as_int(d.w);
  return g;
}

__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) {
  return __fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by));
}

// a * b - c * d, both products rounded.
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) {
  return __fsub_rn(__fmul_rn(a, b), __fmul_rn(c, d));
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
    denom = diff_of_products(d1212, d1313, d1213, d1213);
  } else if (b <= a && b <= c) {
    denom = diff_of_products(d1212, d2323, d1223, d1223);
  } else if (c <= a && c <= b) {
    denom = diff_of_products(d1313, d2323, d1323, d1323);
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

// The three barycentric numerators of pixel (px, py)
// (intersect_and_composite.slang:65-106).
__device__ __forceinline__ void numerators(const TriGeom& g, float px, float py, float& un, float& vn, float& wn) {
  const float q1x = __fsub_rn(px, g.p1x), q1y = __fsub_rn(py, g.p1y);
  const float q2x = __fsub_rn(px, g.p2x), q2y = __fsub_rn(py, g.p2y);
  const float d1x12 = dot2(q1x, q1y, g.e12x, g.e12y);
  const float d1x13 = dot2(q1x, q1y, g.e13x, g.e13y);
  const float d2x12 = dot2(q2x, q2y, g.e12x, g.e12y);
  const float d2x13 = dot2(q2x, q2y, g.e13x, g.e13y);
  vn = diff_of_products(g.d1313, d1x12, g.d1213, d1x13);
  wn = diff_of_products(g.d1212, d1x13, g.d1213, d1x12);
  un = diff_of_products(g.d1223, d2x13, g.d1323, d2x12);
}

// The fast reject: false when a numerator proves the quotient negative.
// NaN numerators pass (the divisions below reject them).
__device__ __forceinline__ bool numerators_pass(const TriGeom& g, float un, float vn, float wn) {
  return !(un < g.thr || vn < g.thr || wn < g.thr);
}

// The divisions and the acceptance test of a pixel whose numerators passed
// (intersect_and_composite.slang:107-136).
__device__ __forceinline__ bool solve_and_accept(float un, float vn, float wn, float dd, float& u, float& v,
                                                 float& w) {
  u = __fdiv_rn(un, dd);
  v = __fdiv_rn(vn, dd);
  w = __fdiv_rn(wn, dd);
  const float sum = __fadd_rn(__fadd_rn(u, v), w);
  if (isnan(u) || isnan(v) || isnan(w)) return false;
  if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f || w < 0.0f || w > 1.0f) return false;
  if (sum < 0.999f || sum > 1.001f) return false;
  return true;
}

// Barycentric solve and acceptance test (intersect_and_composite.slang:65-136).
__device__ __forceinline__ bool hit_test(const TriGeom& g, float px, float py, float& u, float& v, float& w) {
  float un, vn, wn;
  numerators(g, px, py, un, vn, wn);
  if (!numerators_pass(g, un, vn, wn)) return false;
  return solve_and_accept(un, vn, wn, g.dd, u, v, w);
}

// u * a + v * b + w * c, left to right (intersect_and_composite.slang:141-146).
__device__ __forceinline__ float interp(float u, float v, float w, float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(u, a), __fmul_rn(v, b)), __fmul_rn(w, c));
}

// acc + rgb * T * alpha (intersect_and_composite.slang:171-172).
__device__ __forceinline__ float over(float acc, float rgb, float T, float alpha) {
  return __fadd_rn(acc, __fmul_rn(__fmul_rn(rgb, T), alpha));
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

namespace mt {

// ---------------------------------------------------------------------------
// Warp-level culling.
//
// A pixel centre p can only be accepted by hit_test if none of the three
// numerators falls below the fast-reject threshold. For a well-conditioned
// triangle (every angle's sine^2 >= 1e-4, positive finite denominator above
// 2^-20, extent below 8192 px) the numerators are affine functions of p whose
// rounding error is bounded by a few ulps of |coefficients| x |p - p_i|;
// outside the triangle's bounding box grown by 1 px + 1e-3 x extent, one of
// them is negative by orders of magnitude more than that error, so
// hit_test's exact fast reject fires. Such a box is therefore a conservative
// superset of the accepted pixels, and a warp whose pixel rectangle misses it
// skips the triangle without changing any decision. Triangles that are not
// well-conditioned get an infinite box (never culled).
// ---------------------------------------------------------------------------
struct CullBox {
  float x0, x1, y0, y1;
};

__device__ __forceinline__ CullBox cull_box(const TriGeom& g, float p1x, float p1y, float p2x, float p2y, float p3x,
                                            float p3y) {
  const float inf = __int_as_float(0x7f800000);
  CullBox open{-inf, inf, -inf, inf};
  const float xmin = fminf(fminf(p1x, p2x), p3x), xmax = fmaxf(fmaxf(p1x, p2x), p3x);
  const float ymin = fminf(fminf(p1y, p2y), p3y), ymax = fmaxf(fmaxf(p1y, p2y), p3y);
  const float ext = fmaxf(xmax - xmin, ymax - ymin);
  if (!(ext < 8192.0f) || !(fabsf(xmin) < 1e6f && fabsf(xmax) < 1e6f && fabsf(ymin) < 1e6f && fabsf(ymax) < 1e6f))
    return open;
  if (!(g.thr > -inf)) return open;  // fast reject unavailable: no culling
  const float e23x = p3x - p2x, e23y = p3y - p2y;
  const float l12 = g.d1212, l13 = g.d1313, l23 = e23x * e23x + e23y * e23y;
  const float worst = fmaxf(fmaxf(l12 * l13, l12 * l23), l13 * l23);
  if (!(g.dd >= 1e-4f * worst)) return open;
  const float m = 1.0f + 1e-3f * ext;
  return CullBox{xmin - m, xmax + m, ymin - m, ymax + m};
}

__device__ __forceinline__ bool box_overlaps(const CullBox& b, float rx0, float rx1, float ry0, float ry1) {
  return !(b.x1 < rx0 || b.x0 > rx1 || b.y1 < ry0 || b.y0 > ry1);
}

// Pixel of thread `tid` inside its tile. When the tile is a whole number of
// 8x4 blocks each warp covers one 8x4 block (compact warp footprint, so a
// small triangle overlaps few warps); otherwise row-major.
__device__ __forceinline__ void tile_pixel(int tid, int tile_w, int tile_h, int& lx, int& ly) {
  if ((tile_w & 7) == 0 && (tile_h & 3) == 0) {
    const int warp = tid >> 5, lane = tid & 31;
    const int per_row = tile_w >> 3;
    lx = (warp % per_row) * 8 + (lane & 7);
    ly = (warp / per_row) * 4 + (lane >> 3);
  } else {
    lx = tid % tile_w;
    ly = tid / tile_w;
  }
}

// Bounding rectangle of the warp's pixel centres.
__device__ __forceinline__ void warp_rect(float fx, float fy, float& x0, float& x1, float& y0, float& y1) {
  x0 = x1 = fx;
  y0 = y1 = fy;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
  }
}

}  // namespace mt
