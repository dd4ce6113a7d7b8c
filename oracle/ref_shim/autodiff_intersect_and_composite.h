// Adjoints of the [Differentiable] helpers that the reference's hand-written
// fused backward kernel calls through bwd_diff(...) (slangtorch generates
// these by automatic differentiation; slangtorch is absent, so they are
// derived here by hand from the helpers' definitions).
//
// TEST INFRASTRUCTURE ONLY. oracle/build_ref.py includes this file into the
// rewritten intersect_and_composite source right before the backward kernel,
// inside the same namespace, so Vertex / Triangle / Sample / Accumulator and
// compute_barycentric_coordinates are the reference's own definitions.
//
// Conventions (Slang's): diffPair(x) starts with a zero differential; a
// bwd_diff call writes the input differentials of inout pairs; the backward of
// a DiffTensorView load adds into its gradient tensor (atomically), the
// backward of a store reads the gradient tensor. The clamp in compute_alpha
// passes its gradient strictly inside (0, 1). Arithmetic is single precision;
// the operation order of generated derivative code is not reproduced, so
// gradients agree to rounding, not bit for bit.
#pragma once

struct VertexDiff {
  float3 color{0.f, 0.f, 0.f};
  float signed_distance = 0.f;
};
struct TriangleDiff {
  VertexDiff a, b, c;
};
struct SampleDiff {
  float3 rgb{0.f, 0.f, 0.f};
  float sdf = 0.f;
  SampleDiff() = default;
  template <typename S>
  SampleDiff(const float3& r, S s) : rgb(r), sdf((float)s) {}
};
struct AccumulatorDiff {
  float3 rgb{0.f, 0.f, 0.f};
  float transmittance = 0.f;
};

struct SamplePair {
  Sample p;
  SampleDiff d;
};
struct TrianglePair {
  Triangle p;
  TriangleDiff d;
};
struct AccumulatorPair {
  Accumulator p;
  AccumulatorDiff d;
};
struct FloatPair {
  float p;
  float d;
};

inline SamplePair diffPair(const Sample& x) { return {x, SampleDiff{}}; }
inline TrianglePair diffPair(const Triangle& x) { return {x, TriangleDiff{}}; }
inline AccumulatorPair diffPair(const Accumulator& x) { return {x, AccumulatorDiff{}}; }
inline FloatPair diffPair(float x) { return {x, 0.f}; }

// store_accumulator: the four channels at the pixel are stored; their
// differentials are the gradient tensor's values there.
inline void bwd_diff_store_accumulator(AccumulatorPair& acc, const DiffTensorView& out, uint camera, uint2 xy) {
  const uint row = xy.y, col = xy.x;
  acc.d.rgb = float3(out.grad_at(camera, 0u, row, col), out.grad_at(camera, 1u, row, col),
                     out.grad_at(camera, 2u, row, col));
  acc.d.transmittance = out.grad_at(camera, 3u, row, col);
}

// c(x) = 1 / (1 + exp(-x s)) -> dc/dx = s e / (1 + e)^2, dc/ds = x e / (1 + e)^2.
inline void cdf_adjoint(float sdf, float s, float d_cdf, float& d_sdf, float& d_s) {
  const float e = std::exp(-sdf * s);
  const float q = 1.0f + e;
  const float dq = -d_cdf / (q * q);  // d(1/q)
  const float dy = dq * e;            // d exp(y), y = -sdf s
  d_sdf = dy * -s;
  d_s = dy * -sdf;
}

// compute_alpha = clamp(((oc - ic) + 1e-5) / (oc + 1e-5), 0, 1).
inline void bwd_diff_compute_alpha(SamplePair& inner, SamplePair& outer, FloatPair& sharpness, float d_alpha) {
  const float s = sharpness.p;
  const float ic = sdf_to_cdf(inner.p.sdf, s), oc = sdf_to_cdf(outer.p.sdf, s);
  const float num = oc - ic + 1e-5f, den = oc + 1e-5f;
  const float raw = num / den;
  const float d_raw = (raw > 0.f && raw < 1.f) ? d_alpha : 0.f;
  const float d_num = d_raw / den;
  const float d_den = -d_raw * num / (den * den);
  const float d_oc = d_num + d_den, d_ic = -d_num;
  float di_sdf, di_s, do_sdf, do_s;
  cdf_adjoint(inner.p.sdf, s, d_ic, di_sdf, di_s);
  cdf_adjoint(outer.p.sdf, s, d_oc, do_sdf, do_s);
  inner.d = SampleDiff(float3(0.f, 0.f, 0.f), di_sdf);
  outer.d = SampleDiff(float3(0.f, 0.f, 0.f), do_sdf);
  sharpness.d = di_s + do_s;
}

// sample_triangle: rgb / sdf are the barycentric mix of the vertices'; the
// positions are no_diff, so (u, v, w) carry no gradient. A skipped or missed
// triangle returns constants (zero gradient).
inline void bwd_diff_sample_triangle(TrianglePair& tri, float2 point, int last_shell, const SampleDiff& d) {
  tri.d = TriangleDiff{};
  if (tri.p.shell <= last_shell) return;
  const float3 uvw = compute_barycentric_coordinates(tri.p, point);
  const float sum = uvw.x + uvw.y + uvw.z;
  if (std::isnan(uvw.x) || std::isnan(uvw.y) || std::isnan(uvw.z) || uvw.x < 0 || uvw.x > 1 || uvw.y < 0 ||
      uvw.y > 1 || uvw.z < 0 || uvw.z > 1 || sum < 0.999f || sum > 1.001f)
    return;
  const float w[3] = {uvw.x, uvw.y, uvw.z};
  VertexDiff* out[3] = {&tri.d.a, &tri.d.b, &tri.d.c};
  for (int k = 0; k < 3; ++k) {
    out[k]->color = float3(w[k] * d.rgb.x, w[k] * d.rgb.y, w[k] * d.rgb.z);
    out[k]->signed_distance = w[k] * d.sdf;
  }
}

// load_triangle / load_vertex: colours and signed distances are loaded from
// DiffTensorViews at the face's vertices; their gradients are added there.
inline void bwd_diff_load_triangle(const TensorView<float>& vertices, const DiffTensorView& colors,
                                   const DiffTensorView& signed_distances, const TensorView<int>& faces, uint camera,
                                   uint shell, int face, const TriangleDiff& d) {
  (void)vertices;
  (void)shell;
  const VertexDiff* in[3] = {&d.a, &d.b, &d.c};
  for (uint k = 0; k < 3; ++k) {
    const uint v = (uint)faces[(uint)face, k];
    for (uint c = 0; c < 3; ++c) colors.grad_add(in[k]->color[c], camera, v, c);
    signed_distances.grad_add(in[k]->signed_distance, v);
  }
}

inline void bwd_diff_load_sharpness(const DiffTensorView& sharpness, float d) { sharpness.grad_add(d, 0u); }
