// Adjoints of the [Differentiable] helpers that the reference's hand-written
// explicit-mode composite backward kernel calls through bwd_diff(...),
// derived by hand (slangtorch, which would generate them, is absent).
//
// TEST INFRASTRUCTURE ONLY. oracle/build_ref.py includes this file into the
// rewritten composite source right before the backward kernel, inside the same
// namespace. Conventions as for the fused kernel's adjoints: diffPair(x)
// starts with a zero differential, a load's backward adds into the
// DiffTensorView's gradient (atomically), a store's backward reads it, and the
// clamp passes its gradient strictly inside (0, 1).
#pragma once

struct FloatPair {
  float p;
  float d;
};
struct Float3Pair {
  float3 p;
  float3 d;
};

inline FloatPair diffPair(float x) { return {x, 0.f}; }
inline Float3Pair diffPair(const float3& x) { return {x, float3(0.f, 0.f, 0.f)}; }

inline void bwd_diff_store_result(const DiffTensorView& out_colors, const DiffTensorView& out_transmittances,
                                  Float3Pair& color, FloatPair& transmittance, int pixel) {
  const uint p = (uint)pixel;
  color.d = float3(out_colors.grad_at(p, 0u), out_colors.grad_at(p, 1u), out_colors.grad_at(p, 2u));
  transmittance.d = out_transmittances.grad_at(p);
}

inline void cdf_adjoint(float sdf, float s, float d_cdf, float& d_sdf, float& d_s) {
  const float e = std::exp(-sdf * s);
  const float q = 1.0f + e;
  const float dq = -d_cdf / (q * q);
  const float dy = dq * e;
  d_sdf = dy * -s;
  d_s = dy * -sdf;
}

inline void bwd_diff_compute_alpha(FloatPair& inner_sdf, FloatPair& outer_sdf, FloatPair& sharpness, float d_alpha) {
  const float s = sharpness.p;
  const float ic = sdf_to_cdf(inner_sdf.p, s), oc = sdf_to_cdf(outer_sdf.p, s);
  const float num = oc - ic + 1e-5f, den = oc + 1e-5f;
  const float raw = num / den;
  const float d_raw = (raw > 0.f && raw < 1.f) ? d_alpha : 0.f;
  const float d_num = d_raw / den;
  const float d_den = -d_raw * num / (den * den);
  float di_s, do_s;
  cdf_adjoint(inner_sdf.p, s, -d_num, inner_sdf.d, di_s);
  cdf_adjoint(outer_sdf.p, s, d_num + d_den, outer_sdf.d, do_s);
  sharpness.d = di_s + do_s;
}

inline void bwd_diff_load_color(const DiffTensorView& colors, int pixel, int shell, const float3& d) {
  for (uint c = 0; c < 3; ++c) colors.grad_add(d[c], (uint)pixel, (uint)shell, c);
}

inline void bwd_diff_load_sdf(const DiffTensorView& signed_distances, int pixel, int shell, float d) {
  signed_distances.grad_add(d, (uint)pixel, (uint)shell);
}

inline void bwd_diff_load_sharpness(const DiffTensorView& sharpness, float d) { sharpness.grad_add(d, 0u); }
