// Host-side stand-ins for the Slang language features used by the
// reference's compute kernels, so those kernel sources (after the textual
// rewrite in oracle/build_ref.py) compile as C++23 and run on the CPU.
//
// TEST INFRASTRUCTURE ONLY: used to pin the oracle against the reference's
// own kernel code. Semantics follow Slang's: 32-bit int/uint, float literals
// are float, vector types are component-wise, TensorView indexing is
// row-major over explicit sizes.
#pragma once

#include <algorithm>
#include <array>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

using uint = uint32_t;

// ---------------------------------------------------------------------------
// Vectors
// ---------------------------------------------------------------------------
template <typename T, int N>
struct vec;

template <typename T>
struct vec<T, 2> {
  union {
    struct { T x, y; };
    struct { T r, g; };
  };
  vec() = default;
  template <typename A, typename B>
  vec(A a, B b) : x((T)a), y((T)b) {}
  template <typename U>
  explicit vec(const vec<U, 2>& o) : x((T)o.x), y((T)o.y) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T>
struct vec<T, 3> {
  union {
    struct { T x, y, z; };
    struct { T r, g, b; };
    vec<T, 2> xy;  // swizzle .xy
  };
  vec() = default;
  template <typename A, typename B, typename C>
  vec(A a, B b, C c) : x((T)a), y((T)b), z((T)c) {}
  template <typename U>
  explicit vec(const vec<U, 3>& o) : x((T)o.x), y((T)o.y), z((T)o.z) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T>
struct vec<T, 4> {
  union {
    struct { T x, y, z, w; };
    struct { T r, g, b, a; };
    vec<T, 3> xyz;  // swizzle .xyz
    vec<T, 2> xy;   // swizzle .xy
  };
  vec() = default;
  template <typename A, typename B, typename C, typename D>
  vec(A a, B b, C c, D d) : x((T)a), y((T)b), z((T)c), w((T)d) {}
  template <typename U, typename D>
  vec(const vec<U, 3>& v, D d) : x((T)v.x), y((T)v.y), z((T)v.z), w((T)d) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

using uint2 = vec<uint, 2>;
using uint3 = vec<uint, 3>;
using uint4 = vec<uint, 4>;
using int2 = vec<int, 2>;
using int3 = vec<int, 3>;
using float2 = vec<float, 2>;
using float3 = vec<float, 3>;
using float4 = vec<float, 4>;
using uint64_t2 = vec<uint64_t, 2>;
using uint64_t3 = vec<uint64_t, 3>;
using uint64_t4 = vec<uint64_t, 4>;
using bool3 = vec<bool, 3>;

template <typename A, typename B>
using common_t = std::common_type_t<A, B>;

#define SLANG_VEC_BINOP(OP)                                                              \
  template <typename A, typename B, int N>                                               \
  vec<common_t<A, B>, N> operator OP(const vec<A, N>& a, const vec<B, N>& b) {           \
    vec<common_t<A, B>, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = (common_t<A, B>)a[i] OP(common_t<A, B>) b[i];     \
    return r;                                                                            \
  }                                                                                      \
  template <typename A, typename B, int N, typename = std::enable_if_t<std::is_arithmetic_v<B>>> \
  vec<common_t<A, B>, N> operator OP(const vec<A, N>& a, B b) {                          \
    vec<common_t<A, B>, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = (common_t<A, B>)a[i] OP(common_t<A, B>) b;        \
    return r;                                                                            \
  }                                                                                      \
  template <typename A, typename B, int N, typename = std::enable_if_t<std::is_arithmetic_v<A>>> \
  vec<common_t<A, B>, N> operator OP(A a, const vec<B, N>& b) {                          \
    vec<common_t<A, B>, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = (common_t<A, B>)a OP(common_t<A, B>) b[i];        \
    return r;                                                                            \
  }

SLANG_VEC_BINOP(+)
SLANG_VEC_BINOP(-)
SLANG_VEC_BINOP(*)
SLANG_VEC_BINOP(/)
SLANG_VEC_BINOP(%)

template <typename A, int N>
vec<A, N> operator-(const vec<A, N>& a) {
  vec<A, N> r;
  for (int i = 0; i < N; ++i) r[i] = -a[i];
  return r;
}

template <typename A, typename B, int N>
vec<A, N>& operator+=(vec<A, N>& a, const vec<B, N>& b) {
  for (int i = 0; i < N; ++i) a[i] = a[i] + b[i];
  return a;
}

template <typename A, typename B, int N>
vec<bool, N> operator!=(const vec<A, N>& a, const vec<B, N>& b) {
  vec<bool, N> r;
  for (int i = 0; i < N; ++i) r[i] = a[i] != b[i];
  return r;
}

template <int N>
bool any(const vec<bool, N>& v) {
  for (int i = 0; i < N; ++i)
    if (v[i]) return true;
  return false;
}

// ---------------------------------------------------------------------------
// Matrices (row-major, as Slang's floatRxC constructors)
// ---------------------------------------------------------------------------
template <int R, int C>
struct mat {
  float m[R][C];
  template <typename... V>
  mat(V... values) {
    const float f[] = {(float)values...};
    static_assert(sizeof...(V) == R * C, "matrix constructor takes R*C scalars");
    for (int i = 0; i < R * C; ++i) m[i / C][i % C] = f[i];
  }
};
using float4x4 = mat<4, 4>;
using float3x3 = mat<3, 3>;

template <int R, int C>
vec<float, R> mul(const mat<R, C>& a, const vec<float, C>& v) {
  vec<float, R> r;
  for (int i = 0; i < R; ++i) {
    float s = a.m[i][0] * v[0];
    for (int j = 1; j < C; ++j) s = s + a.m[i][j] * v[j];
    r[i] = s;
  }
  return r;
}

// ---------------------------------------------------------------------------
// Scalar and vector intrinsics
// ---------------------------------------------------------------------------
template <typename A, typename B>
common_t<A, B> min(A a, B b) {
  using T = common_t<A, B>;
  return std::min((T)a, (T)b);
}
template <typename A, typename B>
common_t<A, B> max(A a, B b) {
  using T = common_t<A, B>;
  return std::max((T)a, (T)b);
}
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
template <typename A, typename B, int N, typename = std::enable_if_t<std::is_arithmetic_v<B>>>
vec<A, N> max(const vec<A, N>& a, B b) {
  vec<A, N> r;
  for (int i = 0; i < N; ++i) r[i] = max(a[i], (A)b);
  return r;
}
template <typename X, typename L, typename H>
auto clamp(X x, L lo, H hi) {
  using T = common_t<X, common_t<L, H>>;
  return min(max((T)x, (T)lo), (T)hi);
}
inline float abs(float x) { return std::fabs(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float exp(float x) { return std::exp(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline bool isnan(float x) { return std::isnan(x); }
template <typename T, int N>
T dot(const vec<T, N>& a, const vec<T, N>& b) {
  T s = a[0] * b[0];
  for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
  return s;
}
template <int N>
vec<float, N> normalize(const vec<float, N>& v) {
  return v / std::sqrt(dot(v, v));
}
inline int countbits(uint x) { return __builtin_popcount(x); }
inline int countbits(int x) { return __builtin_popcount((uint)x); }
template <typename To, typename From>
To reinterpret(From x) {
  static_assert(sizeof(To) == sizeof(From), "reinterpret needs equal sizes");
  To t;
  std::memcpy(&t, &x, sizeof(To));
  return t;
}
template <typename T>
T detach(T x) {
  return x;
}

// ---------------------------------------------------------------------------
// Tensor views
// ---------------------------------------------------------------------------
template <typename T>
struct TensorView {
  T* ptr = nullptr;
  int ndim = 0;
  uint64_t sizes[6] = {};

  TensorView() = default;
  TensorView(T* p, std::initializer_list<uint64_t> shape) : ptr(p), ndim((int)shape.size()) {
    int i = 0;
    for (uint64_t s : shape) sizes[i++] = s;
  }
  uint size(int i) const { return (uint)sizes[i]; }
  T* data_ptr() const { return ptr; }
  template <typename I, typename = std::enable_if_t<std::is_integral_v<I>>>
  T* data_ptr_at(I i) const {
    return ptr + (int64_t)i;
  }

  template <typename... I>
  uint64_t offset(I... idx) const {
    const uint64_t v[] = {(uint64_t)idx...};
    uint64_t o = 0;
    for (int i = 0; i < (int)sizeof...(I); ++i) o = o * sizes[i] + v[i];
    return o;
  }
  template <typename U, int N>
  uint64_t offset_v(const vec<U, N>& idx) const {
    uint64_t o = 0;
    for (int i = 0; i < N; ++i) o = o * sizes[i] + (uint64_t)idx[i];
    return o;
  }
  template <typename... I>
  T& operator[](I... idx) const
    requires(sizeof...(I) > 1 || (std::is_integral_v<I> && ...))
  {
    return ptr[offset(idx...)];
  }
  template <typename U, int N>
  T& operator[](const vec<U, N>& idx) const {
    return ptr[offset_v(idx)];
  }
  template <typename U, int N>
  void storeOnce(const vec<U, N>& idx, T value) const {
    ptr[offset_v(idx)] = value;
  }
  template <typename U, typename = std::enable_if_t<std::is_integral_v<U>>>
  void storeOnce(U idx, T value) const {
    ptr[(uint64_t)idx] = value;
  }
};
// A float tensor with an optional gradient tensor of the same shape, as
// slangtorch passes (primal, gradient) pairs. Backward kernels read the
// gradient of stored outputs and add into the gradient of loaded inputs.
struct DiffTensorView : TensorView<float> {
  float* grad = nullptr;
  DiffTensorView() = default;
  DiffTensorView(const TensorView<float>& t, float* g = nullptr) : TensorView<float>(t), grad(g) {}
  template <typename... I>
  float grad_at(I... idx) const {
    return grad ? grad[offset(idx...)] : 0.f;
  }
  template <typename... I>
  void grad_add(float value, I... idx) const {
    if (grad) std::atomic_ref<float>(grad[offset(idx...)]).fetch_add(value, std::memory_order_relaxed);
  }
};

// The reference's 64-bit indexing helpers (common.slang), by semantics.
template <typename T, typename U, int N>
T load(const TensorView<T>& x, const vec<U, N>& idx) {
  return x[idx];
}
template <typename T, typename I, typename = std::enable_if_t<std::is_integral_v<I>>>
T load(const TensorView<T>& x, I idx) {
  return x.ptr[(uint64_t)idx];
}
template <typename T, typename U, int N, typename V>
T store(const TensorView<T>& x, const vec<U, N>& idx, V value) {
  x[idx] = (T)value;
  return (T)value;
}
template <typename T, typename I, typename V, typename = std::enable_if_t<std::is_integral_v<I>>>
T store(const TensorView<T>& x, I idx, V value) {
  x.ptr[(uint64_t)idx] = (T)value;
  return (T)value;
}
template <typename U, int N>
void store_once(const DiffTensorView& x, const vec<U, N>& idx, float value) {
  x[idx] = value;
}

// Atomics (emulated blocks run in parallel threads).
enum class MemoryOrder { Relaxed };
inline int slang_atomic_or(int& target, int value, MemoryOrder) {
  return std::atomic_ref<int>(target).fetch_or(value, std::memory_order_relaxed);
}

// ---------------------------------------------------------------------------
// Launch state: the driver sets these per emulated thread.
// ---------------------------------------------------------------------------
inline thread_local uint3 g_block_idx, g_block_dim, g_thread_idx;
inline thread_local std::barrier<>* g_block_barrier = nullptr;

inline uint3 cudaBlockIdx() { return g_block_idx; }
inline uint3 cudaBlockDim() { return g_block_dim; }
inline uint3 cudaThreadIdx() { return g_thread_idx; }
inline void AllMemoryBarrierWithGroupSync() {
  if (g_block_barrier) g_block_barrier->arrive_and_wait();
}
